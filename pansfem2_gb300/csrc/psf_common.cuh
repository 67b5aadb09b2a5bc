// psf_common.cuh -- shared device/host pieces of the GB300 SIMP library.
//
// Persistent kernels synchronise their blocks with grid_sync(), a barrier on
// global-memory atomics whose wait is bounded: after kSpinLimit polls it sets
// PSF_TIMEOUT in the status word and every block returns, so a wait can never
// hang the GPU.  The last block to arrive also folds the per-block partial
// sums of the phase (fixed order: deterministic) before it releases the
// others, so a reduction costs one barrier.  These kernels are launched with
// cudaLaunchCooperativeKernel, which guarantees that all blocks are resident.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "pansfem2_gpu.h"

namespace psf {

// Kernel launches made by this host thread.  Every launch site calls note_launch (a graph
// replay adds its kernel nodes); the iteration and assembly reports give the difference
// over their calls.
inline thread_local long long g_launches = 0;
inline void note_launch(long long n = 1) { g_launches += n; }
inline long long launches() { return g_launches; }


constexpr int kMaxRed = 6;                    // values reduced by one grid_sync
constexpr long long kSpinLimit = 1ll << 23;   // polls (x >= 64 ns each): ~1 s bound

// one slot of per-block partials for up to kMaxRed sums (and one max)
struct GridSync {
    unsigned int count;       // arrivals in the current phase
    unsigned int gen;         // phase generation (release flag)
    int status;               // psf_status set by a device-side failure
    int pad;
    double result[kMaxRed];   // reduced values of the last phase
    double result_max;
};

// explicit single-rounding a*b + c, so that values recomputed in two places agree bit for bit
__device__ __forceinline__ float fma_t(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double fma_t(double a, double b, double c) { return __fma_rn(a, b, c); }

// ------------------------------------------------------------------ warp/block reductions
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// Block-wide sum of NV values per thread; result valid in thread 0.  smem needs
// 32*NV doubles.  Fixed tree order: deterministic for a fixed launch shape.
template <int NV>
__device__ __forceinline__ void block_sum(double (&v)[NV], double *smem) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
    for (int k = 0; k < NV; k++) v[k] = warp_sum(v[k]);
    __syncthreads();
    if (lane == 0) {
#pragma unroll
        for (int k = 0; k < NV; k++) smem[k * 32 + wid] = v[k];
    }
    __syncthreads();
    if (wid == 0) {
#pragma unroll
        for (int k = 0; k < NV; k++) {
            double t = lane < nw ? smem[k * 32 + lane] : 0.0;
            v[k] = warp_sum(t);
        }
    }
}
__device__ __forceinline__ double block_max(double v, double *smem) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    v = warp_max(v);
    __syncthreads();
    if (lane == 0) smem[wid] = v;
    __syncthreads();
    if (wid == 0) v = warp_max(lane < nw ? smem[lane] : -INFINITY);
    return v;
}

__device__ __forceinline__ unsigned int ld_acquire(const unsigned int *p) {
    unsigned int v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ int ld_volatile_int(const int *p) {
    return *(const volatile int *)p;
}

// Grid-wide barrier with a fused reduction.
//   partials: [NV][gridDim.x] doubles; this block's values in v[] (thread 0)
//   and pmax (thread 0) for an optional max over blocks (NMAX = 0 or 1).
// On return every thread of every block sees gs->result[0..NV) and
// gs->result_max.  Returns false if any block recorded a failure; callers
// then return at once.
template <int NV, int NMAX>
__device__ bool grid_sync(GridSync *gs, double *partials, const double (&v)[NV > 0 ? NV : 1],
                          double pmax) {
    __shared__ int s_last;
    __shared__ unsigned int s_gen;
    __shared__ int s_ok;
    __shared__ double s_red[32 * (NV > 0 ? NV : 1)];
    const unsigned int nb = gridDim.x;
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < NV; k++) partials[(size_t)k * nb + blockIdx.x] = v[k];
        if (NMAX) partials[(size_t)NV * nb + blockIdx.x] = pmax;
        unsigned int g = ld_acquire(&gs->gen);
        __threadfence();
        unsigned int arrived = atomicAdd(&gs->count, 1u);
        s_last = (arrived == nb - 1);
        s_gen = g;
    }
    __syncthreads();
    if (s_last) {
        // last block: every thread loads a strided share of the partials (one
        // L2 round trip instead of nb/32 dependent ones), fixed-order tree sum,
        // publish, release
        __threadfence();
        if (NV > 0) {
            double acc[NV > 0 ? NV : 1];
#pragma unroll
            for (int k = 0; k < NV; k++) {
                acc[k] = 0.0;
                for (unsigned int b = threadIdx.x; b < nb; b += blockDim.x)
                    acc[k] += __ldcg(&partials[(size_t)k * nb + b]);
            }
            block_sum<(NV > 0 ? NV : 1)>(acc, s_red);
            if (threadIdx.x == 0) {
#pragma unroll
                for (int k = 0; k < NV; k++) gs->result[k] = acc[k];
            }
        }
        if (NMAX) {
            double m = -INFINITY;
            for (unsigned int b = threadIdx.x; b < nb; b += blockDim.x)
                m = fmax(m, __ldcg(&partials[(size_t)NV * nb + b]));
            m = block_max(m, s_red);
            if (threadIdx.x == 0) gs->result_max = m;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            gs->count = 0;
            __threadfence();
            atomicAdd(&gs->gen, 1u);
            s_ok = 1;
        }
    } else if (threadIdx.x == 0) {
        const unsigned int g = s_gen;
        long long spins = 0;
        int ok = 1;
        while (ld_acquire(&gs->gen) == g) {
            if (spins > 256) __nanosleep(32);   // tight polling first, then back off
            if (++spins > kSpinLimit || ld_volatile_int(&gs->status) != 0) {
                atomicCAS(&gs->status, 0, (int)PSF_TIMEOUT);
                ok = 0;
                break;
            }
        }
        __threadfence();
        s_ok = ok;
    }
    __syncthreads();
    return s_ok && ld_volatile_int(&gs->status) == 0;
}

// ------------------------------------------------------------------ canonical sums
// A sum over n terms whose rounding does not depend on the launch shape: the terms are cut
// into chunks of kChunk consecutive indices; a chunk's sum is formed by one warp (lane l adds
// terms l, l+32, ... of the chunk in order, then an xor butterfly, which leaves the same value
// in every lane because each pairwise addition is commutative), and the chunk sums are added
// by one warp in the same way.  Kernels with different grids, block sizes or thread-block
// clusters (the single-problem and the batched OC bisection) therefore agree bit for bit.
constexpr int kChunk = 256;
__device__ __forceinline__ double warp_xor_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
// sum of nv values v[0..nv) by one warp (all lanes return it)
__device__ __forceinline__ double warp_canonical_sum(const double *v, long long nv) {
    const int lane = threadIdx.x & 31;
    double acc = 0.0;
    for (long long t = lane; t < nv; t += 32) acc += __ldcg(v + t);
    return warp_xor_sum(acc);
}

// reduced values of the last grid_sync, read past L1 (the slot is rewritten every phase)
__device__ __forceinline__ double gs_result(const GridSync *gs, int k) { return __ldcg(&gs->result[k]); }
__device__ __forceinline__ double gs_result_max(const GridSync *gs) { return __ldcg(&gs->result_max); }

// plain barrier (no reduction)
__device__ __forceinline__ bool grid_barrier(GridSync *gs, double *partials) {
    double v[1] = {0.0};
    return grid_sync<0, 0>(gs, partials, v, 0.0);
}

}  // namespace psf

// ------------------------------------------------------------------ host helpers
namespace psf {
void set_error(const std::string &msg);
const char *last_error();
psf_status cuda_status(cudaError_t e, const char *what);
}  // namespace psf

#define PSF_CUDA(call)                                                                  \
    do {                                                                                \
        cudaError_t e_ = (call);                                                        \
        if (e_ != cudaSuccess) return psf::cuda_status(e_, #call);                      \
    } while (0)

#define PSF_CHECK(expr)                                                                 \
    do {                                                                                \
        psf_status s_ = (expr);                                                         \
        if (s_ != PSF_OK) return s_;                                                    \
    } while (0)
