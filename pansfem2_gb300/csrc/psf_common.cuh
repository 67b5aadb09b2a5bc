// psf_common.cuh -- shared device/host pieces of the GB300 SIMP library.
//
// Persistent kernels synchronise their blocks with grid_sync(), a barrier on
// global-memory atomics whose wait is bounded: after kSpinLimit polls it sets
// PSF_TIMEOUT in the status word and every block returns, so a wait can never
// hang the GPU.  A barrier can fold per-block partial sums: every block writes
// its partials, arrives, waits for all arrivals, and then reduces all blocks'
// partials itself in one fixed order, so every block holds the same,
// deterministic sums without a second round through one releasing block.
// These kernels are launched with cudaLaunchCooperativeKernel, which
// guarantees that all blocks are resident.
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


constexpr int kMaxRed = 20;                   // values reduced by one grid_sync (the m = 4 MMA needs 19)
constexpr long long kSpinLimit = 1ll << 23;   // polls (x >= 64 ns each): ~1 s bound
// partial sums a grid_sync needs: two alternating sets (the phase parity) of kMaxRed + 1
// values per block, so a block that has left a barrier never overwrites the partials a
// slower block is still reading
constexpr int kPartialSlots = 2 * (kMaxRed + 1);

// the barrier's global state (reset to zero before every launch)
struct GridSync {
    unsigned int count;       // arrivals since the launch (phase p completes at count = (p + 1) * blocks)
    unsigned int gen;         // unused
    int status;               // psf_status set by a device-side failure
    int pad;
    double result[kMaxRed];   // unused
    double result_max;        // unused
};

// per-block barrier state: the block's phase and the reduced values of its last grid_sync
struct GridBlockState {
    unsigned int phase;
    int ok;
    double res[kMaxRed + 1];
};
static __shared__ GridBlockState s_grid;

// every kernel that calls grid_sync calls this first (all threads)
__device__ __forceinline__ void grid_sync_init() {
    if (threadIdx.x == 0) s_grid.phase = 0;
    __syncthreads();
}

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
// The same sums with about a fifth of the FP64 additions (the FP64 pipe is narrow on GB300):
// every thread stores its values, then warp 0 adds the block's values per lane in four fixed
// chains and finishes with one shuffle tree.  smem holds NV * blockDim.x doubles (blockDim.x a
// multiple of 32); the results are in warp 0.
template <int NV>
__device__ __forceinline__ void block_sum_wide(double (&v)[NV], double *smem) {
    const int t = threadIdx.x, nt = blockDim.x, lane = t & 31, nw = nt >> 5;
    __syncthreads();   // the previous use of smem is over
#pragma unroll
    for (int k = 0; k < NV; k++) smem[k * nt + t] = v[k];
    __syncthreads();
    if (t < 32) {
#pragma unroll
        for (int k = 0; k < NV; k++) {
            const double *s = smem + k * nt + lane;
            double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
            int w = 0;
            for (; w + 4 <= nw; w += 4) {
                a0 += s[32 * w];
                a1 += s[32 * (w + 1)];
                a2 += s[32 * (w + 2)];
                a3 += s[32 * (w + 3)];
            }
            for (; w < nw; w++) a0 += s[32 * w];
            v[k] = warp_sum((a0 + a1) + (a2 + a3));
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
__device__ __forceinline__ void red_release_add(unsigned int *p, unsigned int v) {
    asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ int ld_volatile_int(const int *p) {
    return *(const volatile int *)p;
}

// Grid-wide barrier with a fused reduction.
//   partials: kPartialSlots * gridDim.x doubles; this block's values in v[] (thread 0)
//   and pmax (thread 0) for an optional max over blocks (NMAX = 0 or 1).
// On return every thread of every block sees gs_result(gs, 0..NV) and
// gs_result_max(gs), the same values in every block (partials summed in block
// order by one warp per block: lane l adds blocks l, l + 32, ... in order, then
// an xor butterfly).  Returns false if any block recorded a failure; callers
// then return at once.
template <int NV, int NMAX>
__device__ bool grid_sync(GridSync *gs, double *partials, const double (&v)[NV > 0 ? NV : 1],
                          double pmax, long long spin_limit = kSpinLimit) {
    const unsigned int nb = gridDim.x;
    __syncthreads();   // thread 0 holds the block's values; every thread has read the last results
    if (threadIdx.x == 0) {
        const unsigned int ph = s_grid.phase;
        double *slot = partials + (size_t)(ph & 1u) * (kMaxRed + 1) * nb;
#pragma unroll
        for (int k = 0; k < NV; k++) slot[(size_t)k * nb + blockIdx.x] = v[k];
        if (NMAX) slot[(size_t)NV * nb + blockIdx.x] = pmax;
        red_release_add(&gs->count, 1u);   // arrival, ordered after the partial stores
        const unsigned int target = (ph + 1u) * nb;
        long long spins = 0;
        int ok = 1;
        for (;;) {
            const unsigned int c = ld_acquire(&gs->count);
            const int st = ld_volatile_int(&gs->status);
            if (st != 0) { ok = 0; break; }
            if (c >= target) break;
            if (spins > 256) __nanosleep(32);   // tight polling first, then back off
            if (++spins > spin_limit) {
                atomicCAS(&gs->status, 0, (int)PSF_TIMEOUT);
                ok = 0;
                break;
            }
        }
        s_grid.ok = ok;
        s_grid.phase = ph + 1u;
    }
    __syncthreads();
    if (!s_grid.ok) return false;
    if (NV + NMAX > 0) {
        if (threadIdx.x < 32) {
            const int lane = threadIdx.x;
            const double *slot = partials + (size_t)((s_grid.phase - 1u) & 1u) * (kMaxRed + 1) * nb;
            if (NV > 0) {
                // every lane adds its blocks in ascending order for each value; the loads of
                // several blocks and values are in flight together
                double acc[NV > 0 ? NV : 1];
#pragma unroll
                for (int k = 0; k < NV; k++) acc[k] = 0.0;
#pragma unroll 4
                for (unsigned int b = lane; b < nb; b += 32) {
#pragma unroll
                    for (int k = 0; k < NV; k++) acc[k] += __ldcg(slot + (size_t)k * nb + b);
                }
#pragma unroll
                for (int k = 0; k < NV; k++) {
                    double a = acc[k];
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
                    if (lane == 0) s_grid.res[k] = a;
                }
            }
            if (NMAX) {
                double m = -INFINITY;
                for (unsigned int b = lane; b < nb; b += 32) m = fmax(m, __ldcg(slot + (size_t)NV * nb + b));
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
                if (lane == 0) s_grid.res[kMaxRed] = m;
            }
        }
        __syncthreads();
    }
    return true;
}

// reduced values of this block's last grid_sync
__device__ __forceinline__ double gs_result(const GridSync *, int k) { return s_grid.res[k]; }
__device__ __forceinline__ double gs_result_max(const GridSync *) { return s_grid.res[kMaxRed]; }

// plain barrier (no reduction)
__device__ __forceinline__ bool grid_barrier(GridSync *gs, double *partials) {
    double v[1] = {0.0};
    return grid_sync<0, 0>(gs, partials, v, 0.0);
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
