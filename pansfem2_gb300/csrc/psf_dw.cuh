// psf_dw.cuh -- double-word ("double-single") arithmetic on FP32 pairs.
//
// GB300's FP64 pipe issues about 2 FMAs per clock per SM, against 128 FP32 lanes, so
// element-wise FP64 work with many divisions runs far below the memory roofline.  A
// double-word number x = h + l (|l| <= ulp(h)/2, both floats) carries about 48 bits of
// significand.  The operations below are the published algorithms, built on the
// error-free transformations TwoSum (Knuth), Fast2Sum (Dekker) and TwoProd with an FMA:
//   add   AccurateDWPlusDW   (Joldes, Muller, Popescu, ACM TOMS 44(2), 2017, Alg. 6)
//   mul   DWTimesDW3         (same paper, Alg. 12)
//   mulf  DWTimesFP3         (same paper, Alg. 9)
//   rcp   one Newton step x1 = x0 + x0 (1 - y x0) from the correctly rounded FP32
//         reciprocal x0, with the residual 1 - y x0 formed exactly by TwoProd
// Relative errors are a few units of 2^-48, far inside what the interior-point loops
// that use them need (their stopping tolerance is 1e-7).  The FP32 exponent range
// applies: callers check that their data lie within it.
#pragma once

#include <cuda_runtime.h>

#include <cmath>

#ifdef __CUDACC__
#include "psf_common.cuh"
#endif

// Every operation is also compiled for the host (tests/cpp/dw_check.cu checks them there):
// single-rounding float add / mul / fma on both sides, no contraction.
#ifdef __CUDA_ARCH__
#define PSF_DW_ADD(a, b) __fadd_rn(a, b)
#define PSF_DW_SUB(a, b) __fsub_rn(a, b)
#define PSF_DW_MUL(a, b) __fmul_rn(a, b)
#define PSF_DW_FMA(a, b, c) __fmaf_rn(a, b, c)
#define PSF_DW_RCP(a) __frcp_rn(a)
#define PSF_DW_F2D(v) __double2float_rn(v)
#else
#define PSF_DW_ADD(a, b) psf::dw::h_add(a, b)
#define PSF_DW_SUB(a, b) psf::dw::h_sub(a, b)
#define PSF_DW_MUL(a, b) psf::dw::h_mul(a, b)
#define PSF_DW_FMA(a, b, c) std::fma(a, b, c)
#define PSF_DW_RCP(a) (1.0f / (a))
#define PSF_DW_F2D(v) ((float)(v))
#endif

namespace psf {
namespace dw {

#ifndef __CUDA_ARCH__
// volatile stores keep the host compiler from fusing or reassociating
inline float h_add(float a, float b) { volatile float r = a + b; return r; }
inline float h_sub(float a, float b) { volatile float r = a - b; return r; }
inline float h_mul(float a, float b) { volatile float r = a * b; return r; }
#endif

struct D {
    float h, l;
};

__host__ __device__ __forceinline__ float two_sum(float a, float b, float &e) {
    const float s = PSF_DW_ADD(a, b);
    const float bb = PSF_DW_SUB(s, a);
    e = PSF_DW_ADD(PSF_DW_SUB(a, PSF_DW_SUB(s, bb)), PSF_DW_SUB(b, bb));
    return s;
}
__host__ __device__ __forceinline__ float fast_two_sum(float a, float b, float &e) {   // |a| >= |b|
    const float s = PSF_DW_ADD(a, b);
    e = PSF_DW_SUB(b, PSF_DW_SUB(s, a));
    return s;
}
__host__ __device__ __forceinline__ float two_prod(float a, float b, float &e) {
    const float p = PSF_DW_MUL(a, b);
    e = PSF_DW_FMA(a, b, -p);
    return p;
}

__host__ __device__ __forceinline__ D make(float h, float l) { return D{h, l}; }
__host__ __device__ __forceinline__ D from_float(float v) { return D{v, 0.0f}; }
__host__ __device__ __forceinline__ D from_double(double v) {
    const float h = PSF_DW_F2D(v);
    return D{h, PSF_DW_F2D(v - (double)h)};
}
__host__ __device__ __forceinline__ double to_double(D a) { return (double)a.h + (double)a.l; }
__host__ __device__ __forceinline__ D neg(D a) { return D{-a.h, -a.l}; }
__host__ __device__ __forceinline__ D scale2(D a, float p2) { return D{a.h * p2, a.l * p2}; }   // p2 a power of 2

__host__ __device__ __forceinline__ D add(D x, D y) {
    float sl, tl, vl, zl;
    const float sh = two_sum(x.h, y.h, sl);
    const float th = two_sum(x.l, y.l, tl);
    const float c = PSF_DW_ADD(sl, th);
    const float vh = fast_two_sum(sh, c, vl);
    const float w = PSF_DW_ADD(tl, vl);
    const float zh = fast_two_sum(vh, w, zl);
    return D{zh, zl};
}
__host__ __device__ __forceinline__ D sub(D x, D y) { return add(x, neg(y)); }

__host__ __device__ __forceinline__ D mul(D x, D y) {
    float cl1, zl;
    const float ch = two_prod(x.h, y.h, cl1);
    const float tl0 = PSF_DW_MUL(x.l, y.l);
    const float tl1 = PSF_DW_FMA(x.h, y.l, tl0);
    const float cl2 = PSF_DW_FMA(x.l, y.h, tl1);
    const float cl3 = PSF_DW_ADD(cl1, cl2);
    const float zh = fast_two_sum(ch, cl3, zl);
    return D{zh, zl};
}
__host__ __device__ __forceinline__ D mulf(D x, float y) {
    float cl1, zl;
    const float ch = two_prod(x.h, y, cl1);
    const float cl3 = PSF_DW_FMA(x.l, y, cl1);
    const float zh = fast_two_sum(ch, cl3, zl);
    return D{zh, zl};
}
__host__ __device__ __forceinline__ D sq(D x) { return mul(x, x); }

__host__ __device__ __forceinline__ D rcp(D y) {
    const float x0 = PSF_DW_RCP(y.h);
    float pl;
    const float ph = two_prod(y.h, x0, pl);                          // y.h x0 = ph + pl exactly
    const float e = PSF_DW_FMA(-y.l, x0, PSF_DW_SUB(PSF_DW_SUB(1.0f, ph), pl));   // 1 - y x0
    float zl;
    const float zh = fast_two_sum(x0, PSF_DW_MUL(x0, e), zl);
    return D{zh, zl};
}
__host__ __device__ __forceinline__ D div(D x, D y) { return mul(x, rcp(y)); }

// ordering of normalised pairs
__host__ __device__ __forceinline__ bool lt(D a, D b) { return a.h < b.h || (a.h == b.h && a.l < b.l); }
__host__ __device__ __forceinline__ D max(D a, D b) { return lt(a, b) ? b : a; }   // std::max: first on ties
__host__ __device__ __forceinline__ D min(D a, D b) { return lt(b, a) ? b : a; }   // std::min: first on ties

__host__ __device__ __forceinline__ D ld(const float2 *p, long long i) {
    const float2 v = p[i];
    return D{v.x, v.y};
}
__host__ __device__ __forceinline__ void st(float2 *p, long long i, D v) { p[i] = make_float2(v.h, v.l); }

#ifdef __CUDACC__
// Block sums of NV double-word values: the warp levels in double words (FP32 pipes),
// then the per-warp results in FP64 by warp 0, in a fixed order.  Result in thread 0.
// (A warp tree in FP64 costs every lane five FP64 adds per value, which on GB300's
// FP64 pipe rivals the element work.)
template <int NV>
__device__ __forceinline__ void block_sum_dw(D (&v)[NV], double (&out)[NV], double *smem) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
    for (int k = 0; k < NV; k++) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const D t = make(__shfl_xor_sync(0xffffffffu, v[k].h, o), __shfl_xor_sync(0xffffffffu, v[k].l, o));
            v[k] = add(v[k], t);
        }
    }
    __syncthreads();
    if (lane == 0) {
#pragma unroll
        for (int k = 0; k < NV; k++) smem[k * 32 + wid] = to_double(v[k]);
    }
    __syncthreads();
    if (wid == 0) {
#pragma unroll
        for (int k = 0; k < NV; k++) out[k] = warp_sum(lane < nw ? smem[k * 32 + lane] : 0.0);
    }
}

// block maximum of double-word values, as a double in thread 0
__device__ __forceinline__ double block_max_dw(D v, double *smem) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const D t = make(__shfl_xor_sync(0xffffffffu, v.h, o), __shfl_xor_sync(0xffffffffu, v.l, o));
        v = max(v, t);
    }
    __syncthreads();
    if (lane == 0) smem[wid] = to_double(v);
    __syncthreads();
    double m = -INFINITY;
    if (wid == 0) m = warp_max(lane < nw ? smem[lane] : -INFINITY);
    return m;
}

#endif

}  // namespace dw
}  // namespace psf
