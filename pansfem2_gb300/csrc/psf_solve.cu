// psf_solve.cu -- matrix-free K.u and the Krylov solvers.
//
// Matrix-free operator: y = sum_e E_e P_e^T Ke0 P_e u over the structured grid,
// one thread per node gathering its 2^d surrounding elements (no atomics, no
// element list).  Ke0 travels as a kernel parameter (constant bank): every
// lane of a warp reads the same entry at the same time.  Fixed dofs hold zero
// in every vector and their rows of y are zero, which is K restricted to the
// free dofs in the nodal layout.
//
// Solvers run as persistent cooperative kernels: one launch per solve, two
// fused reduce-barriers per iteration (see psf_common.cuh), every block
// computing the same scalars so that all agree on when to stop.  The search
// direction update p = z + beta p is folded into the next operator phase.
//
// ScalingCG (CG.h:419-453) is the plain FP64 path, on the CSR (bit-exact
// pattern) or matrix-free.  The mixed-precision path runs that iteration in
// FP32 (operator, vectors) with FP64 dot products inside FP64 iterative
// refinement on the true residual.
#include <cmath>
#include <cstdio>

#include "psf_internal.cuh"
#include "psf_ebe.cuh"

namespace psf {


// ------------------------------------------------------------------ plain operator y = K x (+ optional r = b - K x, norm)
template <class T, int KIND>
__global__ void ebe_apply_kernel(Geo g, KeT<T> Ke, const T *__restrict__ Ep, const unsigned char *__restrict__ fixed,
                                 const T *__restrict__ x, T *__restrict__ y) {
    constexpr int nd = ndof_of<KIND>();
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < g.nnodes;
         n += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        node_ijk<KIND>(g, n, i, j, k);
        T yv[nd];
        ebe_node<T, KIND>(g, Ke, Ep, i, j, k, [&](long long a) { return x[a]; }, yv);
#pragma unroll
        for (int a = 0; a < nd; a++) y[n * nd + a] = fixed[n * nd + a] ? T(0) : yv[a];
    }
}

// r = b - K x (FP64), block partial of |r|^2 and |b|^2
template <int KIND>
__global__ void residual64_kernel(Geo g, KeT<double> Ke, const double *__restrict__ Ep,
                                  const unsigned char *__restrict__ fixed, const double *__restrict__ b,
                                  const double *__restrict__ x, double *__restrict__ r, double *partials) {
    constexpr int nd = ndof_of<KIND>();
    __shared__ double sm[64];
    double acc[2] = {0.0, 0.0};
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < g.nnodes;
         n += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        node_ijk<KIND>(g, n, i, j, k);
        double yv[nd];
        ebe_node<double, KIND>(g, Ke, Ep, i, j, k, [&](long long a) { return x[a]; }, yv);
#pragma unroll
        for (int a = 0; a < nd; a++) {
            const long long q = n * nd + a;
            const double rv = fixed[q] ? 0.0 : b[q] - yv[a];
            r[q] = rv;
            acc[0] += rv * rv;
            acc[1] += b[q] * b[q];
        }
    }
    block_sum<2>(acc, sm);
    if (threadIdx.x == 0) {
        partials[blockIdx.x] = acc[0];
        partials[gridDim.x + blockIdx.x] = acc[1];
    }
}

__global__ void finalize_sums(const double *partials, int nb, int nv, double *out) {
    // one warp per value, fixed order
    const int v = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (v >= nv) return;
    double a = 0.0;
    for (int b = lane; b < nb; b += 32) a += partials[(size_t)v * nb + b];
    a = warp_sum(a);
    if (lane == 0) out[v] = a;
}

// x64 += s * d32 (nodal)
__global__ void axpy_mixed(long long n, double s, const float *__restrict__ d, double *__restrict__ x) {
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x)
        x[q] += s * (double)d[q];
}

// ---- outer FP64 flexible CG around an FP32 inner solve (see outer_fcg64)
// z = s * d32; partial z.q_prev
__global__ void fcg_z_kernel(long long n, double s, const float *__restrict__ d, const double *__restrict__ qprev,
                             double *__restrict__ z, double *partials) {
    __shared__ double sm[32];
    double acc[1] = {0.0};
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
        const double zv = s * (double)d[q];
        z[q] = zv;
        acc[0] += zv * qprev[q];
    }
    block_sum<1>(acc, sm);
    if (threadIdx.x == 0) partials[blockIdx.x] = acc[0];
}
// p = z - beta p_prev (p_prev -> p in place); partial p.r
__global__ void fcg_p_kernel(long long n, double beta, const double *__restrict__ z, const double *__restrict__ r,
                             double *__restrict__ p, double *partials) {
    __shared__ double sm[32];
    double acc[1] = {0.0};
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
        const double pv = z[q] - beta * p[q];
        p[q] = pv;
        acc[0] += pv * r[q];
    }
    block_sum<1>(acc, sm);
    if (threadIdx.x == 0) partials[blockIdx.x] = acc[0];
}
// q = K p (FP64, matrix-free); partial p.q
template <int KIND>
__global__ void fcg_q_kernel(Geo g, KeT<double> Ke, const double *__restrict__ Ep, const unsigned char *__restrict__ fixed,
                             const double *__restrict__ p, double *__restrict__ q, double *partials) {
    constexpr int nd = ndof_of<KIND>();
    __shared__ double sm[32];
    double acc[1] = {0.0};
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < g.nnodes;
         n += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        node_ijk<KIND>(g, n, i, j, k);
        double yv[nd];
        ebe_node<double, KIND>(g, Ke, Ep, i, j, k, [&](long long a) { return p[a]; }, yv);
#pragma unroll
        for (int a = 0; a < nd; a++) {
            const long long t = n * nd + a;
            const double qv = fixed[t] ? 0.0 : yv[a];
            q[t] = qv;
            acc[0] += p[t] * qv;
        }
    }
    block_sum<1>(acc, sm);
    if (threadIdx.x == 0) partials[blockIdx.x] = acc[0];
}
// x += alpha p; r -= alpha q; partial |r|^2
__global__ void fcg_update_kernel(long long n, double alpha, const double *__restrict__ p, const double *__restrict__ qv,
                                  double *__restrict__ x, double *__restrict__ r, double *partials) {
    __shared__ double sm[32];
    double acc[1] = {0.0};
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
        x[q] += alpha * p[q];
        const double rv = r[q] - alpha * qv[q];
        r[q] = rv;
        acc[0] += rv * rv;
    }
    block_sum<1>(acc, sm);
    if (threadIdx.x == 0) partials[blockIdx.x] = acc[0];
}

// ------------------------------------------------------------------ persistent Jacobi PCG, matrix-free
template <class T>
struct PcgArgs {
    Geo g;
    KeT<T> Ke;
    const T *Ep;
    const T *D;                      // nodal diagonal (1 on fixed dofs)
    const unsigned char *fixed;
    const double *b;                 // nodal right-hand side (FP64), multiplied by bscale
    double bscale;
    const double *x0;                // optional FP64 start (nullptr: zero start)
    T *x, *r, *z, *pA, *pB, *Ap;
    int itmax;
    double eps;
    GridSync *gs;
    double *partials;
    double *out;                     // out[0] = iterations, out[1] = |r|^2, out[2] = |b|^2, out[3] = converged
};

template <class T, int KIND>
__global__ void __launch_bounds__(256) pcg_ebe_kernel(PcgArgs<T> A) {
    grid_sync_init();
    constexpr int nd = ndof_of<KIND>();
    __shared__ double sm[32 * 2];
    const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long stride = (long long)gridDim.x * blockDim.x;
    const Geo g = A.g;
    // ---- start: r = b - K x0, z = r / D, p_prev = 0
    {
        double acc[2] = {0.0, 0.0};
        for (long long n = tid; n < g.nnodes; n += stride) {
            T kx[nd];
            if (A.x0) {
                int i, j, k;
                node_ijk<KIND>(g, n, i, j, k);
                ebe_node<T, KIND>(g, A.Ke, A.Ep, i, j, k, [&](long long a) { return (T)A.x0[a]; }, kx);
            } else {
#pragma unroll
                for (int a = 0; a < nd; a++) kx[a] = T(0);
            }
#pragma unroll
            for (int a = 0; a < nd; a++) {
                const long long q = n * nd + a;
                const bool fx = A.fixed[q];
                const T bv = fx ? T(0) : (T)(A.b[q] * A.bscale);
                const T rv = fx ? T(0) : bv - kx[a];
                A.x[q] = A.x0 && !fx ? (T)A.x0[q] : T(0);
                A.r[q] = rv;
                const T zv = rv / A.D[q];
                A.z[q] = zv;
                A.pA[q] = T(0);
                acc[0] += (double)zv * (double)rv;
                acc[1] += (double)bv * (double)bv;
            }
        }
        block_sum<2>(acc, sm);
        if (!grid_sync<2, 0>(A.gs, A.partials, acc, 0.0)) return;
    }
    double zr = gs_result(A.gs, 0);
    const double bnorm = sqrt(gs_result(A.gs, 1));
    double beta = 0.0, rr = 0.0;
    T *pp = A.pA, *pn = A.pB;
    int it = 0, conv = 0;
    for (; it < A.itmax; it++) {
        // ---- phase A: p = z + beta p_prev (on the fly for neighbours), Ap = K p, p.Ap
        double pAp[1] = {0.0};
        const T tb = (T)beta;
        for (long long n = tid; n < g.nnodes; n += stride) {
            int i, j, k;
            node_ijk<KIND>(g, n, i, j, k);
            T yv[nd];
            ebe_node<T, KIND>(g, A.Ke, A.Ep, i, j, k,
                              [&](long long a) { return fma_t(tb, pp[a], A.z[a]); }, yv);
#pragma unroll
            for (int a = 0; a < nd; a++) {
                const long long q = n * nd + a;
                const T pv = fma_t(tb, pp[q], A.z[q]);
                const T av = A.fixed[q] ? T(0) : yv[a];
                pn[q] = pv;
                A.Ap[q] = av;
                pAp[0] += (double)pv * (double)av;
            }
        }
        block_sum<1>(pAp, sm);
        if (!grid_sync<1, 0>(A.gs, A.partials, pAp, 0.0)) return;
        const double alpha = zr / gs_result(A.gs, 0);
        // ---- phase B: x += alpha p, r -= alpha Ap, z = r / D, z.r and r.r
        double acc[2] = {0.0, 0.0};
        const T ta = (T)alpha, tma = (T)(-alpha);
        for (long long q = tid; q < g.nnodes * nd; q += stride) {
            const T pv = pn[q];
            A.x[q] = fma_t(ta, pv, A.x[q]);
            const T rv = fma_t(tma, A.Ap[q], A.r[q]);
            A.r[q] = rv;
            const T zv = rv / A.D[q];
            A.z[q] = zv;
            acc[0] += (double)zv * (double)rv;
            acc[1] += (double)rv * (double)rv;
        }
        block_sum<2>(acc, sm);
        if (!grid_sync<2, 0>(A.gs, A.partials, acc, 0.0)) return;
        const double zr1 = gs_result(A.gs, 0);
        rr = gs_result(A.gs, 1);
        beta = zr1 / zr;
        zr = zr1;
        T *t = pp; pp = pn; pn = t;
        if (sqrt(rr) < A.eps * bnorm) { it++; conv = 1; break; }
        if (!isfinite(rr)) { it++; break; }
    }
    if (tid == 0) {
        A.out[0] = it;
        A.out[1] = rr;
        A.out[2] = bnorm * bnorm;
        A.out[3] = conv;
    }
}

// ------------------------------------------------------------------ persistent Jacobi PCG on the CSR (FP64)
// Workspace (5 * rows doubles from w): r, z, p, Ap and the reciprocal diagonal.
struct PcgCsrArgs {
    long long rows;
    int jacobi;                      // 1: ScalingCG (z = r / D), 0: CG (CG.h:123-154, z = r)
    const int *indptr, *indices, *diag;   // diag[i] = position of (i, i), -1 when absent
    const double *data, *b;
    double *x, *r, *z, *p, *Ap, *Dinv;
    const int *sell_ptr, *sell_col;   // the sliced copy (one lane per row), else unused
    const double *sell_val;
    int itmax;
    double eps;
    GridSync *gs;
    double *partials;
    double *out;
};

__host__ __device__ inline void pcg_csr_carve(PcgCsrArgs &a, double *w, long long n) {
    a.r = w;
    a.z = w + n;
    a.p = w + 2 * n;
    a.Ap = w + 3 * n;
    a.Dinv = w + 4 * n;
}

// ScalingCG (CG.h:419-453): x0 = 0, r = b, z = r / D (GetDiagonal :397-404, Scaling :408-415),
// p = z; the recurrence residual ||r|| < eps ||b|| stops it (:443-448).
// On GB300 this iteration is bound by the FP64 pipe, not by HBM (a capture of the previous
// form, which formed p = z + beta p_prev inside the product, showed the FP64 pipe 85% busy
// and DRAM at 19%), so the FP64 work is kept to the minimum: one FMA per stored entry in the
// product, and the Jacobi scaling as a multiplication by the reciprocal diagonal (computed
// once; it differs from the reference's division by at most one rounding).  Three phases per
// iteration:
//   P  p = z + beta p (own rows)                                   -> barrier
//   S  Ap = A p (LANES lanes per row, every load of a row's entries in flight at once), p.Ap
//                                                                  -> barrier + 1 sum
//   U  x += alpha p, r -= alpha Ap, z = r / D, z.r and r.r         -> barrier + 2 sums
// The CSR arrays are read with streaming (evict-first) loads, so the vectors stay in L2.
// Launch shape: LANES lanes per CSR row in the product (32 / LANES rows per warp), THREADS
// threads per block; blocks per SM is chosen at launch (psf_set_launch_shape, autotuned).
// LANES = 1 reads the sliced copy instead (sell_fill_kernel): a warp owns a slice of 32 rows,
// each lane one row, and the warp's loads of the k-th entries of its rows are one contiguous
// 128-byte (columns) and 256-byte (values) segment.  Without the lane reduction and the slot
// padding of the multi-lane form, the product costs one FMA per stored entry, summed in the
// CSR order of the row (the order of CSR::operator* at CSR.h:108-122).
template <int LANES, int THREADS>
__global__ void __launch_bounds__(THREADS, 1024 / THREADS) pcg_csr_kernel(PcgCsrArgs A) {
    constexpr int kPcgRowLanes = LANES;
    grid_sync_init();
    __shared__ double sm[2 * THREADS];
    const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long stride = (long long)gridDim.x * blockDim.x;
    const long long rows = A.rows;
    {
        double acc[2] = {0.0, 0.0};
        for (long long i = tid; i < rows; i += stride) {
            const double bv = A.b[i];
            double Di = 1.0;
            if (A.jacobi) {
                const int d = A.diag[i];
                const double D = d >= 0 ? A.data[d] : 0.0;   // CSR::get(i, i): zero when the entry is absent
                // the reference divides by it (CG.h:412) and lets inf / NaN run; here the solve stops
                if (!(D != 0.0) || !isfinite(D)) atomicCAS(&A.gs->status, 0, (int)PSF_BAD_INPUT);
                Di = 1.0 / D;
            }
            A.Dinv[i] = Di;
            A.x[i] = 0.0;
            A.r[i] = bv;
            const double zv = bv * Di;
            A.z[i] = zv;
            A.p[i] = 0.0;
            acc[0] += zv * bv;
            acc[1] += bv * bv;
        }
        block_sum_wide<2>(acc, sm);
        if (!grid_sync<2, 0>(A.gs, A.partials, acc, 0.0)) return;
    }
    double zr = gs_result(A.gs, 0);
    const double bnorm = sqrt(gs_result(A.gs, 1));
    double beta = 0.0, rr = 0.0;
    int it = 0, conv = 0;
    const int lane = threadIdx.x & 31, sub = lane & (kPcgRowLanes - 1);
    const long long rows_per_warp = 32 / kPcgRowLanes;
    const long long gw = tid >> 5, nw = stride >> 5;
    // entries a lane handles per round (slots): one round covers 20 (4 lanes), 24 (8) or 32 (16)
    // entries of a row, so a 2D row (at most 18) takes one round and its loads are all in flight
    // at once: the indices and values, then the gathers, then the products
    constexpr int SL = kPcgRowLanes == 4 ? 5 : (kPcgRowLanes == 8 ? 3 : 2);
    for (; it < A.itmax; it++) {
        // ---- P
        for (long long i = tid; i < rows; i += stride) A.p[i] = fma(beta, A.p[i], A.z[i]);
        if (!grid_barrier(A.gs, A.partials)) return;
        // ---- S
        double pAp[1] = {0.0};
        if constexpr (LANES == 1) {
            constexpr int U = 6;   // entries in flight per lane (a 2D row of 18 entries: three rounds)
            const long long nsl = (rows + 31) >> 5;
            for (long long sl = gw; sl < nsl; sl += nw) {
                const long long i = (sl << 5) + lane;
                const int s0 = __ldg(A.sell_ptr + sl), s1 = __ldg(A.sell_ptr + sl + 1);
                double v = 0.0;
                // s1 - s0 is a multiple of 32, so the bounds below are the same in every lane
                for (int q = s0; q < s1; q += 32 * U) {
                    int j[U];
                    double a[U];
#pragma unroll
                    for (int t = 0; t < U; t++) {
                        const int qt = q + 32 * t + lane;
                        const bool h = q + 32 * t < s1;
                        j[t] = h ? __ldcs(A.sell_col + qt) : 0;
                        a[t] = h ? __ldcs(A.sell_val + qt) : 0.0;
                    }
                    double g[U];
#pragma unroll
                    for (int t = 0; t < U; t++) g[t] = q + 32 * t < s1 ? A.p[j[t]] : 0.0;
#pragma unroll
                    for (int t = 0; t < U; t++)
                        if (q + 32 * t < s1) v = fma(a[t], g[t], v);
                }
                if (i < rows) {
                    A.Ap[i] = v;
                    pAp[0] = fma(A.p[i], v, pAp[0]);
                }
            }
        } else {
        long long base = gw * rows_per_warp;
        int rs_n = 0, re_n = 0;   // the row bounds are fetched one pass ahead
        {
            const long long i0 = base + lane / kPcgRowLanes;
            if (i0 < rows) { rs_n = __ldg(A.indptr + i0); re_n = __ldg(A.indptr + i0 + 1); }
        }
        for (; base < rows; base += nw * rows_per_warp) {
            const long long i = base + lane / kPcgRowLanes;
            const int rs = rs_n, re = re_n;
            {
                const long long i1 = i + nw * rows_per_warp;
                if (i1 < rows) { rs_n = __ldg(A.indptr + i1); re_n = __ldg(A.indptr + i1 + 1); }
            }
            double v = 0.0;
            if (i < rows) {
                for (int q = rs + sub; q < re; q += SL * kPcgRowLanes) {
                    int j[SL];
                    double a[SL];
#pragma unroll
                    for (int t = 0; t < SL; t++) {
                        const int qt = q + t * kPcgRowLanes;
                        const bool h = qt < re;
                        j[t] = h ? __ldcs(A.indices + qt) : -1;
                        a[t] = h ? __ldcs(A.data + qt) : 0.0;
                    }
                    double g[SL];
#pragma unroll
                    for (int t = 0; t < SL; t++) g[t] = j[t] >= 0 ? A.p[j[t]] : 0.0;
#pragma unroll
                    for (int t = 0; t < SL; t++) v = fma(a[t], g[t], v);
                }
            }
#pragma unroll
            for (int o = 1; o < kPcgRowLanes; o <<= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
            if (sub == 0 && i < rows) {
                A.Ap[i] = v;
                pAp[0] += A.p[i] * v;
            }
        }
        }
        block_sum_wide<1>(pAp, sm);
        if (!grid_sync<1, 0>(A.gs, A.partials, pAp, 0.0)) return;
        const double alpha = zr / gs_result(A.gs, 0);
        // ---- U
        double acc[2] = {0.0, 0.0};
        for (long long i = tid; i < rows; i += stride) {
            A.x[i] = fma(alpha, A.p[i], A.x[i]);
            const double rv = fma(-alpha, A.Ap[i], A.r[i]);
            A.r[i] = rv;
            const double zv = rv * A.Dinv[i];
            A.z[i] = zv;
            acc[0] += zv * rv;
            acc[1] += rv * rv;
        }
        block_sum_wide<2>(acc, sm);
        if (!grid_sync<2, 0>(A.gs, A.partials, acc, 0.0)) return;
        const double zr1 = gs_result(A.gs, 0);
        rr = gs_result(A.gs, 1);
        beta = zr1 / zr;
        zr = zr1;
        if (sqrt(rr) < A.eps * bnorm) { it++; conv = 1; break; }
        if (!isfinite(rr)) { it++; break; }
    }
    if (tid == 0) {
        A.out[0] = it;
        A.out[1] = rr;
        A.out[2] = bnorm * bnorm;
        A.out[3] = conv;
    }
}

// the instantiated shapes: lanes per row {4, 8, 16} x threads per block {256, 512, 1024}
static const void *pcg_csr_fn(int lanes, int threads) {
#define PSF_PCG_SHAPE(L, T) \
    if (lanes == L && threads == T) return (const void *)pcg_csr_kernel<L, T>;
    PSF_PCG_SHAPE(1, 256) PSF_PCG_SHAPE(1, 512) PSF_PCG_SHAPE(1, 1024)
    PSF_PCG_SHAPE(4, 256) PSF_PCG_SHAPE(4, 512) PSF_PCG_SHAPE(4, 1024)
    PSF_PCG_SHAPE(8, 256) PSF_PCG_SHAPE(8, 512) PSF_PCG_SHAPE(8, 1024)
    PSF_PCG_SHAPE(16, 256) PSF_PCG_SHAPE(16, 512) PSF_PCG_SHAPE(16, 1024)
#undef PSF_PCG_SHAPE
    return nullptr;
}

// blocks of a persistent launch: blocks_per_sm per SM (at most what fits), at most one block
// per `work_per_block` units of work, at least one
static psf_status persistent_blocks(const void *fn, int threads, int sms, int blocks_per_sm, long long work,
                                    long long work_per_block, int *blocks) {
    int per_sm = 0;
    PSF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, 0));
    if (per_sm < 1) { set_error("persistent kernel does not fit on an SM"); return PSF_CUDA_ERROR; }
    long long b = (long long)sms * (per_sm < blocks_per_sm ? per_sm : blocks_per_sm);
    const long long need = (work + work_per_block - 1) / work_per_block;
    if (b > need) b = need;
    *blocks = (int)(b < 1 ? 1 : b);
    return PSF_OK;
}

// ------------------------------------------------------------------ host side
template <class T>
static KeT<T> ke_param(const Ctx *c) {
    KeT<T> k{};
    const int nk = c->nen * c->ndof;
    for (int q = 0; q < nk * nk; q++) k.v[q] = (T)c->Ke0_host[q];
    return k;
}

static Geo geo_of(const Ctx *c) {
    Geo g;
    g.nx = c->nx; g.ny = c->ny; g.nz = c->nz;
    g.nnodes = c->nnodes;
    return g;
}

template <class T>
static psf_status ebe_apply_t(Ctx *c, const T *x, T *y, const T *Ep) {
    Geo g = geo_of(c);
    KeT<T> Ke = ke_param<T>(c);
    const int nb = grid_for(c->nnodes, 256, c->num_sms * 8);
    switch (c->kind) {
    case PSF_Q4_PLANE_STRAIN:
        (ebe_apply_kernel<T, 0><<<nb, 256, 0, c->stream>>>(g, Ke, Ep, c->fixed, x, y), ::psf::note_launch());
        break;
    case PSF_Q4_HEAT:
        (ebe_apply_kernel<T, 1><<<nb, 256, 0, c->stream>>>(g, Ke, Ep, c->fixed, x, y), ::psf::note_launch());
        break;
    default:
        (ebe_apply_kernel<T, 2><<<nb, 256, 0, c->stream>>>(g, Ke, Ep, c->fixed, x, y), ::psf::note_launch());
        break;
    }
    PSF_CUDA(cudaGetLastError());
    return PSF_OK;
}

psf_status ebe_apply64(Ctx *c, const double *xn, double *yn) { return ebe_apply_t<double>(c, xn, yn, c->Epad); }
psf_status ebe_apply32(Ctx *c, const float *xn, float *yn) { return ebe_apply_t<float>(c, xn, yn, c->Epadf); }

// r = b - K x in FP64 (nodal); returns |r| and |b| on the host
static psf_status residual64(Ctx *c, const double *b, const double *x, double *r, double *rnorm, double *bnorm) {
    Geo g = geo_of(c);
    KeT<double> Ke = ke_param<double>(c);
    const int nb = grid_for(c->nnodes, 256, c->num_sms * 4);
    switch (c->kind) {
    case PSF_Q4_PLANE_STRAIN:
        (residual64_kernel<0><<<nb, 256, 0, c->stream>>>(
             g, Ke, c->Epad, c->fixed, b, x, r, c->partials),
         ::psf::note_launch());
        break;
    case PSF_Q4_HEAT:
        (residual64_kernel<1><<<nb, 256, 0, c->stream>>>(
             g, Ke, c->Epad, c->fixed, b, x, r, c->partials),
         ::psf::note_launch());
        break;
    default:
        (residual64_kernel<2><<<nb, 256, 0, c->stream>>>(
             g, Ke, c->Epad, c->fixed, b, x, r, c->partials),
         ::psf::note_launch());
        break;
    }
    (finalize_sums<<<1, 64, 0, c->stream>>>(c->partials, nb, 2, c->scal + 8), ::psf::note_launch());
    PSF_CUDA(cudaGetLastError());
    double h[2];
    PSF_CUDA(cudaMemcpyAsync(h, c->scal + 8, 2 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    PSF_CUDA(cudaStreamSynchronize(c->stream));
    *rnorm = sqrt(h[0]);
    *bnorm = sqrt(h[1]);
    return PSF_OK;
}

psf_status add_kernel_time(Ctx *c) {
    float ms = 0.f;
    PSF_CUDA(cudaEventSynchronize(c->evk1));
    PSF_CUDA(cudaEventElapsedTime(&ms, c->evk0, c->evk1));
    c->ksec += ms * 1e-3;
    c->klaunch++;
    return PSF_OK;
}

psf_status residual64_pub(Ctx *c, const double *b, const double *x, double *r, double *rnorm, double *bnorm) {
    return residual64(c, b, x, r, rnorm, bnorm);
}

template <class T, int KIND>
static psf_status run_pcg_ebe(Ctx *c, PcgArgs<T> &a, int *iters, double *rr, double *bb, int *conv) {
    const void *fn = (const void *)pcg_ebe_kernel<T, KIND>;
    int per_sm = 0;
    PSF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, pcg_ebe_kernel<T, KIND>, 256, 0));
    if (per_sm < 1) { set_error("persistent PCG kernel does not fit on an SM"); return PSF_CUDA_ERROR; }
    int blocks = c->num_sms * (per_sm < 4 ? per_sm : 4);
    long long need = (c->nnodes + 255) / 256;
    if (blocks > need) blocks = (int)need;
    if (blocks < 1) blocks = 1;
    void *args[] = {&a};
    PSF_CUDA(cudaEventRecord(c->evk0, c->stream));
    PSF_CHECK(launch_coop(c, fn, blocks, 256, args));
    PSF_CUDA(cudaEventRecord(c->evk1, c->stream));
    PSF_CHECK(read_sync_status(c));
    PSF_CHECK(add_kernel_time(c));
    double h[4];
    PSF_CUDA(cudaMemcpyAsync(h, a.out, sizeof h, cudaMemcpyDeviceToHost, c->stream));
    PSF_CUDA(cudaStreamSynchronize(c->stream));
    *iters = (int)h[0];
    *rr = h[1];
    *bb = h[2];
    *conv = (int)h[3];
    if (!std::isfinite(h[1]) || !std::isfinite(h[2])) {
        set_error("non-finite residual (non-finite matrix or right-hand side entries)");
        return PSF_NOT_FINITE;
    }
    return PSF_OK;
}

// A diagnostic of the bounded device waits: block absent_block never arrives at the barrier (its
// arrival is the flag nothing sets); the others give up after spin_limit polls, record PSF_TIMEOUT
// and return, so the host reads the status and the context stays usable.
__global__ void barrier_timeout_probe(GridSync *gs, double *partials, int absent_block, long long spin_limit) {
    grid_sync_init();
    if ((int)blockIdx.x == absent_block) return;
    double v[1] = {0.0};
    grid_sync<0, 0>(gs, partials, v, 0.0, spin_limit);
}

psf_status diag_barrier_timeout(Ctx *c, int blocks, long long spin_limit) {
    int per_sm = 0;
    PSF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, barrier_timeout_probe, 128, 0));
    if (blocks < 2 || blocks > c->num_sms * per_sm) {
        set_error("psf_diag_barrier_timeout: blocks must be in [2, resident blocks]");
        return PSF_BAD_INPUT;
    }
    GridSync *gs = c->gs;
    double *partials = c->partials;
    int absent = blocks - 1;
    void *args[] = {&gs, &partials, &absent, &spin_limit};
    PSF_CHECK(launch_coop(c, (const void *)barrier_timeout_probe, blocks, 128, args));
    const psf_status st = read_sync_status(c);
    PSF_CHECK(reset_sync(c));
    return st;
}

template <class T>
static psf_status pcg_ebe(Ctx *c, const double *b, double bscale, const double *x0, T *x, T **w, int itmax,
                          double eps, int *iters, double *rr, double *bb, int *conv) {
    PcgArgs<T> a;
    a.g = geo_of(c);
    a.Ke = ke_param<T>(c);
    if constexpr (sizeof(T) == 8) { a.Ep = (const T *)c->Epad; a.D = (const T *)c->Dn; }
    else { a.Ep = (const T *)c->Epadf; a.D = (const T *)c->Dnf; }
    a.fixed = c->fixed;
    a.b = b;
    a.bscale = bscale;
    a.x0 = x0;
    a.x = x; a.r = w[0]; a.z = w[1]; a.pA = w[2]; a.pB = w[3]; a.Ap = w[4];
    a.itmax = itmax;
    a.eps = eps;
    a.gs = c->gs;
    a.partials = c->partials;
    a.out = c->scal + 12;
    switch (c->kind) {
    case PSF_Q4_PLANE_STRAIN: return run_pcg_ebe<T, 0>(c, a, iters, rr, bb, conv);
    case PSF_Q4_HEAT: return run_pcg_ebe<T, 1>(c, a, iters, rr, bb, conv);
    default: return run_pcg_ebe<T, 2>(c, a, iters, rr, bb, conv);
    }
}

// ------------------------------------------------------------------ sliced copy of the CSR
// Slice s (rows 32s .. 32s+31) is as wide as its longest row; entry k of row 32s + l sits at
// slot sell_ptr[s] + 32k + l.  Short rows are padded with column = the row, value 0, so the
// padded products add exact zeros.

// width of every slice (one thread per slice)
__global__ void sell_width_kernel(long long rows, long long nsl, const int *__restrict__ indptr, int *__restrict__ width) {
    for (long long sl = blockIdx.x * (long long)blockDim.x + threadIdx.x; sl < nsl;
         sl += (long long)gridDim.x * blockDim.x) {
        const long long i0 = sl << 5, i1 = i0 + 32 < rows ? i0 + 32 : rows;
        int w = 0;
        for (long long i = i0; i < i1; i++) {
            const int l = indptr[i + 1] - indptr[i];
            w = l > w ? l : w;
        }
        width[sl] = w;
    }
}

// exclusive scan of 32 * width into ptr[0 .. nsl] (one block of 1024 threads, chunked)
__global__ void __launch_bounds__(1024) sell_scan_kernel(long long nsl, int *__restrict__ ptr) {
    __shared__ long long warp_tot[32];
    __shared__ long long carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (long long b = 0; b < nsl; b += 1024) {
        const long long sl = b + threadIdx.x;
        const long long w = sl < nsl ? 32ll * ptr[sl] : 0;
        long long x = w;   // inclusive scan in the warp
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const long long y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) warp_tot[wid] = x;
        __syncthreads();
        if (wid == 0) {
            long long t = warp_tot[lane], u = t;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const long long y = __shfl_up_sync(0xffffffffu, u, o);
                if (lane >= o) u += y;
            }
            warp_tot[lane] = u - t;   // exclusive over the warps
        }
        __syncthreads();
        const long long excl = carry + warp_tot[wid] + x - w;
        __syncthreads();
        if (sl < nsl) ptr[sl] = (int)excl;
        if (threadIdx.x == 1023) carry = excl + w;
        __syncthreads();
    }
    if (threadIdx.x == 0) ptr[nsl] = carry > 0x7fffffffll ? -1 : (int)carry;   // -1: too many slots
}

// the columns and values (one thread per row slot of a slice)
__global__ void sell_fill_kernel(long long rows, long long nsl, const int *__restrict__ indptr,
                                 const int *__restrict__ indices, const double *__restrict__ data,
                                 const int *__restrict__ ptr, int *__restrict__ col, double *__restrict__ val) {
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < (nsl << 5);
         t += (long long)gridDim.x * blockDim.x) {
        const long long sl = t >> 5;
        const int l = (int)(t & 31);
        const int s0 = ptr[sl], wd = (ptr[sl + 1] - s0) >> 5;
        const bool live = t < rows;
        const int rs = live ? indptr[t] : 0, len = live ? indptr[t + 1] - rs : 0;
        const int self = (int)(live ? t : rows - 1);
        for (int k = 0; k < wd; k++) {
            const bool h = k < len;
            col[s0 + 32 * k + l] = h ? indices[rs + k] : self;
            val[s0 + 32 * k + l] = h ? data[rs + k] : 0.0;
        }
    }
}

// builds the context's sliced copy of a device CSR (storage grown on demand)
static psf_status sell_prepare(Ctx *c, long long rows, const int *indptr, const int *indices, const double *data) {
    const long long nsl = (rows + 31) >> 5;
    if (c->sell_ptr_cap < nsl + 1) {
        if (c->sell_ptr) cudaFreeAsync(c->sell_ptr, c->stream);
        c->sell_ptr = nullptr;
        c->sell_ptr_cap = 0;
        PSF_CUDA(cudaMallocAsync((void **)&c->sell_ptr, sizeof(int) * (nsl + 1), c->stream));
        c->sell_ptr_cap = nsl + 1;
    }
    const int gw = grid_for(nsl, 256, 4096);
    (sell_width_kernel<<<gw, 256, 0, c->stream>>>(rows, nsl, indptr, c->sell_ptr), note_launch());
    PSF_CUDA(cudaGetLastError());
    (sell_scan_kernel<<<1, 1024, 0, c->stream>>>(nsl, c->sell_ptr), note_launch());
    PSF_CUDA(cudaGetLastError());
    int total = 0;
    PSF_CUDA(cudaMemcpyAsync(&total, c->sell_ptr + nsl, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    PSF_CUDA(cudaStreamSynchronize(c->stream));
    if (total < 0) { set_error("sliced CSR copy exceeds 2^31 slots"); return PSF_BAD_INPUT; }
    if (c->sell_cap < total) {
        if (c->sell_col) cudaFreeAsync(c->sell_col, c->stream);
        if (c->sell_val) cudaFreeAsync(c->sell_val, c->stream);
        c->sell_col = nullptr;
        c->sell_val = nullptr;
        c->sell_cap = 0;
        PSF_CUDA(cudaMallocAsync((void **)&c->sell_col, sizeof(int) * total, c->stream));
        PSF_CUDA(cudaMallocAsync((void **)&c->sell_val, sizeof(double) * total, c->stream));
        c->sell_cap = total;
    }
    (sell_fill_kernel<<<grid_for(nsl << 5, 256, 65536), 256, 0, c->stream>>>(rows, nsl, indptr, indices, data,
                                                                            c->sell_ptr, c->sell_col, c->sell_val),
     note_launch());
    PSF_CUDA(cudaGetLastError());
    return PSF_OK;
}

// Jacobi PCG (jacobi = 1) or CG (jacobi = 0) on any device CSR; w holds 5*rows doubles
psf_status pcg_csr_any(Ctx *c, long long rows, const int *indptr, const int *indices, const int *diag,
                       const double *data, const double *b, double *x, double *w, int jacobi, int itmax, double eps,
                       int *iters, double *rr, double *bb, int *conv) {
    PcgCsrArgs a;
    a.jacobi = jacobi;
    a.rows = rows;
    a.indptr = indptr; a.indices = indices; a.diag = diag; a.data = data;
    a.b = b;
    a.x = x;
    const long long n = rows;
    pcg_csr_carve(a, w, n);
    a.sell_ptr = nullptr; a.sell_col = nullptr; a.sell_val = nullptr;
    // the solve's time includes building the sliced copy
    PSF_CUDA(cudaEventRecord(c->evk0, c->stream));
    if (c->pcg_lanes == kPcgSliced) {
        PSF_CHECK(sell_prepare(c, rows, indptr, indices, data));
        a.sell_ptr = c->sell_ptr; a.sell_col = c->sell_col; a.sell_val = c->sell_val;
    }
    a.itmax = itmax;
    a.eps = eps;
    a.gs = c->gs;
    a.partials = c->partials;
    a.out = c->scal + 12;
    const void *fn = pcg_csr_fn(c->pcg_lanes, c->pcg_threads);
    if (!fn) { set_error("PCG launch shape not instantiated"); return PSF_BAD_INPUT; }
    int blocks = 0;
    PSF_CHECK(persistent_blocks(fn, c->pcg_threads, c->num_sms, c->pcg_blocks_per_sm, n,
                                c->pcg_threads / c->pcg_lanes, &blocks));
    void *args[] = {&a};
    PSF_CHECK(launch_coop(c, fn, blocks, c->pcg_threads, args));
    PSF_CUDA(cudaEventRecord(c->evk1, c->stream));
    PSF_CHECK(read_sync_status(c));
    PSF_CHECK(add_kernel_time(c));
    double h[4];
    PSF_CUDA(cudaMemcpyAsync(h, a.out, sizeof h, cudaMemcpyDeviceToHost, c->stream));
    PSF_CUDA(cudaStreamSynchronize(c->stream));
    *iters = (int)h[0];
    *rr = h[1];
    *bb = h[2];
    *conv = (int)h[3];
    if (!std::isfinite(h[1]) || !std::isfinite(h[2])) {
        set_error("non-finite residual (non-finite matrix or right-hand side entries)");
        return PSF_NOT_FINITE;
    }
    return PSF_OK;
}

// ------------------------------------------------------------------ BiCGSTAB (CG.h:158-193)
struct BicgArgs {
    long long rows;
    const int *indptr, *indices;
    const double *data, *b;
    double *x, *r, *rd, *p, *Ap, *s, *As;
    int itmax;
    double eps;
    GridSync *gs;
    double *partials;
    double *out;
};

// y[i] = (A v)[i] for the rows of this warp group: four lanes per row, warp-uniform loop
__device__ __forceinline__ void csr_rows4(const BicgArgs &A, const double *__restrict__ v, double *__restrict__ y,
                                          long long tid, long long rstride, double *dot_with, double *dot_out,
                                          double *dot_self) {
    const int sub = threadIdx.x & 3;
    for (long long base = (tid >> 5) << 3; base < A.rows; base += rstride) {
        const long long i = base + ((threadIdx.x & 31) >> 2);
        double acc = 0.0;
        if (i < A.rows)
            for (int q = A.indptr[i] + sub; q < A.indptr[i + 1]; q += 4) acc += A.data[q] * v[A.indices[q]];
        acc += __shfl_xor_sync(0xffffffffu, acc, 1);
        acc += __shfl_xor_sync(0xffffffffu, acc, 2);
        if (sub == 0 && i < A.rows) {
            y[i] = acc;
            if (dot_with) *dot_out += dot_with[i] * acc;
            if (dot_self) *dot_self += acc * acc;
        }
    }
}

// BiCGSTAB of the reference (x0 = 0, shadow residual rd = r0, stop on ||r|| < eps ||b||),
// one persistent launch with five grid phases per iteration
__global__ void __launch_bounds__(256) bicgstab_csr_kernel(BicgArgs A) {
    grid_sync_init();
    __shared__ double sm[32 * 2];
    const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long stride = (long long)gridDim.x * blockDim.x;
    const long long rstride = stride >> 2;
    {
        double acc[2] = {0.0, 0.0};
        for (long long i = tid; i < A.rows; i += stride) {
            const double bv = A.b[i];
            A.x[i] = 0.0;
            A.r[i] = bv;           // r0 = b - A 0
            A.rd[i] = bv;
            A.p[i] = bv;
            acc[0] += bv * bv;     // rd . r
            acc[1] += bv * bv;
        }
        block_sum<2>(acc, sm);
        if (!grid_sync<2, 0>(A.gs, A.partials, acc, 0.0)) return;
    }
    double rdr = gs_result(A.gs, 0);
    const double bnorm = sqrt(gs_result(A.gs, 1));
    double rr = gs_result(A.gs, 1);
    int it = 0, conv = 0;
    for (; it < A.itmax; it++) {
        // Ap = A p, rd . Ap
        double d1[1] = {0.0};
        csr_rows4(A, A.p, A.Ap, tid, rstride, A.rd, &d1[0], nullptr);
        block_sum<1>(d1, sm);
        if (!grid_sync<1, 0>(A.gs, A.partials, d1, 0.0)) return;
        const double alpha = rdr / gs_result(A.gs, 0);
        // s = r - alpha Ap
        for (long long i = tid; i < A.rows; i += stride) A.s[i] = 1.0 * A.r[i] + (-alpha) * A.Ap[i];
        if (!grid_barrier(A.gs, A.partials)) return;
        // As = A s, As . s, As . As
        double d2[2] = {0.0, 0.0};
        csr_rows4(A, A.s, A.As, tid, rstride, A.s, &d2[0], &d2[1]);
        block_sum<2>(d2, sm);
        if (!grid_sync<2, 0>(A.gs, A.partials, d2, 0.0)) return;
        const double omega = gs_result(A.gs, 0) / gs_result(A.gs, 1);
        // x += alpha p + omega s, r = s - omega As, rd . r, r . r
        double d3[2] = {0.0, 0.0};
        for (long long i = tid; i < A.rows; i += stride) {
            A.x[i] = 1.0 * A.x[i] + alpha * A.p[i] + omega * A.s[i];
            const double rv = 1.0 * A.s[i] + (-omega) * A.As[i];
            A.r[i] = rv;
            d3[0] += A.rd[i] * rv;
            d3[1] += rv * rv;
        }
        block_sum<2>(d3, sm);
        if (!grid_sync<2, 0>(A.gs, A.partials, d3, 0.0)) return;
        const double rdr1 = gs_result(A.gs, 0);
        rr = gs_result(A.gs, 1);
        const double beta = alpha / omega * rdr1 / rdr;
        rdr = rdr1;
        if (sqrt(rr) < A.eps * bnorm) { it++; conv = 1; break; }
        if (!isfinite(rr)) { it++; break; }
        // p = beta p + r - beta omega Ap
        const double mbo = -beta * omega;
        for (long long i = tid; i < A.rows; i += stride) A.p[i] = beta * A.p[i] + 1.0 * A.r[i] + mbo * A.Ap[i];
        if (!grid_barrier(A.gs, A.partials)) return;
    }
    if (tid == 0) {
        A.out[0] = it;
        A.out[1] = rr;
        A.out[2] = bnorm * bnorm;
        A.out[3] = conv;
    }
}

// v: six work vectors of `rows` doubles (r, rd, p, Ap, s, As)
psf_status bicgstab_csr_any(Ctx *c, long long rows, const int *indptr, const int *indices, const double *data,
                            const double *b, double *x, double *const v[6], int itmax, double eps, int *iters,
                            double *rr, double *bb, int *conv) {
    BicgArgs a;
    a.rows = rows;
    a.indptr = indptr; a.indices = indices; a.data = data;
    a.b = b;
    a.x = x;
    const long long n = rows;
    a.r = v[0]; a.rd = v[1]; a.p = v[2]; a.Ap = v[3]; a.s = v[4]; a.As = v[5];
    a.itmax = itmax;
    a.eps = eps;
    a.gs = c->gs;
    a.partials = c->partials;
    a.out = c->scal + 12;
    int per_sm = 0;
    PSF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, bicgstab_csr_kernel, 256, 0));
    if (per_sm < 1) { set_error("persistent BiCGSTAB kernel does not fit on an SM"); return PSF_CUDA_ERROR; }
    int blocks = c->num_sms * (per_sm < 4 ? per_sm : 4);
    long long need = (n * 4 + 255) / 256;
    if (blocks > need) blocks = (int)need;
    if (blocks < 1) blocks = 1;
    void *args[] = {&a};
    PSF_CUDA(cudaEventRecord(c->evk0, c->stream));
    PSF_CHECK(launch_coop(c, (const void *)bicgstab_csr_kernel, blocks, 256, args));
    PSF_CUDA(cudaEventRecord(c->evk1, c->stream));
    PSF_CHECK(read_sync_status(c));
    PSF_CHECK(add_kernel_time(c));
    double h[4];
    PSF_CUDA(cudaMemcpyAsync(h, a.out, sizeof h, cudaMemcpyDeviceToHost, c->stream));
    PSF_CUDA(cudaStreamSynchronize(c->stream));
    *iters = (int)h[0];
    *rr = h[1];
    *bb = h[2];
    *conv = (int)h[3];
    return PSF_OK;
}

// Cooperative launch of pcg_csr_kernel (ScalingCG) on caller-owned device
// buffers and the caller's stream, without a context and without allocating:
// w holds at least 5*rows doubles, gs is zeroed here, partials holds kPartialSlots*blocks
// doubles, out receives iterations, |r|^2, |b|^2, converged.
psf_status pcg_csr_launch_raw(cudaStream_t s, long long rows, const int *indptr, const int *indices, const int *diag,
                              const double *data, const double *b, double *x, double *w, int itmax, double eps,
                              GridSync *gs, double *partials, int max_blocks, double *out) {
    PcgCsrArgs a;
    a.jacobi = 1;
    a.rows = rows;
    a.indptr = indptr; a.indices = indices; a.diag = diag; a.data = data;
    a.b = b;
    a.x = x;
    pcg_csr_carve(a, w, rows);
    a.sell_ptr = nullptr; a.sell_col = nullptr; a.sell_val = nullptr;
    a.itmax = itmax;
    a.eps = eps;
    a.gs = gs;
    a.partials = partials;
    a.out = out;
    int dev = 0, sms = 0;
    PSF_CUDA(cudaGetDevice(&dev));
    PSF_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const void *fn = pcg_csr_fn(kPcgDefaultLanes, kPcgDefaultThreads);
    int blocks = 0;
    PSF_CHECK(persistent_blocks(fn, kPcgDefaultThreads, sms, kPcgDefaultBlocksPerSm, rows,
                                kPcgDefaultThreads / kPcgDefaultLanes, &blocks));
    if (blocks > max_blocks) blocks = max_blocks;
    PSF_CUDA(cudaMemsetAsync(gs, 0, sizeof(GridSync), s));
    void *args[] = {&a};
    PSF_CUDA(cudaLaunchCooperativeKernel(fn, dim3(blocks), dim3(kPcgDefaultThreads), args, 0, s));
    note_launch();
    return PSF_OK;
}

// loads the module of the persistent PCG kernel (its code and static data), without a launch
psf_status pcg_csr_load_module() {
    cudaFuncAttributes fa;
    PSF_CUDA(cudaFuncGetAttributes(&fa, pcg_csr_fn(kPcgDefaultLanes, kPcgDefaultThreads)));
    return PSF_OK;
}

static psf_status pcg_csr(Ctx *c, int itmax, double eps, int *iters, double *rr, double *bb, int *conv) {
    // 5 reduced-length buffers carved from the nodal scratch
    return pcg_csr_any(c, c->nfree, c->indptr, c->indices, c->diag, c->data, c->F, c->u, c->w64[0], 1, itmax, eps,
                       iters, rr, bb, conv);
}

psf_status mg_solve(Ctx *c, int itmax, double eps, bool warm, psf_solve_info *info);  // psf_mg.cu

static psf_status sum_partials_host(Ctx *c, int nb, double *out) {
    (finalize_sums<<<1, 32, 0, c->stream>>>(c->partials, nb, 1, c->scal + 8), ::psf::note_launch());
    PSF_CUDA(cudaGetLastError());
    PSF_CUDA(cudaMemcpyAsync(out, c->scal + 8, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    PSF_CUDA(cudaStreamSynchronize(c->stream));
    return PSF_OK;
}

// FP32 Jacobi-PCG inner solve of K d = r / |r| into c->w32[5]
static psf_status inner_solve(Ctx *c, int solver, const double *r, double bscale, int itmax, double tol, int *iters) {
    (void)solver;
    int conv;
    double rr, bb;
    return pcg_ebe<float>(c, r, bscale, nullptr, c->w32[5], c->w32, itmax, tol, iters, &rr, &bb, &conv);
}

// Mixed-precision solve: flexible CG in FP64 (true FP64 operator, dot products,
// recurrences) whose preconditioner is an FP32 inner solve.  Stationary
// refinement x += K32^-1 r stalls once eps32 * cond(K) approaches one (the
// 1M-dof SIMP operators reach that); the K-orthogonalised outer directions
// keep converging.  FCG(1): p = z - (z.Kp_prev / p_prev.Kp_prev) p_prev.
static psf_status outer_fcg64(Ctx *c, int solver, int itmax, double eps, bool warm, psf_solve_info *inf) {
    double *x = c->w64[5], *r = c->w64[6], *z = c->w64[7], *p = c->w64[1], *q = c->w64[2];
    const long long n = c->ndofs;
    if (warm) PSF_CUDA(cudaMemcpyAsync(x, c->un, sizeof(double) * n, cudaMemcpyDeviceToDevice, c->stream));
    else PSF_CUDA(cudaMemsetAsync(x, 0, sizeof(double) * n, c->stream));
    PSF_CUDA(cudaMemsetAsync(p, 0, sizeof(double) * n, c->stream));
    PSF_CUDA(cudaMemsetAsync(q, 0, sizeof(double) * n, c->stream));
    const double inner_tol = 1e-3;
    const int inner_cap = 20000;
    const int max_outer = 200;
    double rn = 0, bn = 0, pq_prev = 1.0;
    PSF_CHECK(residual64(c, c->Fn, x, r, &rn, &bn));
    int total = 0, outer = 0;
    bool ok = bn == 0.0 || rn <= eps * bn;
    const int nb = grid_for(n, 256, c->num_sms * 4);
    Geo g = geo_of(c);
    KeT<double> Ke = ke_param<double>(c);
    for (outer = 0; !ok && outer < max_outer && total < itmax && std::isfinite(rn); outer++) {
        int it = 0;
        PSF_CHECK(inner_solve(c, solver, r, 1.0 / rn, std::min(inner_cap, itmax - total), inner_tol, &it));
        total += it;
        double zq = 0, pr = 0, pq = 0, rr = 0;
        (fcg_z_kernel<<<nb, 256, 0, c->stream>>>(n, rn, c->w32[5], q, z, c->partials), ::psf::note_launch());
        PSF_CHECK(sum_partials_host(c, nb, &zq));
        const double beta = outer > 0 ? zq / pq_prev : 0.0;
        (fcg_p_kernel<<<nb, 256, 0, c->stream>>>(n, beta, z, r, p, c->partials), ::psf::note_launch());
        PSF_CHECK(sum_partials_host(c, nb, &pr));
        switch (c->kind) {
        case PSF_Q4_PLANE_STRAIN:
            (fcg_q_kernel<0><<<nb, 256, 0, c->stream>>>(
                 g, Ke, c->Epad, c->fixed, p, q, c->partials),
             ::psf::note_launch());
            break;
        case PSF_Q4_HEAT:
            (fcg_q_kernel<1><<<nb, 256, 0, c->stream>>>(
                 g, Ke, c->Epad, c->fixed, p, q, c->partials),
             ::psf::note_launch());
            break;
        default:
            (fcg_q_kernel<2><<<nb, 256, 0, c->stream>>>(
                 g, Ke, c->Epad, c->fixed, p, q, c->partials),
             ::psf::note_launch());
            break;
        }
        PSF_CHECK(sum_partials_host(c, nb, &pq));
        if (!(pq > 0.0)) break;   // direction of no energy: nothing more to gain
        const double alpha = pr / pq;
        (fcg_update_kernel<<<nb, 256, 0, c->stream>>>(n, alpha, p, q, x, r, c->partials), ::psf::note_launch());
        PSF_CHECK(sum_partials_host(c, nb, &rr));
        rn = sqrt(rr);
        pq_prev = pq;
        if (rn <= eps * bn) {
            // confirm on the true residual before stopping
            PSF_CHECK(residual64(c, c->Fn, x, r, &rn, &bn));
            ok = rn <= eps * bn;
        }
    }
    PSF_CUDA(cudaMemcpyAsync(c->un, x, sizeof(double) * n, cudaMemcpyDeviceToDevice, c->stream));
    PSF_CHECK(gather_reduced(c, c->un, c->u));
    inf->iterations = total;
    inf->outer_iterations = outer;
    inf->rel_residual_recurrence = bn > 0 ? rn / bn : 0.0;
    return ok ? PSF_OK : PSF_NOT_CONVERGED;
}

// FP64 Jacobi PCG (matrix-free) from the iterate in x: the learned solver's fallback
psf_status pcg_ebe_fallback(Ctx *c, const double *b, double *x, int itmax, double eps, int *iters, bool *conv) {
    int it = 0, cv = 0;
    double rr = 0.0, bb = 0.0;
    PSF_CHECK(pcg_ebe<double>(c, b, 1.0, x, x, c->w64, itmax, eps, &it, &rr, &bb, &cv));
    *iters = it;
    *conv = cv != 0;
    return PSF_OK;
}

psf_status solve(Ctx *c, int solver, int itmax, double eps, bool warm, psf_solve_info *info) {
    psf_solve_info inf{};
    c->ksec = 0.0;
    c->klaunch = 0;
    PSF_CUDA(cudaEventRecord(c->ev0, c->stream));
    psf_status st = PSF_OK;
    if (solver == PSF_SOLVE_CSR_JACOBI_F64) {
        if (!c->have_values) { set_error("psf_solve: assemble first"); return PSF_BAD_INPUT; }
        int it, conv;
        double rr, bb;
        PSF_CHECK(pcg_csr(c, itmax, eps, &it, &rr, &bb, &conv));
        inf.iterations = it;
        inf.outer_iterations = 1;
        inf.rel_residual_recurrence = bb > 0 ? sqrt(rr / bb) : 0.0;
        PSF_CHECK(scatter_reduced(c, c->u, c->un));
        if (!conv) st = PSF_NOT_CONVERGED;
    } else if (solver == PSF_SOLVE_EBE_JACOBI_F64) {
        int it, conv;
        double rr, bb;
        double *x = c->w64[5];
        PSF_CHECK(pcg_ebe<double>(c, c->Fn, 1.0, warm ? c->un : nullptr, x, c->w64, itmax, eps, &it, &rr, &bb, &conv));
        PSF_CUDA(cudaMemcpyAsync(c->un, x, sizeof(double) * c->ndofs, cudaMemcpyDeviceToDevice, c->stream));
        PSF_CHECK(gather_reduced(c, c->un, c->u));
        inf.iterations = it;
        inf.outer_iterations = 1;
        inf.rel_residual_recurrence = bb > 0 ? sqrt(rr / bb) : 0.0;
        if (!conv) st = PSF_NOT_CONVERGED;
    } else if (solver == PSF_SOLVE_IR_JACOBI_F32) {
        st = outer_fcg64(c, solver, itmax, eps, warm, &inf);
        if (st != PSF_OK && st != PSF_NOT_CONVERGED) return st;
    } else if (solver == PSF_SOLVE_IR_MG_F32) {
        st = mg_solve(c, itmax, eps, warm, &inf);
        if (st != PSF_OK && st != PSF_NOT_CONVERGED) return st;
    } else if (solver == PSF_SOLVE_CSR_BICGSTAB_F64) {
        if (!c->have_values) { set_error("psf_solve: assemble first"); return PSF_BAD_INPUT; }
        int it, conv;
        double rr, bb;
        // six vectors of nfree: five in w64[0] (5 * ndofs long), the sixth in w64[1]
        const long long nf = c->nfree;
        double *const v[6] = {c->w64[0], c->w64[0] + nf, c->w64[0] + 2 * nf, c->w64[0] + 3 * nf,
                              c->w64[0] + 4 * nf, c->w64[1]};
        PSF_CHECK(bicgstab_csr_any(c, nf, c->indptr, c->indices, c->data, c->F, c->u, v, itmax, eps, &it, &rr,
                                   &bb, &conv));
        inf.iterations = it;
        inf.outer_iterations = 1;
        inf.rel_residual_recurrence = bb > 0 ? sqrt(rr / bb) : 0.0;
        PSF_CHECK(scatter_reduced(c, c->u, c->un));
        if (!conv) st = PSF_NOT_CONVERGED;
    } else if (solver == PSF_SOLVE_IR_LEARNED_F32) {
        st = learned_solve(c, itmax, eps, warm, &inf);
        if (st != PSF_OK && st != PSF_NOT_CONVERGED) return st;
    } else {
        set_error("psf_solve: unknown solver");
        return PSF_BAD_INPUT;
    }
    PSF_CUDA(cudaEventRecord(c->ev1, c->stream));
    // FP64 true residual of the returned solution
    double rn, bn;
    PSF_CHECK(residual64(c, c->Fn, c->un, c->w64[6], &rn, &bn));
    inf.rel_residual = bn > 0 ? rn / bn : 0.0;
    float ms = 0.f;
    PSF_CUDA(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
    inf.seconds = ms * 1e-3;
    inf.kernel_seconds = c->ksec;
    inf.kernel_launches = c->klaunch;
    if (info) *info = inf;
    return st;
}

}  // namespace psf
