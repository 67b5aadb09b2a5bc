// psf_batch.cu -- many independent 2D heat-conduction SIMP problems (square Q4
// grids of uneven size, one temperature dof per node, OC update) advanced
// together: each SIMP iteration is four launches over all instances
// (filter + moduli + volume; solve; compliance + sensitivities + filtered
// sensitivities; OC), captured once as a CUDA graph and replayed.
//
// A team owns one instance for the whole phase: one CTA, or the CTAs of a
// thread-block cluster (2, 4 or 8), so every barrier of an instance is a block or
// cluster barrier and every reduction is block-local or a fixed-order sum over
// the team: no grid barrier, no atomics, deterministic.  Instances are launched
// largest first.
// The solve is flexible CG on double-word vectors (FP32 pairs: operator, dot products,
// recurrences at ~1e-14 relative accuracy on the FP32 pipes; one SM's FP64 rate would bound
// the largest instances) whose preconditioner is one FP32 V(2,2) multigrid cycle per
// iteration: degree-2 Chebyshev smoothing on the l1-Jacobi scaled operator (PSF_MG_CHEB as
// for the single-problem solver; <= 1 selects plain l1-Jacobi), Galerkin coarse operators built element by element inside the
// block (P^T K P with bilinear P, fixed nodes masked), 9-point coarse stencils,
// and a dense inverse of the coarsest level (<= 64 nodes) in shared memory.
// The FP64 true residual decides convergence.
//
// Each instance follows the single-problem path of this library for the
// heat-sink configuration (the reference's HeatTransfer element, DensityFilter,
// OC with the filtered-volume callback), so its trajectory matches a psf_ctx run
// of the same problem to the solver tolerance.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <vector>

#include "psf_dw.cuh"
#include "psf_internal.cuh"

namespace psf {
namespace batch {

constexpr int kLev = 10;
constexpr int kCoarseNodes = 64;
constexpr int kMaxStencilB = 49;   // filter stencil entries (radius < 3.5 elements)

struct Inst {
    int n, nlev, nc;
    int pad_;
    long long e0, v0;        // level-0 element / node offsets
    long long me[kLev];      // per-level element offsets (coarse element matrices, levels >= 1)
    long long mv[kLev];      // per-level node offsets (multigrid vectors, all levels)
    long long ainv;          // offset of the coarsest dense inverse
    long long c0;            // offset of the OC bisection's chunk sums (2 sets of ceil(n^2 / kChunk))
    double vf;
};

struct Args {
    int ninst;
    const Inst *inst;
    const int *order;        // block b processes instance order[b]
    // level-0 element arrays
    double *s, *rho, *E, *dfdrho, *dfds, *dgds, *snew, *wsum;
    double *vw;              // volume weight of each design variable: sum over e in N(j) of w_ej / wsum_e
    double *ocs;             // OC bisection chunk sums (per instance at Inst::c0)
    double *Bp;              // per OC call: x_j (-dfdx_j / dgdx_j)^iota
    float *Ef;
    float2 *Ew;              // E as double words (the Krylov operator)
    // level-0 node arrays (Krylov vectors, loads, fixed flags)
    double *x, *r, *p, *q, *F;   // r, p, q hold double words during a solve
    const unsigned char *fixed;
    // multigrid arrays
    float *Kel;              // 16 floats per coarse element
    float *St;               // 9 floats per coarse node
    float *D, *mx, *mb, *mr; // per node, all levels
    unsigned char *mfix;     // per node, all levels (level 0 copies the Dirichlet flags)
    float *Ainv;
    double *out;             // per instance, kOut values
    double *red;             // per instance, 2 x kMaxCluster reduction slots
    // parameters
    double k0, kmin, pexp, iota, lmin, lmax, leps, move, eps;
    int itmax, warm;
    double Ke0[16];
    float Ke0f[16];          // float part of Ke0 (the cycle uses it alone)
    float Ke0lo[16];         // Ke0 - Ke0f: Ke0f + Ke0lo carries 48 bits (double-word operator)
    // smoothing steps of the cycle: d0 = om D^-1 r0, d1 = c2 d0 + c3 D^-1 r1 (x += d each step);
    // degree-2 Chebyshev on [1/ratio, 1] of the l1-scaled operator, or l1-Jacobi (om = c3 = 1, c2 = 0)
    float sm_om, sm_c2, sm_c3;
    int nst;                 // filter stencil
    int sdi[kMaxStencilB], sdj[kMaxStencilB];
    double sw[kMaxStencilB];
};

// per-instance outputs
// O_CONV: the solve reached its residual; O_FPREV: the compliance of the last update;
// O_DONE: IsConvergence held (OC.h:67-73), so the design is no longer updated
enum { O_F = 0, O_G, O_LAMBDA, O_ITERS, O_RES, O_CONV, O_PASSES, O_BISECT, O_FPREV, O_DONE, kOut = 10 };

constexpr int kThreads = 512;

// ------------------------------------------------------------------ block helpers
// block-wide sum, every thread gets the result (fixed tree order)
__device__ __forceinline__ double bsum(double v, double *sm) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    v = warp_sum(v);
    __syncthreads();
    if (lane == 0) sm[wid] = v;
    __syncthreads();
    double t = lane < nw ? sm[lane] : 0.0;
    t = warp_sum(t);
    return t;
}

// ---- the team of an instance: the CTAs of one thread-block cluster (a lone CTA when the
// launch has no clusters).  Loops run over the team's threads, instance-wide barriers are
// cluster barriers (release / acquire at cluster scope), and sums go through per-instance
// slots in global memory, read in rank order: deterministic for a fixed team size.
constexpr int kMaxCluster = 8;

struct Team {
    int rank, size, idx;
    long long tid, nt;
};

__device__ __forceinline__ unsigned cl_rank() {
    unsigned r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}
__device__ __forceinline__ unsigned cl_size() {
    unsigned r;
    asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(r));
    return r;
}
__device__ __forceinline__ void cl_sync() {
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

__device__ __forceinline__ Team team(const Args &A) {
    Team t;
    t.size = (int)cl_size();
    t.rank = (int)cl_rank();
    t.tid = (long long)t.rank * blockDim.x + threadIdx.x;
    t.nt = (long long)t.size * blockDim.x;
    t.idx = A.order[blockIdx.x / t.size];
    return t;
}

__device__ __forceinline__ void tsync(const Team &T) {
    if (T.size > 1) cl_sync();
    else __syncthreads();
}

// team-wide sum; the two slot sets alternate so that a set is rewritten only after a later barrier
__device__ __forceinline__ double tsum(const Args &A, const Team &T, double v, double *sm, int &par) {
    const double b = bsum(v, sm);
    if (T.size == 1) return b;
    double *slot = A.red + ((long long)T.idx * 2 + par) * kMaxCluster;
    if (threadIdx.x == 0) slot[T.rank] = b;
    par ^= 1;
    cl_sync();
    double s = 0.0;
    for (int k = 0; k < T.size; k++) s += __ldcg(slot + k);
    return s;
}

__device__ __forceinline__ int corner(int di, int dj) { return di ? (dj ? 2 : 1) : (dj ? 3 : 0); }

// x^p for the penalty exponent (the samples' p = 3 as products; FP64 pow is slow on one SM)
__device__ __forceinline__ double powp(double x, double p) {
    if (p == 3.0) return x * x * x;
    if (p == 2.0) return x * x;
    if (p == 1.0) return x;
    return pow(x, p);
}

// FP64 operator row of node (i, j) of level 0: y = sum over the 4 surrounding elements of E_e Ke0 x_e
__device__ __forceinline__ double op64(const Args &A, const Inst &I, const double *xv, int i, int j) {
    const int n = I.n;
    double y = 0.0;
#pragma unroll
    for (int ci = 0; ci < 2; ci++)
#pragma unroll
        for (int cj = 0; cj < 2; cj++) {
            const int ei = i - 1 + ci, ej = j - 1 + cj;
            if (ei < 0 || ej < 0 || ei >= n || ej >= n) continue;
            const double Ee = A.E[I.e0 + (long long)n * ei + ej];
            const int li = corner(1 - ci, 1 - cj);
            double acc = 0.0;
#pragma unroll
            for (int lb = 0; lb < 4; lb++) {
                const int bi = ei + (lb == 1 || lb == 2), bj = ej + (lb == 2 || lb == 3);
                acc += A.Ke0[li * 4 + lb] * xv[(long long)(n + 1) * bi + bj];
            }
            y += Ee * acc;
        }
    return y;
}

// the FCG operator row on double words: vector and moduli as FP32 pairs, each element's
// Ke0 x_e a compensated dot product (Dot2 with the low-order products folded in), the E_e
// scaling and the node sum in double words; nothing on the FP64 pipe
__device__ __forceinline__ dw::D opdw(const Args &A, const Inst &I, const float2 *xv, int i, int j) {
    const int n = I.n;
    dw::D y = dw::from_float(0.f);
#pragma unroll
    for (int ci = 0; ci < 2; ci++)
#pragma unroll
        for (int cj = 0; cj < 2; cj++) {
            const int ei = i - 1 + ci, ej = j - 1 + cj;
            if (ei < 0 || ej < 0 || ei >= n || ej >= n) continue;
            const float2 Ev = A.Ew[I.e0 + (long long)n * ei + ej];
            const int li = corner(1 - ci, 1 - cj);
            float ps = 0.0f, cs = 0.0f;
#pragma unroll
            for (int lb = 0; lb < 4; lb++) {
                const int bi = ei + (lb == 1 || lb == 2), bj = ej + (lb == 2 || lb == 3);
                const float2 u = xv[(long long)(n + 1) * bi + bj];
                const float kh = A.Ke0f[li * 4 + lb], kl = A.Ke0lo[li * 4 + lb];
                float pe, se;
                const float pr = dw::two_prod(kh, u.x, pe);
                ps = dw::two_sum(ps, pr, se);
                cs += se + pe + __fmaf_rn(kh, u.y, kl * u.x);
            }
            float sl;
            const float sh = dw::fast_two_sum(ps, cs, sl);
            y = dw::add(y, dw::mul(dw::make(Ev.x, Ev.y), dw::make(sh, sl)));
        }
    return y;
}

// FP32 operator row of node (i, j) at level l (level 0: element by element, else the 9-point stencil)
__device__ __forceinline__ float opl(const Args &A, const Inst &I, int l, const float *xv, int i, int j) {
    const int m = I.n >> l;
    if (l == 0) {
        float y = 0.0f;
#pragma unroll
        for (int ci = 0; ci < 2; ci++)
#pragma unroll
            for (int cj = 0; cj < 2; cj++) {
                const int ei = i - 1 + ci, ej = j - 1 + cj;
                if (ei < 0 || ej < 0 || ei >= m || ej >= m) continue;
                const float Ee = A.Ef[I.e0 + (long long)m * ei + ej];
                const int li = corner(1 - ci, 1 - cj);
                float acc = 0.0f;
#pragma unroll
                for (int lb = 0; lb < 4; lb++) {
                    const int bi = ei + (lb == 1 || lb == 2), bj = ej + (lb == 2 || lb == 3);
                    acc += A.Ke0f[li * 4 + lb] * xv[(long long)(m + 1) * bi + bj];
                }
                y += Ee * acc;
            }
        return y;
    }
    const float *st = A.St + (I.mv[l] + (long long)(m + 1) * i + j) * 9;
    float y = 0.0f;
#pragma unroll
    for (int di = -1; di <= 1; di++)
#pragma unroll
        for (int dj = -1; dj <= 1; dj++) {
            const int a = i + di, b = j + dj;
            if (a < 0 || b < 0 || a > m || b > m) continue;
            y += st[(di + 1) * 3 + (dj + 1)] * xv[(long long)(m + 1) * a + b];
        }
    return y;
}

// ------------------------------------------------------------------ multigrid setup (inside the block)
__device__ void mg_setup(const Args &A, const Team &T, const Inst &I, double *sm) {
    const long long tid = T.tid, nt = T.nt;
    // level 0: l1 row sums (E >= 0) and the fixed flags
    {
        const int m = I.n;
        const long long nn = (long long)(m + 1) * (m + 1);
        for (long long v = tid; v < nn; v += nt) {
            const int i = (int)(v / (m + 1)), j = (int)(v % (m + 1));
            const bool fx = A.fixed[I.v0 + v];
            A.mfix[I.mv[0] + v] = fx;
            float d = 0.0f;
            for (int ci = 0; ci < 2; ci++)
                for (int cj = 0; cj < 2; cj++) {
                    const int ei = i - 1 + ci, ej = j - 1 + cj;
                    if (ei < 0 || ej < 0 || ei >= m || ej >= m) continue;
                    const int li = corner(1 - ci, 1 - cj);
                    float a = 0.0f;
                    for (int lb = 0; lb < 4; lb++) a += fabsf(A.Ke0f[li * 4 + lb]);
                    d += A.Ef[I.e0 + (long long)m * ei + ej] * a;
                }
            A.D[I.mv[0] + v] = fx ? 1.0f : d;
        }
    }
    tsync(T);
    for (int l = 1; l < I.nlev; l++) {
        const int mf = I.n >> (l - 1), mc = I.n >> l;
        const long long nnc = (long long)(mc + 1) * (mc + 1);
        // coarse fixed flags: a coarse node is fixed when the coincident fine node is
        for (long long v = tid; v < nnc; v += nt) {
            const int i = (int)(v / (mc + 1)), j = (int)(v % (mc + 1));
            A.mfix[I.mv[l] + v] = A.mfix[I.mv[l - 1] + (long long)(mf + 1) * (2 * i) + 2 * j];
        }
        tsync(T);
        // Galerkin element matrices: Kc = sum over the 4 fine children of P_f^T K_f P_f
        const long long nec = (long long)mc * mc;
        for (long long e = tid; e < nec; e += nt) {
            const int ci = (int)(e / mc), cj = (int)(e % mc);
            float Kc[16];
#pragma unroll
            for (int q = 0; q < 16; q++) Kc[q] = 0.0f;
            bool cfix[4];
#pragma unroll
            for (int a = 0; a < 4; a++) {
                const int ai = ci + (a == 1 || a == 2), aj = cj + (a == 2 || a == 3);
                cfix[a] = A.mfix[I.mv[l] + (long long)(mc + 1) * ai + aj];
            }
#pragma unroll
            for (int f = 0; f < 4; f++) {
                const int fx = f & 1, fy = f >> 1;
                const int fi = 2 * ci + fx, fj = 2 * cj + fy;   // fine element
                float Kf[16];
                if (l == 1) {
                    const float Ee = A.Ef[I.e0 + (long long)mf * fi + fj];
#pragma unroll
                    for (int q = 0; q < 16; q++) Kf[q] = Ee * A.Ke0f[q];
                } else {
                    const float *src = A.Kel + (I.me[l - 1] + (long long)mf * fi + fj) * 16;
#pragma unroll
                    for (int q = 0; q < 16; q++) Kf[q] = src[q];
                }
                // P_f[lf][a]: weight of coarse node a at the fine element's local node lf
                float P[16];
#pragma unroll
                for (int lf = 0; lf < 4; lf++) {
                    const int x = fx + (lf == 1 || lf == 2), y = fy + (lf == 2 || lf == 3);   // 0..2 in the coarse element
                    const bool ffix = A.mfix[I.mv[l - 1] + (long long)(mf + 1) * (2 * ci + x) + (2 * cj + y)];
#pragma unroll
                    for (int a = 0; a < 4; a++) {
                        const int ax = (a == 1 || a == 2), ay = (a == 2 || a == 3);
                        const float wx = 1.0f - 0.5f * fabsf((float)(x - 2 * ax));
                        const float wy = 1.0f - 0.5f * fabsf((float)(y - 2 * ay));
                        P[lf * 4 + a] = (ffix || cfix[a] || wx <= 0.0f || wy <= 0.0f) ? 0.0f : wx * wy;
                    }
                }
                float Q[16];   // K_f P
#pragma unroll
                for (int r = 0; r < 4; r++)
#pragma unroll
                    for (int b = 0; b < 4; b++) {
                        float t = 0.0f;
#pragma unroll
                        for (int k = 0; k < 4; k++) t += Kf[r * 4 + k] * P[k * 4 + b];
                        Q[r * 4 + b] = t;
                    }
#pragma unroll
                for (int a = 0; a < 4; a++)
#pragma unroll
                    for (int b = 0; b < 4; b++) {
                        float t = 0.0f;
#pragma unroll
                        for (int k = 0; k < 4; k++) t += P[k * 4 + a] * Q[k * 4 + b];
                        Kc[a * 4 + b] += t;
                    }
            }
            float *dst = A.Kel + (I.me[l] + e) * 16;
#pragma unroll
            for (int q = 0; q < 16; q++) dst[q] = Kc[q];
        }
        tsync(T);
        // 9-point stencils and l1 diagonals (identity rows on fixed nodes)
        for (long long v = tid; v < nnc; v += nt) {
            const int i = (int)(v / (mc + 1)), j = (int)(v % (mc + 1));
            float st[9];
#pragma unroll
            for (int q = 0; q < 9; q++) st[q] = 0.0f;
            const bool fx = A.mfix[I.mv[l] + v];
            if (fx) {
                st[4] = 1.0f;
            } else {
                for (int ci = 0; ci < 2; ci++)
                    for (int cj = 0; cj < 2; cj++) {
                        const int ei = i - 1 + ci, ej = j - 1 + cj;
                        if (ei < 0 || ej < 0 || ei >= mc || ej >= mc) continue;
                        const float *K = A.Kel + (I.me[l] + (long long)mc * ei + ej) * 16;
                        const int li = corner(1 - ci, 1 - cj);
                        for (int lb = 0; lb < 4; lb++) {
                            const int bi = ei + (lb == 1 || lb == 2) - i, bj = ej + (lb == 2 || lb == 3) - j;
                            st[(bi + 1) * 3 + (bj + 1)] += K[li * 4 + lb];
                        }
                    }
            }
            float d = 0.0f;
#pragma unroll
            for (int q = 0; q < 9; q++) d += fabsf(st[q]);
            float *dst = A.St + (I.mv[l] + v) * 9;
#pragma unroll
            for (int q = 0; q < 9; q++) dst[q] = st[q];
            A.D[I.mv[l] + v] = d > 0.0f ? d : 1.0f;
        }
        tsync(T);
    }
    // coarsest level: dense matrix from the stencils, Gauss-Jordan inverse in the shared memory of
    // the team's first CTA (FP64)
    if (T.rank == 0) {
        const int btid = threadIdx.x, bnt = blockDim.x;
        const int l = I.nlev - 1, mc = I.n >> l, nc = I.nc;
        double *M = sm;   // nc x 2nc
        for (int t = btid; t < nc * 2 * nc; t += bnt) M[t] = 0.0;
        __syncthreads();
        for (int v = btid; v < nc; v += bnt) {
            const int i = v / (mc + 1), j = v % (mc + 1);
            const float *st = A.St + (I.mv[l] + v) * 9;
            for (int di = -1; di <= 1; di++)
                for (int dj = -1; dj <= 1; dj++) {
                    const int a = i + di, b = j + dj;
                    if (a < 0 || b < 0 || a > mc || b > mc) continue;
                    M[v * 2 * nc + (mc + 1) * a + b] = st[(di + 1) * 3 + (dj + 1)];
                }
            M[v * 2 * nc + nc + v] = 1.0;
        }
        __syncthreads();
        double *fcol = M + (size_t)nc * 2 * nc;   // column k of the other rows, read before the update
        for (int k = 0; k < nc; k++) {
            // the coarse operator is SPD (fixed rows identity): no pivoting
            const double piv = M[k * 2 * nc + k];
            __syncthreads();
            for (int c = btid; c < 2 * nc; c += bnt) M[k * 2 * nc + c] /= piv;
            for (int r = btid; r < nc; r += bnt) fcol[r] = (r == k) ? 0.0 : M[r * 2 * nc + k];
            __syncthreads();
            for (int t = btid; t < nc * 2 * nc; t += bnt) {
                const int r = t / (2 * nc), c = t % (2 * nc);
                if (r != k) M[t] -= fcol[r] * M[k * 2 * nc + c];
            }
            __syncthreads();
        }
        for (int t = btid; t < nc * nc; t += bnt) A.Ainv[I.ainv + t] = (float)M[(t / nc) * 2 * nc + nc + (t % nc)];
    }
    tsync(T);
}

// ------------------------------------------------------------------ the V(2,2) cycle (FP32)
// smoothing step `step` (0 or 1) on level l; the correction d is kept in mr between the steps
__device__ void smooth_step(const Args &A, const Team &T, const Inst &I, int l, int step) {
    const int m = I.n >> l;
    const long long tid = T.tid, nt = T.nt;
    const long long nn = (long long)(m + 1) * (m + 1);
    const float *x = A.mx + I.mv[l];
    float *t = A.mr + I.mv[l];
    const float *b = A.mb + I.mv[l];
    const float c2 = step ? A.sm_c2 : 0.0f, c3 = step ? A.sm_c3 : A.sm_om;
    for (long long v = tid; v < nn; v += nt) {
        const int i = (int)(v / (m + 1)), j = (int)(v % (m + 1));
        const float dprev = step ? t[v] : 0.0f;
        t[v] = A.mfix[I.mv[l] + v] ? 0.0f : c2 * dprev + c3 * (b[v] - opl(A, I, l, x, i, j)) / A.D[I.mv[l] + v];
    }
    tsync(T);
    float *xw = A.mx + I.mv[l];
    for (long long v = tid; v < nn; v += nt) xw[v] += t[v];
    tsync(T);
}

__device__ void vcycle(const Args &A, const Team &T, const Inst &I) {
    const long long tid = T.tid, nt = T.nt;
    for (int l = 0; l < I.nlev - 1; l++) {
        smooth_step(A, T, I, l, 0);
        smooth_step(A, T, I, l, 1);
        // residual into mr
        const int m = I.n >> l;
        const long long nn = (long long)(m + 1) * (m + 1);
        {
            const float *x = A.mx + I.mv[l], *b = A.mb + I.mv[l];
            float *r = A.mr + I.mv[l];
            for (long long v = tid; v < nn; v += nt) {
                const int i = (int)(v / (m + 1)), j = (int)(v % (m + 1));
                r[v] = A.mfix[I.mv[l] + v] ? 0.0f : b[v] - opl(A, I, l, x, i, j);
            }
        }
        tsync(T);
        // restriction (P^T, fixed nodes masked) and the first sweep of the coarse level from zero
        const int mc = m >> 1;
        const long long nnc = (long long)(mc + 1) * (mc + 1);
        const float *r = A.mr + I.mv[l];
        for (long long v = tid; v < nnc; v += nt) {
            const int I2 = (int)(v / (mc + 1)), J2 = (int)(v % (mc + 1));
            float acc = 0.0f;
            if (!A.mfix[I.mv[l + 1] + v]) {
                for (int dx = -1; dx <= 1; dx++)
                    for (int dy = -1; dy <= 1; dy++) {
                        const int fi = 2 * I2 + dx, fj = 2 * J2 + dy;
                        if (fi < 0 || fj < 0 || fi > m || fj > m) continue;
                        const float w = (dx ? 0.5f : 1.0f) * (dy ? 0.5f : 1.0f);
                        acc += w * r[(long long)(m + 1) * fi + fj];   // r is zero on fixed fine nodes
                    }
            }
            A.mb[I.mv[l + 1] + v] = acc;
            A.mx[I.mv[l + 1] + v] = 0.0f;
        }
        tsync(T);
    }
    // coarsest: x = Ainv b
    {
        const int l = I.nlev - 1, nc = I.nc;
        const float *Ai = A.Ainv + I.ainv, *b = A.mb + I.mv[l];
        for (long long v = tid; v < nc; v += nt) {
            float acc = 0.0f;
            for (int c = 0; c < nc; c++) acc += Ai[v * nc + c] * b[c];
            A.mx[I.mv[l] + v] = acc;
        }
        tsync(T);
    }
    for (int l = I.nlev - 2; l >= 0; l--) {
        const int m = I.n >> l, mc = m >> 1;
        const long long nn = (long long)(m + 1) * (m + 1);
        const float *xc = A.mx + I.mv[l + 1];
        float *x = A.mx + I.mv[l];
        for (long long v = tid; v < nn; v += nt) {
            if (A.mfix[I.mv[l] + v]) continue;
            const int i = (int)(v / (m + 1)), j = (int)(v % (m + 1));
            const int i0 = i >> 1, j0 = j >> 1, i1 = (i + 1) >> 1, j1 = (j + 1) >> 1;
            const float c = 0.25f * (xc[(long long)(mc + 1) * i0 + j0] + xc[(long long)(mc + 1) * i0 + j1] +
                                     xc[(long long)(mc + 1) * i1 + j0] + xc[(long long)(mc + 1) * i1 + j1]);
            x[v] += c;
        }
        tsync(T);
        smooth_step(A, T, I, l, 0);
        smooth_step(A, T, I, l, 1);
    }
}

// ------------------------------------------------------------------ phase kernels

__device__ __forceinline__ double filt(const Args &A, const Inst &I, const double *v, int i, int j) {
    const int n = I.n;
    double s = 0.0;
    for (int q = 0; q < A.nst; q++) {
        const int a = i + A.sdi[q], b = j + A.sdj[q];
        if (a < 0 || b < 0 || a >= n || b >= n) continue;
        s += A.sw[q] * v[(long long)n * a + b];
    }
    return s;
}

// rho = filter(s), E = kmin + (k0 - kmin) rho^p, g = sum(rho) / (vf n^2) - 1
// a converged instance (IsConvergence held at an earlier update) keeps its design and its
// fields, as the samples leave their loop: every phase returns at once for it
__device__ __forceinline__ bool frozen(const Args &A, int idx) { return A.out[(long long)idx * kOut + O_DONE] != 0.0; }

__global__ void __launch_bounds__(kThreads) filter_moduli_batch(const __grid_constant__ Args A) {
    __shared__ double sm[32];
    const Team T = team(A);
    if (frozen(A, T.idx)) return;
    const Inst &I = A.inst[T.idx];
    int par = 0;
    const int n = I.n;
    const long long ne = (long long)n * n;
    const double *s = A.s + I.e0;
    double vol = 0.0;
    for (long long e = T.tid; e < ne; e += T.nt) {
        const int i = (int)(e / n), j = (int)(e % n);
        const double r = filt(A, I, s, i, j) / A.wsum[I.e0 + e];
        A.rho[I.e0 + e] = r;
        const double rp = powp(r, A.pexp);
        const double Ee = A.k0 * rp + A.kmin * (1.0 - rp);
        A.E[I.e0 + e] = Ee;
        A.Ef[I.e0 + e] = (float)Ee;
        const dw::D Ed = dw::from_double(Ee);
        A.Ew[I.e0 + e] = make_float2(Ed.h, Ed.l);
        vol += r;
    }
    vol = tsum(A, T, vol, sm, par);
    if (T.tid == 0) A.out[(long long)T.idx * kOut + O_G] = vol / (I.vf * (double)ne) - 1.0;
}

// flexible CG on double-word vectors with one FP32 V-cycle per iteration; FP64 true residual checks
__global__ void __launch_bounds__(kThreads) solve_batch(const __grid_constant__ Args A) {
    extern __shared__ double dyn[];
    double *sm = dyn;            // 32 doubles of reduction space, then the coarse inverse workspace
    const Team T = team(A);
    if (frozen(A, T.idx)) return;
    const Inst &I = A.inst[T.idx];
    int par = 0;
    const int idx = T.idx;
    const int n = I.n;
    const long long tid = T.tid, nt = T.nt;
    const long long nn = (long long)(n + 1) * (n + 1);
    double *x = A.x + I.v0;
    // the Krylov vectors live in the FP64 arrays' memory as double words (FP32 pairs):
    // x, r, p, q; the solution returns to FP64 (in place) for every true residual
    float2 *X = (float2 *)(A.x + I.v0), *R = (float2 *)(A.r + I.v0), *P = (float2 *)(A.p + I.v0),
           *Q = (float2 *)(A.q + I.v0);
    auto ld = [](const float2 *a, long long t) { const float2 v = a[t]; return dw::make(v.x, v.y); };
    auto st = [](float2 *a, long long t, dw::D v) { a[t] = make_float2(v.h, v.l); };
    const double *F = A.F + I.v0;
    const unsigned char *fx = A.fixed + I.v0;
    mg_setup(A, T, I, sm + 32);
    int total = 0, passes = 0;
    bool conv = false;
    double rr = 0.0, bb = 0.0;
    for (int pass = 0; pass < 3 && total < A.itmax && !conv; pass++) {
        passes++;
        // r = F - K x in FP64 (x = 0 on the first pass unless warm), then x to double words
        double acc[2] = {0.0, 0.0};
        for (long long v = tid; v < nn; v += nt) {
            if (pass == 0 && !A.warm) x[v] = 0.0;
        }
        tsync(T);
        for (long long v = tid; v < nn; v += nt) {
            const int i = (int)(v / (n + 1)), j = (int)(v % (n + 1));
            const double bv = fx[v] ? 0.0 : F[v];
            const double rv = fx[v] ? 0.0 : bv - op64(A, I, x, i, j);
            st(R, v, dw::from_double(rv));
            st(P, v, dw::from_float(0.f));
            st(Q, v, dw::from_float(0.f));
            acc[0] += rv * rv;
            acc[1] += bv * bv;
        }
        rr = tsum(A, T, acc[0], sm, par);
        bb = tsum(A, T, acc[1], sm, par);   // a team barrier: every neighbour read of x is done
        for (long long v = tid; v < nn; v += nt) st(X, v, dw::from_double(x[v]));   // in place, own entries
        if (bb == 0.0 || rr <= A.eps * A.eps * bb) {
            conv = true;
            for (long long v = tid; v < nn; v += nt) x[v] = dw::to_double(ld(X, v));
            break;
        }
        double pq_prev = 1.0;
        for (int it = 0; total < A.itmax; it++) {
            total++;
            // z = |r| V(r / |r|)
            const double rn = sqrt(rr);
            const float sc = (float)(1.0 / rn);
            for (long long v = tid; v < nn; v += nt) {
                const float2 rv = R[v];
                const float bv = fx[v] ? 0.0f : rv.x * sc + rv.y * sc;
                A.mb[I.mv[0] + v] = bv;
                A.mx[I.mv[0] + v] = fx[v] ? 0.0f : bv / A.D[I.mv[0] + v];
            }
            tsync(T);
            vcycle(A, T, I);
            const dw::D rnD = dw::from_double(rn);
            dw::D a3[3] = {dw::from_float(0.f), dw::from_float(0.f), dw::from_float(0.f)};
            for (long long v = tid; v < nn; v += nt) {
                const dw::D zv = fx[v] ? dw::from_float(0.f) : dw::mulf(rnD, A.mx[I.mv[0] + v]);
                a3[0] = dw::add(a3[0], dw::mul(zv, ld(Q, v)));
                a3[1] = dw::add(a3[1], dw::mul(zv, ld(R, v)));
                a3[2] = dw::add(a3[2], dw::mul(ld(P, v), ld(R, v)));
            }
            const double zq = tsum(A, T, dw::to_double(a3[0]), sm, par),
                         zr = tsum(A, T, dw::to_double(a3[1]), sm, par),
                         pr0 = tsum(A, T, dw::to_double(a3[2]), sm, par);
            const double beta = it > 0 ? zq / pq_prev : 0.0;
            const double pr = zr - beta * pr0;
            const dw::D betaD = dw::from_double(beta);
            for (long long v = tid; v < nn; v += nt) {
                const dw::D zv = fx[v] ? dw::from_float(0.f) : dw::mulf(rnD, A.mx[I.mv[0] + v]);
                st(P, v, dw::sub(zv, dw::mul(betaD, ld(P, v))));
            }
            tsync(T);
            dw::D pqa = dw::from_float(0.f);
            for (long long v = tid; v < nn; v += nt) {
                const int i = (int)(v / (n + 1)), j = (int)(v % (n + 1));
                const dw::D qv = fx[v] ? dw::from_float(0.f) : opdw(A, I, P, i, j);
                st(Q, v, qv);
                pqa = dw::add(pqa, dw::mul(ld(P, v), qv));
            }
            const double pq = tsum(A, T, dw::to_double(pqa), sm, par);
            if (!(pq > 0.0)) break;
            const dw::D alphaD = dw::from_double(pr / pq);
            dw::D ra = dw::from_float(0.f);
            for (long long v = tid; v < nn; v += nt) {
                st(X, v, dw::add(ld(X, v), dw::mul(alphaD, ld(P, v))));
                const dw::D rv = dw::sub(ld(R, v), dw::mul(alphaD, ld(Q, v)));
                st(R, v, rv);
                ra = dw::add(ra, dw::sq(rv));
            }
            rr = tsum(A, T, dw::to_double(ra), sm, par);
            pq_prev = pq;
            if (rr <= A.eps * A.eps * bb || !isfinite(rr)) break;
        }
        // x back to FP64 (own entries), then the FP64 true residual
        for (long long v = tid; v < nn; v += nt) x[v] = dw::to_double(ld(X, v));
        tsync(T);
        double ta = 0.0;
        for (long long v = tid; v < nn; v += nt) {
            const int i = (int)(v / (n + 1)), j = (int)(v % (n + 1));
            const double rv = fx[v] ? 0.0 : F[v] - op64(A, I, x, i, j);
            ta += rv * rv;
        }
        rr = tsum(A, T, ta, sm, par);
        conv = rr <= A.eps * A.eps * bb;
    }
    if (T.tid == 0) {
        double *o = A.out + (long long)idx * kOut;
        o[O_ITERS] = total;
        o[O_RES] = bb > 0.0 ? sqrt(rr / bb) : 0.0;
        o[O_CONV] = conv ? 1.0 : 0.0;
        o[O_PASSES] = passes;
    }
}

// f = sum_e E_e T_e.Ke0 T_e; dfdrho = -p (k0 - kmin) rho^(p-1) T_e.Ke0 T_e; filtered sensitivities
__global__ void __launch_bounds__(kThreads) sens_batch(const __grid_constant__ Args A) {
    __shared__ double sm[32];
    const Team T = team(A);
    if (frozen(A, T.idx)) return;
    const Inst &I = A.inst[T.idx];
    int par = 0;
    const int n = I.n;
    const long long ne = (long long)n * n;
    const double *Tv = A.x + I.v0;
    double f = 0.0;
    for (long long e = T.tid; e < ne; e += T.nt) {
        const int i = (int)(e / n), j = (int)(e % n);
        double te[4];
#pragma unroll
        for (int a = 0; a < 4; a++)
            te[a] = Tv[(long long)(n + 1) * (i + (a == 1 || a == 2)) + (j + (a == 2 || a == 3))];
        double qv = 0.0;
#pragma unroll
        for (int a = 0; a < 4; a++) {
            double v = 0.0;
#pragma unroll
            for (int b = 0; b < 4; b++) v += A.Ke0[a * 4 + b] * te[b];
            qv += te[a] * v;
        }
        A.dfdrho[I.e0 + e] = -A.pexp * (-A.kmin + A.k0) * powp(A.rho[I.e0 + e], A.pexp - 1.0) * qv;
        f += A.E[I.e0 + e] * qv;
    }
    f = tsum(A, T, f, sm, par);
    if (T.tid == 0) A.out[(long long)T.idx * kOut + O_F] = f;
    tsync(T);
    const double dg = 1.0 / (I.vf * (double)ne);
    for (long long e = T.tid; e < ne; e += T.nt) {
        const int i = (int)(e / n), j = (int)(e % n);
        const double w = A.wsum[I.e0 + e];
        A.dfds[I.e0 + e] = filt(A, I, A.dfdrho + I.e0, i, j) / w;
        double sw = 0.0;
        for (int q = 0; q < A.nst; q++) {
            const int a = i + A.sdi[q], b = j + A.sdj[q];
            if (a < 0 || b < 0 || a >= n || b >= n) continue;
            sw += A.sw[q] * dg;
        }
        A.dgds[I.e0 + e] = sw / w;
    }
}

// OC (OC.h:76-107) with the samples' filtered-volume constraint, bisection inside the team.
// The trial design x (-dfdx / (dgdx lambda))^iota is formed as [x (-dfdx / dgdx)^iota] lambda^-iota,
// so the per-element power is taken once per update and a bisection step costs a multiplication
// and a clamp per element; the filtered volume sum_e (sum_j w_ej x_j) / wsum_e is sum_j vw_j x_j
// with the weights vw precomputed.  The volume is summed in the canonical chunk order
// (psf_common.cuh), and the element arithmetic is the single-problem OC kernel's (psf_opt.cu
// oc_fact_kernel): both paths take the same bisection branches on the same inputs, whatever
// the team size.
__global__ void __launch_bounds__(kThreads) oc_batch(const __grid_constant__ Args A) {
    __shared__ double s_tot;
    const Team T = team(A);
    const Inst &I = A.inst[T.idx];
    // IsConvergence (OC.h:67-73) before the update, as the samples test it (sample :188-191): a
    // converged instance keeps its design (the samples leave their loop there)
    {
        double *o = A.out + (long long)T.idx * kOut;
        const double f = o[O_F], fp = o[O_FPREV];
        if (o[O_DONE] != 0.0 || fabs(f - fp) / (f + fp) < 1.0e-5) {
            if (T.tid == 0) o[O_DONE] = 1.0;
            return;
        }
    }
    const int n = I.n;
    const long long ne = (long long)n * n;
    const long long nc = (ne + kChunk - 1) / kChunk;
    const int lane = threadIdx.x & 31;
    const long long gw = T.tid >> 5, nw = T.nt >> 5;
    double *x = A.s + I.e0, *xn = A.snew + I.e0, *Bp = A.Bp + I.e0;
    const double *dfdx = A.dfds + I.e0, *dgdx = A.dgds + I.e0, *vw = A.vw + I.e0;
    for (long long c = gw; c < nc; c += nw)
        for (long long e = c * kChunk + lane; e < ne && e < (c + 1) * kChunk; e += 32) {
            const double b = -dfdx[e] / dgdx[e];
            Bp[e] = x[e] * (A.iota == 0.5 ? sqrt(b) : pow(b, A.iota));
        }
    const double vscale = 1.0 / (I.vf * (double)ne);
    double l0 = A.lmin, l1 = A.lmax, lambda = 0.0;
    int steps = 0;
    while ((l1 - l0) / (l1 + l0) > A.leps && steps < 4000) {
        lambda = 0.5 * (l1 + l0);
        double *cs = A.ocs + I.c0 + (steps & 1) * nc;
        steps++;
        const double li = A.iota == 0.5 ? 1.0 / sqrt(lambda) : pow(lambda, -A.iota);
        for (long long c = gw; c < nc; c += nw) {
            double acc = 0.0;
            for (long long e = c * kChunk + lane; e < ne && e < (c + 1) * kChunk; e += 32) {
                const double xe = x[e];
                double v = Bp[e] * li;
                const double lo0 = (1.0 - A.move) * xe, hi0 = (1.0 + A.move) * xe;
                const double lo = (0.0 < lo0) ? lo0 : 0.0;
                const double hi = (hi0 < 1.0) ? hi0 : 1.0;
                if (v < lo) v = lo;
                else if (v > hi) v = hi;
                xn[e] = v;
                acc += vw[e] * v;
            }
            acc = warp_xor_sum(acc);
            if (lane == 0) cs[c] = acc;
        }
        tsync(T);
        if (threadIdx.x < 32) {
            const double tot = warp_canonical_sum(cs, nc);
            if (threadIdx.x == 0) s_tot = tot;
        }
        __syncthreads();
        const double g = s_tot * vscale - 1.0;
        if (g > 0.0) l0 = lambda;
        else l1 = lambda;
        __syncthreads();   // s_tot is rewritten by the next step
    }
    for (long long c = gw; c < nc; c += nw)
        for (long long e = c * kChunk + lane; e < ne && e < (c + 1) * kChunk; e += 32) x[e] = xn[e];
    if (T.tid == 0) {
        double *o = A.out + (long long)T.idx * kOut;
        o[O_LAMBDA] = lambda;
        o[O_BISECT] = steps;
        o[O_FPREV] = o[O_F];
    }
}

}  // namespace batch
}  // namespace psf

// ------------------------------------------------------------------ host
using psf::batch::Args;
using psf::batch::Inst;

struct psf_batch {
    int ninst = 0;
    std::vector<Inst> hinst;
    std::vector<int> order;
    Args a{};
    size_t ne_tot = 0, nv_tot = 0, mg_nodes = 0, mg_elems = 0, ainv_tot = 0;
    size_t smem = 0;
    int threads = psf::batch::kThreads;
    int cluster = 1;
    cudaStream_t stream = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    size_t graph_nodes = 0;   // kernel nodes of one iteration's graph
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    std::vector<void *> allocs;
    std::vector<double> hout;
    bool begun = false;
};

namespace {

template <class T>
psf_status balloc(psf_batch *b, T **p, size_t n) {
    void *q = nullptr;
    cudaError_t e = cudaMalloc(&q, std::max<size_t>(n, 1) * sizeof(T));
    if (e != cudaSuccess) return psf::cuda_status(e, "cudaMalloc (batch)");
    b->allocs.push_back(q);
    *p = reinterpret_cast<T *>(q);
    return PSF_OK;
}

void batch_free(psf_batch *b) {
    if (!b) return;
    if (b->stream) cudaStreamSynchronize(b->stream);
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    for (void *p : b->allocs) cudaFree(p);
    if (b->ev0) cudaEventDestroy(b->ev0);
    if (b->ev1) cudaEventDestroy(b->ev1);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
}

// one phase over all instances: a team of `cluster` CTAs per instance
cudaError_t launch_phase(psf_batch *b, void (*kern)(Args), size_t smem) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(b->ninst * b->cluster));
    cfg.blockDim = dim3((unsigned)b->threads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = b->stream;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = (unsigned)b->cluster;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = b->cluster > 1 ? 1 : 0;
    ::psf::note_launch();
    return cudaLaunchKernelEx(&cfg, kern, b->a);
}

psf_status launch_phases(psf_batch *b) {
    PSF_CUDA(launch_phase(b, psf::batch::filter_moduli_batch, 0));
    PSF_CUDA(launch_phase(b, psf::batch::solve_batch, b->smem));
    PSF_CUDA(launch_phase(b, psf::batch::sens_batch, 0));
    PSF_CUDA(launch_phase(b, psf::batch::oc_batch, 0));
    return PSF_OK;
}

}  // namespace

extern "C" {

psf_status psf_batch_create(int ninst, const int *side, const int *edge, const int *patch_w, const int *patch_i0,
                            const double *vf, int threads, int cluster, psf_batch **out) {
    if (!out || ninst < 1 || !side || !edge || !patch_w || !patch_i0 || !vf) return PSF_BAD_INPUT;
    if (cluster != 1 && cluster != 2 && cluster != 4 && cluster != psf::batch::kMaxCluster) {
        psf::set_error("psf_batch_create: cluster must be 1, 2, 4 or 8");
        return PSF_BAD_INPUT;
    }
    if (threads != 128 && threads != 256 && threads != psf::batch::kThreads) {
        psf::set_error("psf_batch_create: threads must be 128, 256 or 512 (the kernels' launch bound)");
        return PSF_BAD_INPUT;
    }
    *out = nullptr;
    for (int i = 0; i < ninst; i++)
        if (side[i] < 4 || side[i] % 2 || edge[i] < 0 || edge[i] > 3 || patch_w[i] < 1 || patch_i0[i] < 0 ||
            patch_i0[i] + patch_w[i] > side[i] || !(vf[i] > 0.0 && vf[i] <= 1.0)) {
            psf::set_error("psf_batch_create: invalid instance (even side >= 4, patch inside the edge, 0 < vf <= 1)");
            return PSF_BAD_INPUT;
        }
    psf_batch *b = new psf_batch();
    b->ninst = ninst;
    b->threads = threads;
    b->cluster = cluster;
    b->hinst.resize(ninst);
    size_t ne = 0, nv = 0, mgn = 0, mge = 0, ai = 0, ocs = 0;
    int ncmax = 0;
    for (int k = 0; k < ninst; k++) {
        Inst &I = b->hinst[k];
        std::memset(&I, 0, sizeof(Inst));
        I.n = side[k];
        I.vf = vf[k];
        I.e0 = (long long)ne;
        I.v0 = (long long)nv;
        ne += (size_t)I.n * I.n;
        nv += (size_t)(I.n + 1) * (I.n + 1);
        int l = 0, m = I.n;
        I.mv[0] = (long long)mgn;
        mgn += (size_t)(m + 1) * (m + 1);
        while (l + 1 < psf::batch::kLev && (m + 1) * (m + 1) > psf::batch::kCoarseNodes && m % 2 == 0 && m >= 4) {
            l++;
            m /= 2;
            I.mv[l] = (long long)mgn;
            mgn += (size_t)(m + 1) * (m + 1);
            I.me[l] = (long long)mge;
            mge += (size_t)m * m;
        }
        I.nlev = l + 1;
        I.nc = (m + 1) * (m + 1);
        if (I.nc > psf::batch::kCoarseNodes) {
            delete b;
            psf::set_error("psf_batch_create: a side does not coarsen to <= 64 nodes (use sides with a large power of 2)");
            return PSF_BAD_INPUT;
        }
        if (I.nlev < 2) {
            delete b;
            psf::set_error("psf_batch_create: side too small for a coarse level");
            return PSF_BAD_INPUT;
        }
        I.ainv = (long long)ai;
        ai += (size_t)I.nc * I.nc;
        I.c0 = (long long)ocs;
        ocs += 2 * (((size_t)I.n * I.n + psf::kChunk - 1) / psf::kChunk);
        ncmax = std::max(ncmax, I.nc);
    }
    b->ne_tot = ne;
    b->nv_tot = nv;
    b->mg_nodes = mgn;
    b->mg_elems = mge;
    b->ainv_tot = ai;
    b->smem = sizeof(double) * (32 + (size_t)ncmax * 2 * ncmax + ncmax);
    // largest instances first
    b->order.resize(ninst);
    std::iota(b->order.begin(), b->order.end(), 0);
    std::stable_sort(b->order.begin(), b->order.end(),
                     [b](int x, int y) { return b->hinst[x].n > b->hinst[y].n; });
    Args &a = b->a;
    a.ninst = ninst;
    psf_status s = PSF_OK;
    auto ck = [&s](psf_status t) { if (s == PSF_OK) s = t; };
    ck(psf::cuda_status(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking), "stream"));
    ck(psf::cuda_status(cudaEventCreate(&b->ev0), "event"));
    ck(psf::cuda_status(cudaEventCreate(&b->ev1), "event"));
    Inst *dinst = nullptr;
    int *dorder = nullptr;
    unsigned char *dfixed = nullptr;
    ck(balloc(b, &dinst, ninst));
    ck(balloc(b, &dorder, ninst));
    for (double **pp : {&a.s, &a.rho, &a.E, &a.dfdrho, &a.dfds, &a.dgds, &a.snew, &a.wsum, &a.vw, &a.Bp})
        ck(balloc(b, pp, ne));
    ck(balloc(b, &a.Ef, ne));
    ck(balloc(b, &a.Ew, ne));
    for (double **pp : {&a.x, &a.r, &a.p, &a.q, &a.F}) ck(balloc(b, pp, nv));
    ck(balloc(b, &dfixed, nv));
    ck(balloc(b, &a.Kel, mge * 16));
    ck(balloc(b, &a.St, mgn * 9));
    for (float **pp : {&a.D, &a.mx, &a.mb, &a.mr}) ck(balloc(b, pp, mgn));
    ck(balloc(b, &a.mfix, mgn));
    ck(balloc(b, &a.Ainv, ai));
    ck(balloc(b, &a.out, (size_t)ninst * psf::batch::kOut));
    ck(balloc(b, &a.red, (size_t)ninst * 2 * psf::batch::kMaxCluster));
    ck(balloc(b, &a.ocs, ocs));
    if (s != PSF_OK) {
        batch_free(b);
        return s;
    }
    a.inst = dinst;
    a.order = dorder;
    a.fixed = dfixed;
    // Dirichlet patches and lumped loads (area / 4 per adjacent unit element)
    std::vector<unsigned char> hfix(nv, 0);
    std::vector<double> hF(nv, 0.0);
    for (int k = 0; k < ninst; k++) {
        const Inst &I = b->hinst[k];
        const int n = I.n;
        for (int i = 0; i <= n; i++)
            for (int j = 0; j <= n; j++) {
                const long long v = I.v0 + (long long)(n + 1) * i + j;
                const int c = (i > 0 && j > 0) + (i < n && j > 0) + (i > 0 && j < n) + (i < n && j < n);
                hF[v] = c * 0.25;
                int t = -1;
                if (edge[k] == 0 && j == 0) t = i;
                if (edge[k] == 1 && j == n) t = i;
                if (edge[k] == 2 && i == 0) t = j;
                if (edge[k] == 3 && i == n) t = j;
                if (t >= patch_i0[k] && t <= patch_i0[k] + patch_w[k]) hfix[v] = 1;
            }
    }
    ck(psf::cuda_status(cudaMemcpy(dinst, b->hinst.data(), sizeof(Inst) * ninst, cudaMemcpyHostToDevice), "copy"));
    ck(psf::cuda_status(cudaMemcpy(dorder, b->order.data(), sizeof(int) * ninst, cudaMemcpyHostToDevice), "copy"));
    ck(psf::cuda_status(cudaMemcpy(dfixed, hfix.data(), nv, cudaMemcpyHostToDevice), "copy"));
    ck(psf::cuda_status(cudaMemcpy(a.F, hF.data(), sizeof(double) * nv, cudaMemcpyHostToDevice), "copy"));
    ck(psf::cuda_status(cudaMemset(a.x, 0, sizeof(double) * nv), "memset"));
    // element matrix of the unit heat element, from the library's own element routine (bit-exact with the reference)
    psf_ctx *tmp = nullptr;
    if (s == PSF_OK) s = psf_create(&tmp, PSF_Q4_HEAT, 1, 1, 0, 1.0, 1.0, 0.0, 0.3, 1.0);
    double Ke[16];
    if (s == PSF_OK) s = psf_element_matrix(tmp, 1.0, Ke);
    if (tmp) psf_destroy(tmp);
    if (s != PSF_OK) {
        batch_free(b);
        return s;
    }
    for (int q = 0; q < 16; q++) {
        a.Ke0[q] = Ke[q];
        a.Ke0f[q] = (float)Ke[q];
        a.Ke0lo[q] = (float)(Ke[q] - (double)a.Ke0f[q]);
    }
    {
        const char *e = getenv("PSF_MG_CHEB");
        const double ratio = e ? atof(e) : 40.0;   // the single-problem solver's default (psf_mg.cu)
        a.sm_om = 1.0f; a.sm_c2 = 0.0f; a.sm_c3 = 1.0f;
        if (ratio > 1.0) {
            const double lo = 1.0 / ratio, theta = 0.5 * (1.0 + lo), delta = 0.5 * (1.0 - lo), sigma = theta / delta;
            const double rho0 = 1.0 / sigma, rho1 = 1.0 / (2.0 * sigma - rho0);
            a.sm_om = (float)(1.0 / theta);
            a.sm_c2 = (float)(rho1 * rho0);
            a.sm_c3 = (float)(2.0 * rho1 / delta);
        }
    }
    *out = b;
    return PSF_OK;
}

psf_status psf_batch_destroy(psf_batch *b) {
    batch_free(b);
    return PSF_OK;
}

psf_status psf_batch_begin(psf_batch *b, const psf_simp_params *prm) {
    if (!b || !prm) return PSF_BAD_INPUT;
    if (prm->optimizer != 0 || !(prm->R > 0) || prm->cg_itmax < 1 || !(prm->cg_eps > 0)) {
        psf::set_error("psf_batch_begin: the batch runs OC with a density filter (optimizer 0, R > 0)");
        return PSF_BAD_INPUT;
    }
    Args &a = b->a;
    a.k0 = prm->E1;
    a.kmin = prm->E0;
    a.pexp = prm->p;
    a.iota = prm->oc_iota;
    a.lmin = prm->oc_lmin;
    a.lmax = prm->oc_lmax;
    a.leps = prm->oc_leps;
    a.move = prm->oc_move;
    a.eps = prm->cg_eps;
    a.itmax = prm->cg_itmax;
    a.warm = prm->warm_start ? 1 : 0;
    // filter stencil on unit elements: w = (R - d) / R for d <= R (the samples' neighbour weights)
    const int rr = (int)std::floor(prm->R);
    a.nst = 0;
    for (int di = -rr; di <= rr; di++)
        for (int dj = -rr; dj <= rr; dj++) {
            const double d = std::sqrt(std::pow(di * 1.0, 2.0) + std::pow(dj * 1.0, 2.0));
            if (d <= prm->R) {
                if (a.nst >= psf::batch::kMaxStencilB) {
                    psf::set_error("psf_batch_begin: filter radius too large");
                    return PSF_BAD_INPUT;
                }
                a.sdi[a.nst] = di;
                a.sdj[a.nst] = dj;
                a.sw[a.nst] = (prm->R - d) / prm->R;
                a.nst++;
            }
        }
    // per-element weight sums, initial design
    std::vector<double> ws(b->ne_tot), s0(b->ne_tot);
    for (int k = 0; k < b->ninst; k++) {
        const Inst &I = b->hinst[k];
        const int n = I.n;
        for (int i = 0; i < n; i++)
            for (int j = 0; j < n; j++) {
                double w = 0.0;
                for (int q = 0; q < a.nst; q++) {
                    const int x = i + a.sdi[q], y = j + a.sdj[q];
                    if (x < 0 || y < 0 || x >= n || y >= n) continue;
                    w += a.sw[q];
                }
                ws[I.e0 + (long long)n * i + j] = w;
                s0[I.e0 + (long long)n * i + j] = I.vf;
            }
    }
    // volume weights vw_j = sum over e in N(j) of w_ej / wsum_e (the filter is symmetric: w_ej = w_je)
    std::vector<double> vw(b->ne_tot, 0.0);
    for (int k = 0; k < b->ninst; k++) {
        const Inst &I = b->hinst[k];
        const int n = I.n;
        for (int i = 0; i < n; i++)
            for (int j = 0; j < n; j++) {
                double acc = 0.0;
                for (int q = 0; q < a.nst; q++) {
                    const int x = i + a.sdi[q], y = j + a.sdj[q];
                    if (x < 0 || y < 0 || x >= n || y >= n) continue;
                    acc += a.sw[q] / ws[I.e0 + (long long)n * x + y];
                }
                vw[I.e0 + (long long)n * i + j] = acc;
            }
    }
    PSF_CUDA(cudaMemcpy(a.vw, vw.data(), sizeof(double) * vw.size(), cudaMemcpyHostToDevice));
    PSF_CUDA(cudaMemcpy(a.wsum, ws.data(), sizeof(double) * ws.size(), cudaMemcpyHostToDevice));
    PSF_CUDA(cudaMemcpy(a.s, s0.data(), sizeof(double) * s0.size(), cudaMemcpyHostToDevice));
    PSF_CUDA(cudaMemset(a.x, 0, sizeof(double) * b->nv_tot));
    PSF_CUDA(cudaMemset(a.out, 0, sizeof(double) * b->ninst * psf::batch::kOut));   // f_prev = 0, not done
    PSF_CUDA(cudaFuncSetAttribute(psf::batch::solve_batch, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)b->smem));
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->exec = nullptr;
    b->graph = nullptr;
    // one SIMP iteration of every instance as a graph
    PSF_CUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    psf_status st = launch_phases(b);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(b->stream, &g);
    if (st != PSF_OK) {
        if (g) cudaGraphDestroy(g);
        return st;
    }
    PSF_CUDA(e);
    b->graph = g;
    PSF_CUDA(cudaGraphInstantiate(&b->exec, g, 0));
    b->graph_nodes = 0;
    PSF_CUDA(cudaGraphGetNodes(g, nullptr, &b->graph_nodes));
    b->hout.assign((size_t)b->ninst * psf::batch::kOut, 0.0);
    b->begun = true;
    return PSF_OK;
}

psf_status psf_batch_step(psf_batch *b, int iters, double *seconds) {
    if (!b || !b->begun || iters < 1) return PSF_BAD_INPUT;
    PSF_CUDA(cudaEventRecord(b->ev0, b->stream));
    for (int k = 0; k < iters; k++) PSF_CUDA(cudaGraphLaunch(b->exec, b->stream));
    ::psf::note_launch((long long)iters * (long long)b->graph_nodes);
    PSF_CUDA(cudaEventRecord(b->ev1, b->stream));
    PSF_CUDA(cudaEventSynchronize(b->ev1));
    float ms = 0.f;
    PSF_CUDA(cudaEventElapsedTime(&ms, b->ev0, b->ev1));
    if (seconds) *seconds = ms * 1e-3;
    return PSF_OK;
}

psf_status psf_batch_profile(psf_batch *b, double *phase_seconds) {
    if (!b || !b->begun || !phase_seconds) return PSF_BAD_INPUT;
    cudaEvent_t ev[5];
    for (auto &e : ev) PSF_CUDA(cudaEventCreate(&e));
    PSF_CUDA(cudaEventRecord(ev[0], b->stream));
    PSF_CUDA(launch_phase(b, psf::batch::filter_moduli_batch, 0));
    PSF_CUDA(cudaEventRecord(ev[1], b->stream));
    PSF_CUDA(launch_phase(b, psf::batch::solve_batch, b->smem));
    PSF_CUDA(cudaEventRecord(ev[2], b->stream));
    PSF_CUDA(launch_phase(b, psf::batch::sens_batch, 0));
    PSF_CUDA(cudaEventRecord(ev[3], b->stream));
    PSF_CUDA(launch_phase(b, psf::batch::oc_batch, 0));
    PSF_CUDA(cudaEventRecord(ev[4], b->stream));
    PSF_CUDA(cudaEventSynchronize(ev[4]));
    for (int k = 0; k < 4; k++) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, ev[k], ev[k + 1]);
        phase_seconds[k] = ms * 1e-3;
    }
    for (auto &e : ev) cudaEventDestroy(e);
    return PSF_OK;
}

psf_status psf_batch_results(psf_batch *b, double *out) {
    if (!b || !out) return PSF_BAD_INPUT;
    PSF_CUDA(cudaMemcpy(out, b->a.out, sizeof(double) * b->ninst * psf::batch::kOut, cudaMemcpyDeviceToHost));
    return PSF_OK;
}

psf_status psf_batch_fields(psf_batch *b, int k, double *s, double *rho, double *T) {
    if (!b || k < 0 || k >= b->ninst) return PSF_BAD_INPUT;
    const Inst &I = b->hinst[k];
    const size_t ne = (size_t)I.n * I.n, nv = (size_t)(I.n + 1) * (I.n + 1);
    if (s) PSF_CUDA(cudaMemcpy(s, b->a.s + I.e0, sizeof(double) * ne, cudaMemcpyDeviceToHost));
    if (rho) PSF_CUDA(cudaMemcpy(rho, b->a.rho + I.e0, sizeof(double) * ne, cudaMemcpyDeviceToHost));
    if (T) PSF_CUDA(cudaMemcpy(T, b->a.x + I.v0, sizeof(double) * nv, cudaMemcpyDeviceToHost));
    return PSF_OK;
}

}  // extern "C"
