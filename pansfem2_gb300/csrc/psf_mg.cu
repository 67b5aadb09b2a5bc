// psf_mg.cu -- geometric multigrid preconditioned CG in FP32 inside FP64
// iterative refinement (PSF_SOLVE_IR_MG_F32).
//
// Hierarchy: the structured grid is coarsened by 2 per axis (a coarse axis of
// ceil(n/2) elements) while every axis has at least 2 elements and the level
// has more than kCoarseDofs dofs.  Coarse node I sits on fine node 2I; on an odd
// axis the last coarse node lies one fine element beyond the grid (a ghost
// node), and the last coarse element holds one fine child along that axis, the
// missing one counting as an element of zero stiffness.  Coarse operators are
// Galerkin products built element by element: bilinear (trilinear)
// prolongation restricted to one coarse element depends only on that
// element's nodes, so A_c = P^T A_f P is the sum over coarse elements of
// K_c = sum_children P_c^T K_child P_c.  Element matrices are stored per coarse
// element (FP32), with the rows / columns of fixed dofs zeroed at every level;
// a coarse node is fixed where its coincident fine node is (a ghost node never
// is; where its only fine neighbour is fixed its row is empty and the smoother
// and the coarsest solve treat it as an identity row).
//
// Cycle: V(2,2) with degree-2 Chebyshev smoothing on the l1-Jacobi scaled operator,
// full restriction R = P^T, and an
// exact coarsest solve by a dense FP64 inverse (Gauss-Jordan on the device),
// all in FP32 on the normalised residual.  The Krylov method around it is
// flexible CG in FP64 (operator, dot products, recurrences), so FP32 rounding
// only perturbs the preconditioner.  The whole solve is one persistent
// cooperative kernel; a final FP64 true residual confirms convergence.
#include <cmath>
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "psf_dw.cuh"
#include "psf_internal.cuh"

namespace psf {

constexpr int kMaxLev = 14;
// coarsen while the level has more dofs than this: the dense FP64 inverse of the
// coarsest level is built by one block in n dependent steps, so keep n small
constexpr long long kCoarseDofs = 40;

struct KeF {
    float v[576];
};
struct KeT64 {
    double v[576];
};
// the FP64 element matrix split into float pairs hi + lo (48 significant bits)
struct KeDS {
    float hi[576], lo[576];
};

static inline psf_status residual64_check(Ctx *c, const double *b, const double *x, double *r, double *rn, double *bn) {
    return residual64_pub(c, b, x, r, rn, bn);
}

struct MgLev {
    int nx, ny, nz;              // elements
    long long nnodes, ndofs, ne;
    float *K;                    // element matrices (levels >= 1), ne * nk * nk (Galerkin build)
    float *S;                    // node stencil (levels >= 1): [slot][a][b][node], 3^d slots of nd x nd
    float *Ep;                   // padded moduli (level 0)
    float *D;                    // nodal diagonal, 1 on fixed dofs
    unsigned char *fixed;
    float *x, *xt, *b, *r;
};

struct MgHier {
    int nlev = 0;
    MgLev L[kMaxLev];
    int nc = 0;                  // coarsest dofs
    double *Ac = nullptr;        // coarsest dense matrix / inverse (nc x nc)
    std::vector<void *> allocs;
    bool built_for_current_E = false;
    unsigned long long *trace = nullptr;   // phase timestamps (PSF_MG_TRACE)
    float2 *xw = nullptr, *rw = nullptr, *pw = nullptr, *qw = nullptr, *Ew = nullptr;   // double-word FCG
    long long npad = 0;
    float *tbuf = nullptr;       // private buffers of the fused grid levels
    size_t tbuf_bytes = 0;
    size_t max_dyn = 0;          // dynamic shared memory the solver kernels may take
};

// ------------------------------------------------------------------ geometry helpers
template <int KIND>
struct KT {
    static constexpr bool is3d = KIND == PSF_H8_SOLID;
    static constexpr int nd = KIND == PSF_Q4_PLANE_STRAIN ? 2 : (KIND == PSF_Q4_HEAT ? 1 : 3);
    static constexpr int nen = is3d ? 8 : 4;
    static constexpr int nk = nen * nd;
};

__device__ __forceinline__ int corner_q(int di, int dj, int dk) { return (di ? (dj ? 2 : 1) : (dj ? 3 : 0)) + 4 * dk; }
__device__ __forceinline__ void corner_of(int q, int &qi, int &qj, int &qk) {
    qi = (q == 1 || q == 2 || q == 5 || q == 6);
    qj = (q == 2 || q == 3 || q == 6 || q == 7);
    qk = q >= 4;
}

template <int KIND>
__device__ __forceinline__ long long lnode(const MgLev &L, int i, int j, int k) {
    return KT<KIND>::is3d ? ((long long)(L.ny + 1) * i + j) * (L.nz + 1) + k : (long long)(L.ny + 1) * i + j;
}
template <int KIND>
__device__ __forceinline__ void lnode_ijk(const MgLev &L, long long n, int &i, int &j, int &k) {
    if (KT<KIND>::is3d) {
        k = (int)(n % (L.nz + 1));
        long long r = n / (L.nz + 1);
        j = (int)(r % (L.ny + 1));
        i = (int)(r / (L.ny + 1));
    } else {
        k = 0;
        j = (int)(n % (L.ny + 1));
        i = (int)(n / (L.ny + 1));
    }
}
template <int KIND>
__device__ __forceinline__ long long lelem(const MgLev &L, int i, int j, int k) {
    return KT<KIND>::is3d ? ((long long)L.ny * i + j) * L.nz + k : (long long)L.ny * i + j;
}

// the nd values of node m of a node-major vector (one 8-byte load for two dofs)
template <int ND>
__device__ __forceinline__ void load_node(const float *__restrict__ v, long long m, float *o) {
    if constexpr (ND == 2) {
        const float2 t = *reinterpret_cast<const float2 *>(v + 2 * m);
        o[0] = t.x;
        o[1] = t.y;
    } else {
#pragma unroll
        for (int b = 0; b < ND; b++) o[b] = v[m * ND + b];
    }
}

// 2D level 0: the 3 x 3 node neighbourhood of node (i, j) (u[a][b] = node (clamp(i + a - 1),
// clamp(j + b - 1))) and the moduli of its four elements
template <int ND>
struct L0Gather {
    float u[3][3][ND];
    float E[2][2];
};
template <int KIND, class LD>
__device__ __forceinline__ void l0_gather(const MgLev &L, LD ld, int i, int j, L0Gather<KT<KIND>::nd> &g) {
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
        for (int b = 0; b < 3; b++) {
            const int mi = min(max(i + a - 1, 0), L.nx), mj = min(max(j + b - 1, 0), L.ny);
            ld(lnode<KIND>(L, mi, mj, 0), mi, mj, 0, g.u[a][b]);
        }
#pragma unroll
    for (int ci = 0; ci < 2; ci++)
#pragma unroll
        for (int cj = 0; cj < 2; cj++) g.E[ci][cj] = L.Ep[(long long)(i + ci) * (L.ny + 2) + (j + cj)];
}
// y = sum over the four elements of E_e (Ke0 u_e) rows of the node, element by element
template <int KIND>
__device__ __forceinline__ void l0_compute(const KeF &Ke, const L0Gather<KT<KIND>::nd> &g, float *y) {
    using T = KT<KIND>;
#pragma unroll
    for (int a = 0; a < T::nd; a++) y[a] = 0.f;
#pragma unroll
    for (int ci = 0; ci < 2; ci++)
#pragma unroll
        for (int cj = 0; cj < 2; cj++) {
            const int li = corner_q(1 - ci, 1 - cj, 0);
            float ue[T::nk];
#pragma unroll
            for (int q = 0; q < T::nen; q++) {
                int qi, qj, qk;
                corner_of(q, qi, qj, qk);
#pragma unroll
                for (int b = 0; b < T::nd; b++) ue[q * T::nd + b] = g.u[ci + qi][cj + qj][b];
            }
            const float Ee = g.E[ci][cj];
#pragma unroll
            for (int a = 0; a < T::nd; a++) {
                float acc = 0.f;
                const int row = (li * T::nd + a) * T::nk;
#pragma unroll
                for (int l = 0; l < T::nk; l++) acc += Ke.v[row + l] * ue[l];
                y[a] += Ee * acc;
            }
        }
}

// y = (A_l v)(node) for the ndof dofs of node (i,j,k); level 0 uses E*Ke0, coarse levels their
// element matrices.  The vector is read through ld(m, mi, mj, mk, out): the nd values of node
// m = (mi, mj, mk).  In 2D the 3 x 3 node neighbourhood is read once and shared by the four
// elements (the sums are the same as element by element).
template <int KIND, class LD>
__device__ __forceinline__ void apply_node_f(const MgLev &L, int lev, const KeF &Ke, LD ld, int i, int j, int k,
                                             float *y) {
    using T = KT<KIND>;
#pragma unroll
    for (int a = 0; a < T::nd; a++) y[a] = 0.f;
    if (lev > 0) {
        // coarse levels: assembled node stencil, structure of arrays (coalesced
        // across the warp's consecutive nodes); out-of-grid slots hold zeros
        const long long n = lnode<KIND>(L, i, j, k);
        int slot = 0;
#pragma unroll
        for (int di = -1; di <= 1; di++)
#pragma unroll
            for (int dj = -1; dj <= 1; dj++)
#pragma unroll
                for (int dk = (T::is3d ? -1 : 0); dk <= (T::is3d ? 1 : 0); dk++, slot++) {
                    const int mi = min(max(i + di, 0), L.nx), mj = min(max(j + dj, 0), L.ny),
                              mk = T::is3d ? min(max(k + dk, 0), L.nz) : 0;
                    const long long m = lnode<KIND>(L, mi, mj, mk);
                    float vb[T::nd];
                    ld(m, mi, mj, mk, vb);
#pragma unroll
                    for (int a = 0; a < T::nd; a++)
#pragma unroll
                        for (int b = 0; b < T::nd; b++)
                            y[a] += L.S[((long long)(slot * T::nd + a) * T::nd + b) * L.nnodes + n] * vb[b];
                }
        return;
    }
    if constexpr (!T::is3d) {
        L0Gather<T::nd> g;
        l0_gather<KIND>(L, ld, i, j, g);
        l0_compute<KIND>(Ke, g, y);
    } else {
#pragma unroll
    for (int ci = 0; ci < 2; ci++)
#pragma unroll
        for (int cj = 0; cj < 2; cj++)
#pragma unroll
            for (int ck = 0; ck < (T::is3d ? 2 : 1); ck++) {
                const int ei = i - 1 + ci, ej = j - 1 + cj, ek = T::is3d ? k - 1 + ck : 0;
                const int li = corner_q(1 - ci, 1 - cj, T::is3d ? 1 - ck : 0);
                float ue[T::nk];
#pragma unroll
                for (int q = 0; q < T::nen; q++) {
                    int qi, qj, qk;
                    corner_of(q, qi, qj, qk);
                    const int ni = min(max(ei + qi, 0), L.nx), nj = min(max(ej + qj, 0), L.ny),
                              nk2 = T::is3d ? min(max(ek + qk, 0), L.nz) : 0;
                    ld(lnode<KIND>(L, ni, nj, nk2), ni, nj, nk2, ue + q * T::nd);
                }
                const float Ee = L.Ep[T::is3d ? ((long long)(ei + 1) * (L.ny + 2) + (ej + 1)) * (L.nz + 2) + (ek + 1)
                                              : (long long)(ei + 1) * (L.ny + 2) + (ej + 1)];
#pragma unroll
                for (int a = 0; a < T::nd; a++) {
                    float acc = 0.f;
                    const int row = (li * T::nd + a) * T::nk;
#pragma unroll
                    for (int l = 0; l < T::nk; l++) acc += Ke.v[row + l] * ue[l];
                    y[a] += Ee * acc;
                }
            }
    }
}

template <int KIND>
__device__ __forceinline__ void apply_node(const MgLev &L, int lev, const KeF &Ke, const float *__restrict__ v, int i,
                                           int j, int k, float *y) {
    apply_node_f<KIND>(L, lev, Ke, [v](long long m, int, int, int, float *o) { load_node<KT<KIND>::nd>(v, m, o); },
                       i, j, k, y);
}

// interpolation weight of coarse corner q at fine position (fx, fy, fz) in {0, 1/2, 1}
__device__ __forceinline__ float interp_w(int q, int hx, int hy, int hz, bool is3d) {
    // hx, hy, hz in {0, 1, 2} = fine offsets in halves of the coarse element
    int qi, qj, qk;
    corner_of(q, qi, qj, qk);
    const float wx = qi ? hx * 0.5f : (2 - hx) * 0.5f;
    const float wy = qj ? hy * 0.5f : (2 - hy) * 0.5f;
    const float wz = is3d ? (qk ? hz * 0.5f : (2 - hz) * 0.5f) : 1.f;
    return wx * wy * wz;
}

// ------------------------------------------------------------------ hierarchy set-up kernels
// coarse element matrices: K_c = sum_children P_c^T K_child P_c, then masked by the coarse fixed set
template <int KIND>
__global__ void galerkin_kernel(MgLev F, MgLev Cc, int fine_lev, KeF Ke) {
    using T = KT<KIND>;
    constexpr int nk = T::nk, nen = T::nen, nd = T::nd;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < Cc.ne; e += (long long)gridDim.x * blockDim.x) {
        int ci, cj, ck = 0;
        if (T::is3d) {
            ck = (int)(e % Cc.nz);
            long long r = e / Cc.nz;
            cj = (int)(r % Cc.ny);
            ci = (int)(r / Cc.ny);
        } else {
            cj = (int)(e % Cc.ny);
            ci = (int)(e / Cc.ny);
        }
        float Kc[nk * nk];
        for (int q = 0; q < nk * nk; q++) Kc[q] = 0.f;
        for (int ch = 0; ch < (T::is3d ? 8 : 4); ch++) {
            int a, b, c;
            corner_of(ch, a, b, c);
            const int fi = 2 * ci + a, fj = 2 * cj + b, fk = T::is3d ? 2 * ck + c : 0;
            // a child beyond an odd fine axis does not exist (zero stiffness)
            if (fi >= F.nx || fj >= F.ny || (T::is3d && fk >= F.nz)) continue;
            // child matrix (masked at the fine level)
            float Kf[nk * nk];
            const long long fe = lelem<KIND>(F, fi, fj, fk);
            if (fine_lev == 0) {
                const float E = F.Ep[T::is3d ? ((long long)(fi + 1) * (F.ny + 2) + (fj + 1)) * (F.nz + 2) + (fk + 1)
                                             : (long long)(fi + 1) * (F.ny + 2) + (fj + 1)];
                for (int q = 0; q < nk * nk; q++) Kf[q] = E * Ke.v[q];
                bool fx[nk];
                for (int f = 0; f < nen; f++) {
                    int qi, qj, qk;
                    corner_of(f, qi, qj, qk);
                    const long long m = lnode<KIND>(F, fi + qi, fj + qj, fk + qk);
                    for (int s = 0; s < nd; s++) fx[f * nd + s] = F.fixed[m * nd + s] != 0;
                }
                for (int r = 0; r < nk; r++)
                    for (int s = 0; s < nk; s++)
                        if (fx[r] || fx[s]) Kf[r * nk + s] = 0.f;
            } else {
                const float *src = F.K + fe * (nk * nk);
                for (int q = 0; q < nk * nk; q++) Kf[q] = src[q];
            }
            // W[f][q]: fine local node f of this child from coarse corner q
            float W[nen * nen];
            for (int f = 0; f < nen; f++) {
                int qi, qj, qk;
                corner_of(f, qi, qj, qk);
                for (int q = 0; q < nen; q++) W[f * nen + q] = interp_w(q, a + qi, b + qj, c + qk, T::is3d);
            }
            // Kc += (W x I)^T Kf (W x I)
            for (int fr = 0; fr < nen; fr++)
                for (int s = 0; s < nd; s++) {
                    // t[q'][s'] = sum_f' Kf[fr s][f' s'] W[f'][q']
                    float t[nk];
                    for (int q2 = 0; q2 < nen; q2++)
                        for (int s2 = 0; s2 < nd; s2++) {
                            float acc = 0.f;
                            for (int f2 = 0; f2 < nen; f2++) acc += Kf[(fr * nd + s) * nk + f2 * nd + s2] * W[f2 * nen + q2];
                            t[q2 * nd + s2] = acc;
                        }
                    for (int q = 0; q < nen; q++) {
                        const float w = W[fr * nen + q];
                        if (w == 0.f) continue;
                        for (int l = 0; l < nk; l++) Kc[(q * nd + s) * nk + l] += w * t[l];
                    }
                }
        }
        // mask by the coarse fixed set
        bool cx[nk];
        for (int f = 0; f < nen; f++) {
            int qi, qj, qk;
            corner_of(f, qi, qj, qk);
            const long long m = lnode<KIND>(Cc, ci + qi, cj + qj, ck + qk);
            for (int s = 0; s < nd; s++) cx[f * nd + s] = Cc.fixed[m * nd + s] != 0;
        }
        float *dst = Cc.K + e * (nk * nk);
        for (int r = 0; r < nk; r++)
            for (int s = 0; s < nk; s++) dst[r * nk + s] = (cx[r] || cx[s]) ? 0.f : Kc[r * nk + s];
    }
}

// coarse fixed set from the coincident fine nodes
template <int KIND>
__global__ void coarse_fixed_kernel(MgLev F, MgLev Cc) {
    using T = KT<KIND>;
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < Cc.nnodes; n += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        lnode_ijk<KIND>(Cc, n, i, j, k);
        const bool ghost = 2 * i > F.nx || 2 * j > F.ny || (T::is3d && 2 * k > F.nz);
        const long long m = ghost ? 0 : lnode<KIND>(F, 2 * i, 2 * j, 2 * k);
        for (int s = 0; s < T::nd; s++) Cc.fixed[n * T::nd + s] = ghost ? 0 : F.fixed[m * T::nd + s];
    }
}

// Node stencil of a coarse level from its (masked) element matrices: the block
// coupling node n to neighbour m sums, over the elements holding both, the
// element matrix block (local n, local m).  Also the l1 row sums sum_j |A_ij|
// (the smoother's diagonal: l1-Jacobi converges for any SPD operator).
template <int KIND>
__global__ void coarse_stencil_kernel(MgLev L) {
    using T = KT<KIND>;
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < L.nnodes; n += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        lnode_ijk<KIND>(L, n, i, j, k);
        float d1[T::nd];
        for (int a = 0; a < T::nd; a++) d1[a] = 0.f;
        int slot = 0;
        for (int di = -1; di <= 1; di++)
            for (int dj = -1; dj <= 1; dj++)
                for (int dk = (T::is3d ? -1 : 0); dk <= (T::is3d ? 1 : 0); dk++, slot++) {
                    float blk[T::nd * T::nd];
                    for (int q = 0; q < T::nd * T::nd; q++) blk[q] = 0.f;
                    const int mi = i + di, mj = j + dj, mk = k + dk;
                    const bool mok = mi >= 0 && mi <= L.nx && mj >= 0 && mj <= L.ny && (!T::is3d || (mk >= 0 && mk <= L.nz));
                    if (mok) {
                        for (int ei = max(i, mi) - 1; ei <= min(i, mi); ei++)
                            for (int ej = max(j, mj) - 1; ej <= min(j, mj); ej++)
                                for (int ek = (T::is3d ? max(k, mk) - 1 : 0); ek <= (T::is3d ? min(k, mk) : 0); ek++) {
                                    if (ei < 0 || ei >= L.nx || ej < 0 || ej >= L.ny) continue;
                                    if (T::is3d && (ek < 0 || ek >= L.nz)) continue;
                                    const float *Ke = L.K + lelem<KIND>(L, ei, ej, ek) * (T::nk * T::nk);
                                    const int ln = corner_q(i - ei, j - ej, T::is3d ? k - ek : 0);
                                    const int lm = corner_q(mi - ei, mj - ej, T::is3d ? mk - ek : 0);
                                    for (int a = 0; a < T::nd; a++)
                                        for (int b = 0; b < T::nd; b++)
                                            blk[a * T::nd + b] += Ke[(ln * T::nd + a) * T::nk + lm * T::nd + b];
                                }
                    }
                    for (int a = 0; a < T::nd; a++)
                        for (int b = 0; b < T::nd; b++) {
                            L.S[((long long)(slot * T::nd + a) * T::nd + b) * L.nnodes + n] = blk[a * T::nd + b];
                            d1[a] += fabsf(blk[a * T::nd + b]);
                        }
                }
        for (int a = 0; a < T::nd; a++) {
            const long long q = n * T::nd + a;
            L.D[q] = (L.fixed[q] || !(d1[a] > 0.f)) ? 1.f : d1[a];
        }
    }
}

// dense coarsest matrix (FP64) from its element matrices; fixed dofs -> identity
template <int KIND>
__global__ void coarse_dense_kernel(MgLev L, double *A, int n) {
    using T = KT<KIND>;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < L.ne; e += (long long)gridDim.x * blockDim.x) {
        int i, j, k = 0;
        if (T::is3d) {
            k = (int)(e % L.nz);
            long long r = e / L.nz;
            j = (int)(r % L.ny);
            i = (int)(r / L.ny);
        } else {
            j = (int)(e % L.ny);
            i = (int)(e / L.ny);
        }
        long long dof[T::nk];
        for (int q = 0; q < T::nen; q++) {
            int qi, qj, qk;
            corner_of(q, qi, qj, qk);
            const long long m = lnode<KIND>(L, i + qi, j + qj, k + qk);
            for (int s = 0; s < T::nd; s++) dof[q * T::nd + s] = m * T::nd + s;
        }
        const float *Kel = L.K + e * (T::nk * T::nk);
        for (int r = 0; r < T::nk; r++)
            for (int s = 0; s < T::nk; s++) {
                const float v = Kel[r * T::nk + s];
                if (v != 0.f) atomicAdd(&A[dof[r] * n + dof[s]], (double)v);
            }
    }
}

__global__ void dense_fix_identity(double *A, const unsigned char *fixed, int n) {
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x)
        if (fixed[q] || A[(long long)q * n + q] == 0.0) {
            for (int t = 0; t < n; t++) { A[(long long)q * n + t] = 0.0; A[(long long)t * n + q] = 0.0; }
            A[(long long)q * n + q] = 1.0;
        }
}

// in-place Gauss-Jordan inverse of an SPD matrix (no pivoting), one block
__global__ void gauss_jordan_kernel(double *A, int n) {
    for (int k = 0; k < n; k++) {
        const double piv = 1.0 / A[(long long)k * n + k];
        __syncthreads();
        for (long long q = threadIdx.x; q < (long long)n * n; q += blockDim.x) {
            const int i = (int)(q / n), j = (int)(q % n);
            if (i != k && j != k) A[q] -= A[(long long)i * n + k] * A[(long long)k * n + j] * piv;
        }
        __syncthreads();
        for (int t = threadIdx.x; t < n; t += blockDim.x) {
            if (t != k) {
                A[(long long)k * n + t] *= piv;
                A[(long long)t * n + k] *= -piv;
            }
        }
        __syncthreads();
        if (threadIdx.x == 0) A[(long long)k * n + k] = piv;
        __syncthreads();
    }
}

// ------------------------------------------------------------------ the persistent solver kernel
// FP64 flexible CG, preconditioned by one FP32 V-cycle per iteration:
//   z = rn * V(r / rn);  beta = z.q_prev / p_prev.q_prev;  p = z - beta p_prev;
//   q = K p (FP64 matrix-free);  alpha = p.r / p.q;  x += alpha p;  r -= alpha q.
// The recurrences, dot products and operator stay in FP64; the cycle works on
// the normalised residual in FP32, so rounding in it perturbs the
// preconditioner only (no cond(K) amplification as in an FP32 inner solve).
struct MgFcgArgs {
    int nlev;
    int lsmall;               // first level run by block 0 alone (1 <= lsmall <= nlev - 1)
    MgLev L[kMaxLev];
    KeF Ke;                   // level-0 element matrix (FP32, cycle)
    KeT64 Ke64;               // level-0 element matrix (FP64, operator)
    KeDS Kds;                 // the same as float pairs hi + lo (double-word operator)
    const double *Ainv;
    int nc;
    float omega;              // first smoothing step from zero: x = omega D^-1 b
    // second smoothing step x2 = x1 + sm_c2 (x1 - x0) + sm_c3 D^-1 (b - A x1); l1-Jacobi: 0, 1.
    // Chebyshev of degree 2 on [1/ratio, 1] (D the l1 row sums bound the spectrum of
    // D^-1 A by 1): omega = 1/theta, c2 = rho1 rho0, c3 = 2 rho1 / delta.
    float sm_c2, sm_c3;
    const double *Ep64;       // padded FP64 moduli
    const double *b;          // nodal right-hand side
    double *x, *r, *z, *p, *q;
    int warm;                 // x holds the start vector
    int itmax;
    double eps;
    GridSync *gs;
    double *partials;
    double *out;              // iterations, |r|^2, |b|^2, converged, V-cycles
    unsigned long long *trace;   // optional: [0] = count, then %globaltimer after each sync of one iteration
    int trace_iter;
    int trace_steps;             // also after the block-level steps of the fused phases (block 0's view)
    // block 0's shared-memory levels: lsm (>= lsmall; nlev = none), byte offsets into dynamic
    // shared memory of S, D, x, xt, b, r, fixed per level, of the coarsest inverse (-1 = global)
    int lsm;
    int nslot;                // stencil floats per node: 3^d slots x nd x nd
    int smo[kMaxLev][7];
    int smo_ainv;
        // double-word Krylov vectors (mg_fcg_dw_kernel): x, r, p, q as FP32 pairs, padded moduli
    float2 *xw, *rw, *pw, *qw, *Ew;
    long long npad;           // padded moduli entries
    // fused grid levels (levels < lsmall with fuse[l] = 1): block b owns tile b of the level's
    // node grid, tg[l] tiles per axis of ts[l] nodes; tbuf holds two private buffers of
    // tbuf_half floats per block (the tile grown by two nodes per side)
    int fuse[kMaxLev];
    int tg[kMaxLev][3], ts[kMaxLev][3];
    float *tbuf;
    long long tbuf_half;
    // levels with tsm[l] = 1 keep the two buffers in dynamic shared memory from byte tsm_off
    // (tsm_half floats each) instead
    int tsm[kMaxLev];
    int tsm_off, tsm_half;
};

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
    return t;
}
// block 0 / thread 0 stamps the time after a grid sync of the traced iteration (the count
// is kept in shared memory: a global read-back would add its latency to every stamp)
__shared__ unsigned int s_trace_n;
__device__ __forceinline__ void trace_init() {
    if (threadIdx.x == 0) s_trace_n = 0;
}
__device__ __forceinline__ void stamp(const MgFcgArgs &A, bool on) {
    if (on && A.trace && blockIdx.x == 0 && threadIdx.x == 0) {
        const unsigned int n = s_trace_n;
        if (n < 1000) {
            A.trace[1 + n] = global_ns();
            A.trace[0] = n + 1;
            s_trace_n = n + 1;
        }
    }
}

// one smoothing step on level l:
//   first step  (xprev == xin): xout = xin + omega (b - A xin) / D
//   second step: xout = xin + c2 (xin - xprev) + c3 (b - A xin) / D, xprev == nullptr meaning 0
// (xout may alias xprev: every dof reads its own xprev before writing xout)
template <int KIND>
__device__ __forceinline__ void smooth_step(const MgFcgArgs &A, const MgLev *LV, int l, const float *xin,
                                            const float *xprev, float *xout, bool second, long long tid,
                                            long long stride) {
    using T = KT<KIND>;
    const MgLev &L = LV[l];
    const float c2 = second ? A.sm_c2 : 0.f, c3 = second ? A.sm_c3 : A.omega;
    for (long long n = tid; n < L.nnodes; n += stride) {
        int i, j, k;
        lnode_ijk<KIND>(L, n, i, j, k);
        float y[T::nd];
        apply_node<KIND>(L, l, A.Ke, xin, i, j, k, y);
#pragma unroll
        for (int s = 0; s < T::nd; s++) {
            const long long q = n * T::nd + s;
            const float xv = xin[q];
            const float xp = (second && xprev) ? xprev[q] : 0.f;
            xout[q] = L.fixed[q] ? 0.f : xv + c2 * (xv - xp) + c3 * (L.b[q] - y[s]) / L.D[q];
        }
    }
}

// barrier of a phase: the grid (all blocks) or block 0 alone
__device__ __forceinline__ bool phase_sync(const MgFcgArgs &A, bool grid) {
    if (grid) return grid_barrier(A.gs, A.partials);
    __syncthreads();
    return true;
}

// down-leg of level l: second pre-sweep, residual, restriction to level l+1 (and its first sweep)
template <int KIND>
__device__ bool down_level(const MgFcgArgs &A, const MgLev *LV, int l, long long tid, long long stride, bool grid,
                           bool tr) {
    using T = KT<KIND>;
    const int nl = A.nlev;
    const MgLev &L = LV[l];
    smooth_step<KIND>(A, LV, l, L.x, nullptr, L.xt, true, tid, stride);   // second pre-smoothing step (x0 = 0)
    if (!phase_sync(A, grid)) return false;
    stamp(A, tr);
    for (long long n = tid; n < L.nnodes; n += stride) {              // residual r = b - A xt
        int i, j, k;
        lnode_ijk<KIND>(L, n, i, j, k);
        float y[T::nd];
        apply_node<KIND>(L, l, A.Ke, L.xt, i, j, k, y);
#pragma unroll
        for (int s = 0; s < T::nd; s++) {
            const long long q = n * T::nd + s;
            L.r[q] = L.fixed[q] ? 0.f : L.b[q] - y[s];
        }
    }
    if (!phase_sync(A, grid)) return false;
    stamp(A, tr);
    const MgLev &Cc = LV[l + 1];
    for (long long n = tid; n < Cc.nnodes; n += stride) {             // restriction b_c = P^T r
        int i, j, k;
        lnode_ijk<KIND>(Cc, n, i, j, k);
        float acc[T::nd];
#pragma unroll
        for (int s = 0; s < T::nd; s++) acc[s] = 0.f;
        for (int di = -1; di <= 1; di++)
            for (int dj = -1; dj <= 1; dj++)
                for (int dk = (T::is3d ? -1 : 0); dk <= (T::is3d ? 1 : 0); dk++) {
                    const int fi = 2 * i + di, fj = 2 * j + dj, fk = 2 * k + dk;
                    if (fi < 0 || fi > L.nx || fj < 0 || fj > L.ny || (T::is3d && (fk < 0 || fk > L.nz))) continue;
                    const float w = (di ? 0.5f : 1.f) * (dj ? 0.5f : 1.f) * (dk ? 0.5f : 1.f);
                    const long long m = lnode<KIND>(L, fi, fj, fk);
#pragma unroll
                    for (int s = 0; s < T::nd; s++) acc[s] += w * L.r[m * T::nd + s];
                }
#pragma unroll
        for (int s = 0; s < T::nd; s++) {
            const long long q = n * T::nd + s;
            const float bv = Cc.fixed[q] ? 0.f : acc[s];
            Cc.b[q] = bv;
            Cc.x[q] = (l + 1 < nl - 1) ? A.omega * bv / Cc.D[q] : 0.f;   // first sweep from zero
        }
    }
    if (!phase_sync(A, grid)) return false;
    stamp(A, tr);
    return true;
}

// coarsest level: x = Ainv b (dense, FP64), one warp per row (the lanes read a row contiguously)
__device__ __forceinline__ void coarsest_solve(const MgFcgArgs &A, const MgLev *LV, const double *Ainv,
                                               long long tid, long long stride) {
    const MgLev &Cc = LV[A.nlev - 1];
    const int n = A.nc;
    const int lane = threadIdx.x & 31;
    for (long long q = tid >> 5; q < n; q += stride >> 5) {
        double acc = 0.0;
        const double *row = Ainv + q * n;
        for (int t = lane; t < n; t += 32) acc += row[t] * (double)Cc.b[t];
        acc = warp_sum(acc);
        if (lane == 0) Cc.x[q] = Cc.fixed[q] ? 0.f : (float)acc;
    }
}

// up-leg of level l: x = xt + P x_c, two post-smoothing sweeps (result in x)
template <int KIND>
__device__ bool up_level(const MgFcgArgs &A, const MgLev *LV, int l, long long tid, long long stride, bool grid,
                         bool tr) {
    using T = KT<KIND>;
    const MgLev &L = LV[l];
    const MgLev &Cc = LV[l + 1];
    for (long long n = tid; n < L.nnodes; n += stride) {              // x = xt + P x_c
        int i, j, k;
        lnode_ijk<KIND>(L, n, i, j, k);
        const int ci = i >> 1, cj = j >> 1, ck = k >> 1;
        const int hi = i & 1, hj = j & 1, hk = k & 1;
        float acc[T::nd];
#pragma unroll
        for (int s = 0; s < T::nd; s++) acc[s] = 0.f;
        for (int a = 0; a <= hi; a++)
            for (int b = 0; b <= hj; b++)
                for (int c = 0; c <= (T::is3d ? hk : 0); c++) {
                    const float w = (hi ? 0.5f : 1.f) * (hj ? 0.5f : 1.f) * ((T::is3d && hk) ? 0.5f : 1.f);
                    const long long m = lnode<KIND>(Cc, ci + a, cj + b, ck + c);
#pragma unroll
                    for (int s = 0; s < T::nd; s++) acc[s] += w * Cc.x[m * T::nd + s];
                }
#pragma unroll
        for (int s = 0; s < T::nd; s++) {
            const long long q = n * T::nd + s;
            L.x[q] = L.fixed[q] ? 0.f : L.xt[q] + acc[s];
        }
    }
    if (!phase_sync(A, grid)) return false;
    stamp(A, tr);
    smooth_step<KIND>(A, LV, l, L.x, nullptr, L.xt, false, tid, stride);   // post-smoothing, step 1
    if (!phase_sync(A, grid)) return false;
    stamp(A, tr);
    smooth_step<KIND>(A, LV, l, L.xt, L.x, L.x, true, tid, stride);        // step 2 -> x
    if (l > 0 || !grid) {
        if (!phase_sync(A, grid)) return false;
        stamp(A, tr);
    }
    return true;
}

// V(2,2)-cycle; on entry L[0].b holds the level-0 right-hand side and L[0].x its
// first sweep from zero (w b / D), both written by the caller before a barrier.
// On exit L[0].x holds the result, written by the node loop of the last sweep
// (same node -> thread mapping as the caller's next node loop, no barrier).
// Levels lsmall.. (a few thousand nodes and less) run in block 0 alone with
// block barriers while the other blocks wait at one grid barrier: a grid
// barrier costs microseconds, far more than those levels' work.
// Block 0's view of the hierarchy (shared memory, filled by block0_levels): the levels
// from A.lsm on have their stencils, diagonals, fixed flags and vectors in dynamic shared
// memory, the coarsest inverse too.  They are constant during a solve and are read by
// every phase of block 0's serial part of the cycle.
struct Block0View {
    MgLev L[kMaxLev];
    const double *Ainv;
};

// Copies the shared-memory levels in (block 0 only; the other blocks return at once).
__device__ void block0_levels(const MgFcgArgs &A, Block0View &V, unsigned char *dsm) {
    if (blockIdx.x != 0) return;
    if (threadIdx.x == 0) {
        for (int l = 0; l < A.nlev; l++) {
            V.L[l] = A.L[l];
            if (l >= A.lsm) {
                const int *o = A.smo[l];
                V.L[l].S = (float *)(dsm + o[0]);
                V.L[l].D = (float *)(dsm + o[1]);
                V.L[l].x = (float *)(dsm + o[2]);
                V.L[l].xt = (float *)(dsm + o[3]);
                V.L[l].b = (float *)(dsm + o[4]);
                V.L[l].r = (float *)(dsm + o[5]);
                V.L[l].fixed = dsm + o[6];
            }
        }
        V.Ainv = A.smo_ainv >= 0 ? (const double *)(dsm + A.smo_ainv) : A.Ainv;
    }
    for (int l = A.lsm; l < A.nlev; l++) {
        const MgLev &G = A.L[l];
        const int *o = A.smo[l];
        const long long ns = (l > 0) ? G.nnodes * A.nslot : 0;   // stencil floats (levels >= 1)
        float *S = (float *)(dsm + o[0]);
        float *D = (float *)(dsm + o[1]);
        unsigned char *F = dsm + o[6];
        for (long long t = threadIdx.x; t < ns; t += blockDim.x) S[t] = G.S[t];
        for (long long t = threadIdx.x; t < G.ndofs; t += blockDim.x) {
            D[t] = G.D[t];
            F[t] = G.fixed[t];
        }
    }
    if (A.smo_ainv >= 0) {
        double *Ai = (double *)(dsm + A.smo_ainv);
        for (long long t = threadIdx.x; t < (long long)A.nc * A.nc; t += blockDim.x) Ai[t] = A.Ainv[t];
    }
    __syncthreads();
}

// ------------------------------------------------------------------ fused grid levels
// A grid level's down-leg (second pre-sweep, residual, restriction) and up-leg (prolongation,
// two post-sweeps) each run as one grid phase instead of three: every block takes a tile of
// the level's nodes, grown by two nodes per side, and computes the intermediate sweeps on the
// grown tile into block-private buffers, the outer rings redundantly (each ring is the
// neighbourhood the next step reads).  Every node gets the same arithmetic as in the
// three-phase form, so the cycle's result is identical bit for bit; the grid barriers of a
// V-cycle fall from 6 per grid level to 2.
struct Box {
    int i0, i1, j0, j1, k0, k1;   // half-open node ranges
};

template <int KIND>
__device__ __forceinline__ bool own_box(const MgFcgArgs &A, int l, Box &b) {
    const int *tg = A.tg[l], *ts = A.ts[l];
    if ((int)blockIdx.x >= tg[0] * tg[1] * tg[2]) return false;
    int q = blockIdx.x;
    const int bk = q % tg[2];
    q /= tg[2];
    const int bj = q % tg[1], bi = q / tg[1];
    const MgLev &L = A.L[l];
    b.i0 = bi * ts[0]; b.i1 = min(b.i0 + ts[0], L.nx + 1);
    b.j0 = bj * ts[1]; b.j1 = min(b.j0 + ts[1], L.ny + 1);
    if (KT<KIND>::is3d) { b.k0 = bk * ts[2]; b.k1 = min(b.k0 + ts[2], L.nz + 1); }
    else { b.k0 = 0; b.k1 = 1; }
    return b.i0 < b.i1 && b.j0 < b.j1 && b.k0 < b.k1;
}

template <int KIND>
__device__ __forceinline__ Box grow(const Box &b, int h, const MgLev &L) {
    Box g;
    g.i0 = max(b.i0 - h, 0); g.i1 = min(b.i1 + h, L.nx + 1);
    g.j0 = max(b.j0 - h, 0); g.j1 = min(b.j1 + h, L.ny + 1);
    if (KT<KIND>::is3d) { g.k0 = max(b.k0 - h, 0); g.k1 = min(b.k1 + h, L.nz + 1); }
    else { g.k0 = 0; g.k1 = 1; }
    return g;
}

__device__ __forceinline__ int box_vol(const Box &b) { return (b.i1 - b.i0) * (b.j1 - b.j0) * (b.k1 - b.k0); }
__device__ __forceinline__ void box_ijk(const Box &b, int t, int &i, int &j, int &k) {
    const int nk = b.k1 - b.k0, nj = b.j1 - b.j0;
    k = b.k0 + t % nk;
    t /= nk;
    j = b.j0 + t % nj;
    i = b.i0 + t / nj;
}
__device__ __forceinline__ int box_at(const Box &b, int i, int j, int k) {
    return ((i - b.i0) * (b.j1 - b.j0) + (j - b.j0)) * (b.k1 - b.k0) + (k - b.k0);
}
__device__ __forceinline__ bool box_has(const Box &b, int i, int j, int k) {
    return i >= b.i0 && i < b.i1 && j >= b.j0 && j < b.j1 && k >= b.k0 && k < b.k1;
}

// the block's two private buffers of level l
__device__ __forceinline__ void tile_buffers(const MgFcgArgs &A, int l, float *&PX, float *&PR) {
    extern __shared__ __align__(16) unsigned char dsm[];
    if (A.tsm[l]) {
        PX = (float *)(dsm + A.tsm_off);
        PR = PX + A.tsm_half;
    } else {
        PX = A.tbuf + (size_t)blockIdx.x * 2 * A.tbuf_half;
        PR = PX + A.tbuf_half;
    }
}

// down-leg of grid level l as one phase (ends with the grid barrier)
template <int KIND>
__device__ bool down_fused(const MgFcgArgs &A, int l, bool tr) {
    using T = KT<KIND>;
    constexpr int nd = T::nd;
    const MgLev &L = A.L[l];
    const MgLev &Cc = A.L[l + 1];
    Box own;
    if (own_box<KIND>(A, l, own)) {
        const Box g2 = grow<KIND>(own, 2, L), g1 = grow<KIND>(own, 1, L);
        float *PX, *PR;
        tile_buffers(A, l, PX, PR);
        const float c2 = A.sm_c2, c3 = A.sm_c3;
        // second pre-sweep (from the first sweep in L.x) on the tile + 2 rings; own nodes to L.xt
        for (int t = threadIdx.x, nv = box_vol(g2); t < nv; t += blockDim.x) {
            int i, j, k;
            box_ijk(g2, t, i, j, k);
            const long long n = lnode<KIND>(L, i, j, k);
            float y[nd];
            apply_node<KIND>(L, l, A.Ke, L.x, i, j, k, y);
            const bool mine = box_has(own, i, j, k);
#pragma unroll
            for (int s = 0; s < nd; s++) {
                const long long q = n * nd + s;
                const float xv = L.x[q];
                const float x2 = L.fixed[q] ? 0.f : xv + c2 * (xv - 0.f) + c3 * (L.b[q] - y[s]) / L.D[q];
                PX[t * nd + s] = x2;
                if (mine) L.xt[q] = x2;
            }
        }
        __syncthreads();
        stamp(A, tr && A.trace_steps);
        // residual on the tile + 1 ring
        auto ldx = [&](long long, int mi, int mj, int mk, float *o) { load_node<nd>(PX, box_at(g2, mi, mj, mk), o); };
        for (int t = threadIdx.x, nv = box_vol(g1); t < nv; t += blockDim.x) {
            int i, j, k;
            box_ijk(g1, t, i, j, k);
            const long long n = lnode<KIND>(L, i, j, k);
            float y[nd];
            apply_node_f<KIND>(L, l, A.Ke, ldx, i, j, k, y);
            const int o = box_at(g2, i, j, k);
#pragma unroll
            for (int s = 0; s < nd; s++) {
                const long long q = n * nd + s;
                PR[o * nd + s] = L.fixed[q] ? 0.f : L.b[q] - y[s];
            }
        }
        __syncthreads();
        stamp(A, tr && A.trace_steps);
        // restriction to the coarse nodes on the tile (a ghost coarse node beyond an odd axis
        // belongs to the last tile of that axis)
        Box cb;
        cb.i0 = (own.i0 + 1) >> 1; cb.i1 = own.i1 == L.nx + 1 ? Cc.nx + 1 : (own.i1 + 1) >> 1;
        cb.j0 = (own.j0 + 1) >> 1; cb.j1 = own.j1 == L.ny + 1 ? Cc.ny + 1 : (own.j1 + 1) >> 1;
        if (T::is3d) { cb.k0 = (own.k0 + 1) >> 1; cb.k1 = own.k1 == L.nz + 1 ? Cc.nz + 1 : (own.k1 + 1) >> 1; }
        else { cb.k0 = 0; cb.k1 = 1; }
        const bool first = l + 1 < A.nlev - 1;
        for (int t = threadIdx.x, nv = cb.i1 > cb.i0 && cb.j1 > cb.j0 && cb.k1 > cb.k0 ? box_vol(cb) : 0; t < nv;
             t += blockDim.x) {
            int i, j, k;
            box_ijk(cb, t, i, j, k);
            float acc[nd];
#pragma unroll
            for (int s = 0; s < nd; s++) acc[s] = 0.f;
            for (int di = -1; di <= 1; di++)
                for (int dj = -1; dj <= 1; dj++)
                    for (int dk = (T::is3d ? -1 : 0); dk <= (T::is3d ? 1 : 0); dk++) {
                        const int fi = 2 * i + di, fj = 2 * j + dj, fk = 2 * k + dk;
                        if (fi < 0 || fi > L.nx || fj < 0 || fj > L.ny || (T::is3d && (fk < 0 || fk > L.nz))) continue;
                        const float w = (di ? 0.5f : 1.f) * (dj ? 0.5f : 1.f) * (dk ? 0.5f : 1.f);
                        const int o = box_at(g2, fi, fj, fk);
#pragma unroll
                        for (int s = 0; s < nd; s++) acc[s] += w * PR[o * nd + s];
                    }
            const long long n = lnode<KIND>(Cc, i, j, k);
#pragma unroll
            for (int s = 0; s < nd; s++) {
                const long long q = n * nd + s;
                const float bv = Cc.fixed[q] ? 0.f : acc[s];
                Cc.b[q] = bv;
                Cc.x[q] = first ? A.omega * bv / Cc.D[q] : 0.f;   // first sweep from zero
            }
        }
    }
    if (A.trace_steps) {
        __syncthreads();
        stamp(A, tr);
    }
    if (!grid_barrier(A.gs, A.partials)) return false;
    stamp(A, tr);
    return true;
}

// up-leg of grid level l as one phase: x = xt + P x_c and two post-sweeps, the result in L.x
// of the own nodes; on(q, x) sees every own dof's result.  Ends with the grid barrier when
// `barrier` (the caller's next phase reads other blocks' nodes).
template <int KIND, class ON>
__device__ bool up_fused(const MgFcgArgs &A, int l, bool tr, bool barrier, ON on) {
    using T = KT<KIND>;
    constexpr int nd = T::nd;
    const MgLev &L = A.L[l];
    const MgLev &Cc = A.L[l + 1];
    Box own;
    if (own_box<KIND>(A, l, own)) {
        const Box g2 = grow<KIND>(own, 2, L), g1 = grow<KIND>(own, 1, L);
        float *PX, *PR;
        tile_buffers(A, l, PX, PR);
        // x = xt + P x_c on the tile + 2 rings
        for (int t = threadIdx.x, nv = box_vol(g2); t < nv; t += blockDim.x) {
            int i, j, k;
            box_ijk(g2, t, i, j, k);
            const int ci = i >> 1, cj = j >> 1, ck = k >> 1;
            const int hi = i & 1, hj = j & 1, hk = k & 1;
            float acc[nd];
#pragma unroll
            for (int s = 0; s < nd; s++) acc[s] = 0.f;
            for (int a = 0; a <= hi; a++)
                for (int b = 0; b <= hj; b++)
                    for (int c = 0; c <= (T::is3d ? hk : 0); c++) {
                        const float w = (hi ? 0.5f : 1.f) * (hj ? 0.5f : 1.f) * ((T::is3d && hk) ? 0.5f : 1.f);
                        const long long m = lnode<KIND>(Cc, ci + a, cj + b, ck + c);
#pragma unroll
                        for (int s = 0; s < nd; s++) acc[s] += w * Cc.x[m * nd + s];
                    }
            const long long n = lnode<KIND>(L, i, j, k);
#pragma unroll
            for (int s = 0; s < nd; s++) {
                const long long q = n * nd + s;
                PX[t * nd + s] = L.fixed[q] ? 0.f : L.xt[q] + acc[s];
            }
        }
        __syncthreads();
        stamp(A, tr && A.trace_steps);
        // post-smoothing step 1 on the tile + 1 ring
        auto ldx = [&](long long, int mi, int mj, int mk, float *o) { load_node<nd>(PX, box_at(g2, mi, mj, mk), o); };
        for (int t = threadIdx.x, nv = box_vol(g1); t < nv; t += blockDim.x) {
            int i, j, k;
            box_ijk(g1, t, i, j, k);
            const long long n = lnode<KIND>(L, i, j, k);
            float y[nd];
            apply_node_f<KIND>(L, l, A.Ke, ldx, i, j, k, y);
            const int o = box_at(g2, i, j, k);
#pragma unroll
            for (int s = 0; s < nd; s++) {
                const long long q = n * nd + s;
                const float xv = PX[o * nd + s];
                PR[o * nd + s] = L.fixed[q] ? 0.f : xv + 0.f * (xv - 0.f) + A.omega * (L.b[q] - y[s]) / L.D[q];
            }
        }
        __syncthreads();
        stamp(A, tr && A.trace_steps);
        // post-smoothing step 2 on the own nodes -> L.x
        auto ldt = [&](long long, int mi, int mj, int mk, float *o) { load_node<nd>(PR, box_at(g2, mi, mj, mk), o); };
        const float c2 = A.sm_c2, c3 = A.sm_c3;
        for (int t = threadIdx.x, nv = box_vol(own); t < nv; t += blockDim.x) {
            int i, j, k;
            box_ijk(own, t, i, j, k);
            const long long n = lnode<KIND>(L, i, j, k);
            float y[nd];
            apply_node_f<KIND>(L, l, A.Ke, ldt, i, j, k, y);
            const int o = box_at(g2, i, j, k);
#pragma unroll
            for (int s = 0; s < nd; s++) {
                const long long q = n * nd + s;
                const float xv = PR[o * nd + s], xp = PX[o * nd + s];
                L.x[q] = L.fixed[q] ? 0.f : xv + c2 * (xv - xp) + c3 * (L.b[q] - y[s]) / L.D[q];
            }
        }
        // the caller's view of the result, in a second pass over the same nodes in the same
        // thread order (each thread reads back what it wrote)
        for (int t = threadIdx.x, nv = box_vol(own); t < nv; t += blockDim.x) {
            int i, j, k;
            box_ijk(own, t, i, j, k);
            const long long n = lnode<KIND>(L, i, j, k);
#pragma unroll
            for (int s = 0; s < nd; s++) on(n * nd + s, L.x[n * nd + s]);
        }
    }
    if (A.trace_steps) {
        __syncthreads();
        stamp(A, tr);
    }
    if (barrier) {
        if (!grid_barrier(A.gs, A.partials)) return false;
        stamp(A, tr);
    }
    return true;
}

// Block 0's part of the cycle: the levels from lsmall down and back up, with block barriers.
// When the interface level lsmall sits in shared memory its right-hand side and first sweep
// (written by the grid phases) are copied in first and its result copied out at the end.
template <int KIND>
__device__ void block0_part(const MgFcgArgs &A, const Block0View &V, bool tb) {
    const int nl = A.nlev, ls = A.lsmall;
    const long long bt = threadIdx.x, bs = blockDim.x;
    const bool in_smem = A.lsm <= ls;
    if (in_smem) {
        const MgLev &G = A.L[ls], &S = V.L[ls];
        for (long long t = bt; t < G.ndofs; t += bs) {
            S.b[t] = G.b[t];
            S.x[t] = G.x[t];
        }
        __syncthreads();
    }
    for (int l = ls; l < nl - 1; l++) down_level<KIND>(A, V.L, l, bt, bs, false, tb);
    coarsest_solve(A, V.L, V.Ainv, bt, bs);
    __syncthreads();
    stamp(A, tb);
    for (int l = nl - 2; l >= ls; l--) up_level<KIND>(A, V.L, l, bt, bs, false, tb);
    if (in_smem) {
        __syncthreads();
        const MgLev &G = A.L[ls], &S = V.L[ls];
        for (long long t = bt; t < G.ndofs; t += bs) G.x[t] = S.x[t];
    }
}

// V(2,2)-cycle with the grid levels fused where fuse[l] is set (the others run as three
// phases each); on(q, x) sees the level-0 result of every dof this thread wrote, with no
// barrier after the last sweep (the caller's reduction follows).
template <int KIND, class ON>
__device__ bool vcycle_fused(const MgFcgArgs &A, const Block0View &V, long long tid, long long stride, bool tr, ON on) {
    const int ls = A.lsmall;
    for (int l = 0; l < ls; l++) {
        if (A.fuse[l]) {
            if (!down_fused<KIND>(A, l, tr)) return false;
        } else if (!down_level<KIND>(A, A.L, l, tid, stride, true, tr)) {
            return false;
        }
    }
    if (blockIdx.x == 0) block0_part<KIND>(A, V, tr && A.trace_steps);
    if (!grid_barrier(A.gs, A.partials)) return false;
    stamp(A, tr);
    auto none = [](long long, float) {};
    for (int l = ls - 1; l >= 1; l--) {
        if (A.fuse[l]) {
            if (!up_fused<KIND>(A, l, tr, true, none)) return false;
        } else if (!up_level<KIND>(A, A.L, l, tid, stride, true, tr)) {
            return false;
        }
    }
    if (ls >= 1 && A.fuse[0]) return up_fused<KIND>(A, 0, tr, false, on);
    if (ls >= 1 && !up_level<KIND>(A, A.L, 0, tid, stride, true, tr)) return false;
    // level 0 unfused (or the cycle is the coarsest solve alone): the last node loop wrote
    // the own dofs in the grid-stride order
    const MgLev &L0 = A.L[0];
    for (long long n = tid; n < L0.nnodes; n += stride)
#pragma unroll
        for (int s = 0; s < KT<KIND>::nd; s++) {
            const long long q = n * KT<KIND>::nd + s;
            on(q, L0.x[q]);
        }
    return true;
}

template <int KIND>
__device__ bool vcycle(const MgFcgArgs &A, const Block0View &V, long long tid, long long stride, bool tr) {
    const int ls = A.lsmall;
    for (int l = 0; l < ls; l++)
        if (!down_level<KIND>(A, A.L, l, tid, stride, true, tr)) return false;
    if (blockIdx.x == 0) block0_part<KIND>(A, V, false);
    if (!grid_barrier(A.gs, A.partials)) return false;
    stamp(A, tr);
    for (int l = ls - 1; l >= 0; l--)
        if (!up_level<KIND>(A, A.L, l, tid, stride, true, tr)) return false;
    return true;
}

// q = K v (FP64 matrix-free) for node n; partial v.q returned
template <int KIND>
__device__ __forceinline__ double apply64_node(const MgFcgArgs &A, const double *__restrict__ v, long long n,
                                               double *__restrict__ out) {
    using T = KT<KIND>;
    const MgLev &L = A.L[0];
    int i, j, k;
    lnode_ijk<KIND>(L, n, i, j, k);
    double y[T::nd];
#pragma unroll
    for (int a = 0; a < T::nd; a++) y[a] = 0.0;
#pragma unroll
    for (int ci = 0; ci < 2; ci++)
#pragma unroll
        for (int cj = 0; cj < 2; cj++)
#pragma unroll
            for (int ck = 0; ck < (T::is3d ? 2 : 1); ck++) {
                const int ei = i - 1 + ci, ej = j - 1 + cj, ek = T::is3d ? k - 1 + ck : 0;
                const int li = corner_q(1 - ci, 1 - cj, T::is3d ? 1 - ck : 0);
                const double Ee = A.Ep64[T::is3d ? ((long long)(ei + 1) * (L.ny + 2) + (ej + 1)) * (L.nz + 2) + (ek + 1)
                                                 : (long long)(ei + 1) * (L.ny + 2) + (ej + 1)];
                if (Ee == 0.0) continue;
                double ue[T::nk];
#pragma unroll
                for (int q = 0; q < T::nen; q++) {
                    int qi, qj, qk;
                    corner_of(q, qi, qj, qk);
                    const long long m = lnode<KIND>(L, min(max(ei + qi, 0), L.nx), min(max(ej + qj, 0), L.ny),
                                                    T::is3d ? min(max(ek + qk, 0), L.nz) : 0);
#pragma unroll
                    for (int b = 0; b < T::nd; b++) ue[q * T::nd + b] = v[m * T::nd + b];
                }
#pragma unroll
                for (int a = 0; a < T::nd; a++) {
                    double acc = 0.0;
                    const int row = (li * T::nd + a) * T::nk;
#pragma unroll
                    for (int l = 0; l < T::nk; l++) acc += A.Ke64.v[row + l] * ue[l];
                    y[a] += Ee * acc;
                }
            }
    double d = 0.0;
#pragma unroll
    for (int a = 0; a < T::nd; a++) {
        const long long t = n * T::nd + a;
        const double qv = L.fixed[t] ? 0.0 : y[a];
        out[t] = qv;
        d += v[t] * qv;
    }
    return d;
}

constexpr int kMgThreads = 512;   // one block per SM: half the barrier arrivals of 2 x 256

// q = K v for node n with v, q and the moduli as double words (FP32 pairs): each element's
// K0 u_e row product is a compensated dot product (Ogita, Rump, Oishi, "Accurate sum and dot
// product", SIAM J. Sci. Comput. 26(6), 2005, Dot2: TwoProd + TwoSum per term, with the
// low-order products of K0 = Kh + Kl and v = vh + vl folded into the correction), then
// scaled by E_e and summed over the node's elements in double words.  Returns the partial
// v.q of the node in double words.  Nothing here runs on the FP64 pipe.
template <int KIND, class LD>
__device__ __forceinline__ void applydw_core(const MgFcgArgs &A, LD vload, long long n, dw::D *y) {
    using T = KT<KIND>;
    const MgLev &L = A.L[0];
    int i, j, k;
    lnode_ijk<KIND>(L, n, i, j, k);
#pragma unroll
    for (int a = 0; a < T::nd; a++) y[a] = dw::from_float(0.f);
#pragma unroll
    for (int ci = 0; ci < 2; ci++)
#pragma unroll
        for (int cj = 0; cj < 2; cj++)
#pragma unroll
            for (int ck = 0; ck < (T::is3d ? 2 : 1); ck++) {
                const int ei = i - 1 + ci, ej = j - 1 + cj, ek = T::is3d ? k - 1 + ck : 0;
                const int li = corner_q(1 - ci, 1 - cj, T::is3d ? 1 - ck : 0);
                const float2 Ev = A.Ew[T::is3d ? ((long long)(ei + 1) * (L.ny + 2) + (ej + 1)) * (L.nz + 2) + (ek + 1)
                                               : (long long)(ei + 1) * (L.ny + 2) + (ej + 1)];
                if (Ev.x == 0.f) continue;
                float ps[T::nd], cs[T::nd];
#pragma unroll
                for (int a = 0; a < T::nd; a++) ps[a] = cs[a] = 0.0f;
#pragma unroll
                for (int q = 0; q < T::nen; q++) {
                    int qi, qj, qk;
                    corner_of(q, qi, qj, qk);
                    const long long m = lnode<KIND>(L, min(max(ei + qi, 0), L.nx), min(max(ej + qj, 0), L.ny),
                                                    T::is3d ? min(max(ek + qk, 0), L.nz) : 0);
#pragma unroll
                    for (int b = 0; b < T::nd; b++) {
                        const float2 u = vload(m * T::nd + b);
                        const int l = q * T::nd + b;
#pragma unroll
                        for (int a = 0; a < T::nd; a++) {
                            const int kk = (li * T::nd + a) * T::nk + l;
                            float pe, se;
                            const float pr = dw::two_prod(A.Kds.hi[kk], u.x, pe);
                            ps[a] = dw::two_sum(ps[a], pr, se);
                            cs[a] += se + pe + __fmaf_rn(A.Kds.hi[kk], u.y, A.Kds.lo[kk] * u.x);
                        }
                    }
                }
                const dw::D Ed = dw::make(Ev.x, Ev.y);
#pragma unroll
                for (int a = 0; a < T::nd; a++) {
                    float sl;
                    const float sh = dw::fast_two_sum(ps[a], cs[a], sl);
                    y[a] = dw::add(y[a], dw::mul(Ed, dw::make(sh, sl)));
                }
            }
}

// The same product for an FP32 vector x (exact in double words with a zero low part): the
// low-order term is lo * x alone, and in 2D the 3 x 3 node neighbourhood is read once.
// Per element the terms are summed in the same order as above.
template <int KIND>
__device__ __forceinline__ void applydw_x32(const MgFcgArgs &A, const float *__restrict__ x, long long n, dw::D *y) {
    using T = KT<KIND>;
    if constexpr (T::is3d) {
        applydw_core<KIND>(A, [x](long long t) { return make_float2(x[t], 0.f); }, n, y);
    } else {
        const MgLev &L = A.L[0];
        int i, j, k;
        lnode_ijk<KIND>(L, n, i, j, k);
        float u[3][3][T::nd];
#pragma unroll
        for (int a = 0; a < 3; a++)
#pragma unroll
            for (int b = 0; b < 3; b++) {
                const int mi = min(max(i + a - 1, 0), L.nx), mj = min(max(j + b - 1, 0), L.ny);
                load_node<T::nd>(x, lnode<KIND>(L, mi, mj, 0), u[a][b]);
            }
#pragma unroll
        for (int a = 0; a < T::nd; a++) y[a] = dw::from_float(0.f);
#pragma unroll
        for (int ci = 0; ci < 2; ci++)
#pragma unroll
            for (int cj = 0; cj < 2; cj++) {
                const int ei = i - 1 + ci, ej = j - 1 + cj;
                const int li = corner_q(1 - ci, 1 - cj, 0);
                const float2 Ev = A.Ew[(long long)(ei + 1) * (L.ny + 2) + (ej + 1)];
                if (Ev.x == 0.f) continue;
                float ps[T::nd], cs[T::nd];
#pragma unroll
                for (int a = 0; a < T::nd; a++) ps[a] = cs[a] = 0.0f;
#pragma unroll
                for (int q = 0; q < T::nen; q++) {
                    int qi, qj, qk;
                    corner_of(q, qi, qj, qk);
#pragma unroll
                    for (int b = 0; b < T::nd; b++) {
                        const float uv = u[ci + qi][cj + qj][b];
                        const int l = q * T::nd + b;
#pragma unroll
                        for (int a = 0; a < T::nd; a++) {
                            const int kk = (li * T::nd + a) * T::nk + l;
                            float pe, se;
                            const float pr = dw::two_prod(A.Kds.hi[kk], uv, pe);
                            ps[a] = dw::two_sum(ps[a], pr, se);
                            cs[a] += se + pe + A.Kds.lo[kk] * uv;
                        }
                    }
                }
                const dw::D Ed = dw::make(Ev.x, Ev.y);
#pragma unroll
                for (int a = 0; a < T::nd; a++) {
                    float sl;
                    const float sh = dw::fast_two_sum(ps[a], cs[a], sl);
                    y[a] = dw::add(y[a], dw::mul(Ed, dw::make(sh, sl)));
                }
            }
    }
}

template <int KIND>
__device__ __forceinline__ dw::D applydw_node(const MgFcgArgs &A, const float2 *__restrict__ v, long long n,
                                              float2 *__restrict__ out) {
    using T = KT<KIND>;
    const MgLev &L = A.L[0];
    dw::D y[T::nd];
    applydw_core<KIND>(A, [v](long long t) { return v[t]; }, n, y);
    dw::D d = dw::from_float(0.f);
#pragma unroll
    for (int a = 0; a < T::nd; a++) {
        const long long t = n * T::nd + a;
        const dw::D qv = L.fixed[t] ? dw::from_float(0.f) : y[a];
        out[t] = make_float2(qv.h, qv.l);
        const float2 vv = v[t];
        d = dw::add(d, dw::mul(dw::make(vv.x, vv.y), qv));
    }
    return d;
}

template <int KIND>
__global__ void __launch_bounds__(kMgThreads, 1) mg_fcg_kernel(MgFcgArgs A) {
    grid_sync_init();
    trace_init();
    using T = KT<KIND>;
    __shared__ double sm[32 * 4];
    __shared__ Block0View B0;
    extern __shared__ __align__(16) unsigned char dsm[];
    block0_levels(A, B0, dsm);
    const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long stride = (long long)gridDim.x * blockDim.x;
    const MgLev &L0 = A.L[0];
    // ---- start: r = b - K x0 (x0 = 0 unless warm)
    {
        double acc[2] = {0.0, 0.0};
        if (A.warm) {
            for (long long n = tid; n < L0.nnodes; n += stride) {
                apply64_node<KIND>(A, A.x, n, A.r);   // r = K x (own dofs)
#pragma unroll
                for (int s = 0; s < T::nd; s++) {
                    const long long t = n * T::nd + s;
                    const double bv = L0.fixed[t] ? 0.0 : A.b[t];
                    const double rv = L0.fixed[t] ? 0.0 : bv - A.r[t];
                    A.r[t] = rv;
                    A.p[t] = 0.0;
                    A.q[t] = 0.0;
                    acc[0] += bv * bv;
                    acc[1] += rv * rv;
                }
            }
        } else {
            for (long long n = tid; n < L0.nnodes; n += stride)
#pragma unroll
                for (int s = 0; s < T::nd; s++) {
                    const long long t = n * T::nd + s;
                    const double bv = L0.fixed[t] ? 0.0 : A.b[t];
                    A.x[t] = 0.0;
                    A.r[t] = bv;
                    A.p[t] = 0.0;
                    A.q[t] = 0.0;
                    acc[0] += bv * bv;
                    acc[1] += bv * bv;
                }
        }
        block_sum<2>(acc, sm);
        if (!grid_sync<2, 0>(A.gs, A.partials, acc, 0.0)) return;
    }
    const double bnorm = sqrt(gs_result(A.gs, 0));
    double rr = gs_result(A.gs, 1);
    double rn = sqrt(rr), pq_prev = 1.0;
    int it = 0, conv = (rn <= A.eps * bnorm) ? 1 : 0, cycles = 0;
    for (; !conv && it < A.itmax; it++) {
        // ---- preconditioner: one FP32 V-cycle on r / |r|
        const float sc = (float)(1.0 / rn);
        for (long long n = tid; n < L0.nnodes; n += stride)
#pragma unroll
            for (int s = 0; s < T::nd; s++) {
                const long long t = n * T::nd + s;
                const float bv = L0.fixed[t] ? 0.f : (float)A.r[t] * sc;
                L0.b[t] = bv;
                L0.x[t] = L0.fixed[t] ? 0.f : A.omega * bv / L0.D[t];
            }
        const bool tr = it == A.trace_iter;
        stamp(A, tr);
        if (!grid_barrier(A.gs, A.partials)) return;
        stamp(A, tr);
        if (!vcycle<KIND>(A, B0, tid, stride, tr)) return;
        cycles++;
        // ---- z = |r| V(r/|r|); z.q_prev, z.r, p_prev.r
        double a3[3] = {0.0, 0.0, 0.0};
        for (long long n = tid; n < L0.nnodes; n += stride)
#pragma unroll
            for (int s = 0; s < T::nd; s++) {
                const long long t = n * T::nd + s;
                const double zv = rn * (double)L0.x[t];
                A.z[t] = zv;
                a3[0] += zv * A.q[t];
                a3[1] += zv * A.r[t];
                a3[2] += A.p[t] * A.r[t];
            }
        block_sum<3>(a3, sm);
        if (!grid_sync<3, 0>(A.gs, A.partials, a3, 0.0)) return;
        stamp(A, tr);
        const double beta = it > 0 ? gs_result(A.gs, 0) / pq_prev : 0.0;
        const double pr = gs_result(A.gs, 1) - beta * gs_result(A.gs, 2);
        // ---- p = z - beta p_prev (own dofs, node mapping)
        for (long long n = tid; n < L0.nnodes; n += stride)
#pragma unroll
            for (int s = 0; s < T::nd; s++) {
                const long long t = n * T::nd + s;
                A.p[t] = A.z[t] - beta * A.p[t];
            }
        if (!grid_barrier(A.gs, A.partials)) return;
        stamp(A, tr);
        // ---- q = K p, p.q
        double pq[1] = {0.0};
        for (long long n = tid; n < L0.nnodes; n += stride)
            pq[0] += apply64_node<KIND>(A, A.p, n, A.q);
        block_sum<1>(pq, sm);
        if (!grid_sync<1, 0>(A.gs, A.partials, pq, 0.0)) return;
        stamp(A, tr);
        const double pqv = gs_result(A.gs, 0);
        if (!(pqv > 0.0)) { it++; break; }
        const double alpha = pr / pqv;
        // ---- x += alpha p, r -= alpha q, |r|^2
        double ra[1] = {0.0};
        for (long long n = tid; n < L0.nnodes; n += stride)
#pragma unroll
            for (int s = 0; s < T::nd; s++) {
                const long long t = n * T::nd + s;
                A.x[t] += alpha * A.p[t];
                const double rv = A.r[t] - alpha * A.q[t];
                A.r[t] = rv;
                ra[0] += rv * rv;
            }
        block_sum<1>(ra, sm);
        if (!grid_sync<1, 0>(A.gs, A.partials, ra, 0.0)) return;
        stamp(A, tr);
        rr = gs_result(A.gs, 0);
        rn = sqrt(rr);
        pq_prev = pqv;
        if (rn <= A.eps * bnorm) { it++; conv = 1; break; }
        if (!isfinite(rr)) { it++; break; }
    }
    if (tid == 0) {
        A.out[0] = it;
        A.out[1] = rr;
        A.out[2] = bnorm * bnorm;
        A.out[3] = conv;
        A.out[4] = cycles;
    }
}

// The same flexible CG with its Krylov vectors and operator in double words (FP32
// pairs, ~48-bit significands) instead of FP64: the recurrences keep about 1e-14
// relative accuracy, far below the 1e-8 the solve needs, while every vector update,
// dot product and K p runs on the FP32 pipes (GB300's FP64 rate is a small fraction
// of its FP32 rate; with FP64 vectors the operator alone was a fifth of an iteration).
// Dot products are reduced in double words per warp and in FP64 across warps and
// blocks, in a fixed order.  The FP64 true residual of the result is checked by the
// caller, as for the FP64 kernel.
template <int KIND>
__global__ void __launch_bounds__(kMgThreads, 1) mg_fcg_dw_kernel(MgFcgArgs A) {
    grid_sync_init();
    trace_init();
    using T = KT<KIND>;
    using dw::D;
    __shared__ double sm[32 * 4];
    __shared__ Block0View B0;
    extern __shared__ __align__(16) unsigned char dsm[];
    block0_levels(A, B0, dsm);
    const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long stride = (long long)gridDim.x * blockDim.x;
    const MgLev &L0 = A.L[0];
    float2 *X = A.xw, *R = A.rw, *P = A.pw, *Q = A.qw;
    auto ld = [](const float2 *a, long long t) { const float2 v = a[t]; return dw::make(v.x, v.y); };
    auto st = [](float2 *a, long long t, D v) { a[t] = make_float2(v.h, v.l); };
    // ---- start: moduli in double words; r = b - K x0 in FP64 (x0 = 0 unless warm)
    {
        for (long long e = tid; e < A.npad; e += stride) {
            const D Ed = dw::from_double(A.Ep64[e]);
            A.Ew[e] = make_float2(Ed.h, Ed.l);
        }
        double acc[2] = {0.0, 0.0};
        for (long long n = tid; n < L0.nnodes; n += stride) {
            if (A.warm) apply64_node<KIND>(A, A.x, n, A.r);   // r = K x0 (own dofs)
#pragma unroll
            for (int s = 0; s < T::nd; s++) {
                const long long t = n * T::nd + s;
                const double bv = L0.fixed[t] ? 0.0 : A.b[t];
                const double rv = L0.fixed[t] ? 0.0 : (A.warm ? bv - A.r[t] : bv);
                st(R, t, dw::from_double(rv));
                st(X, t, A.warm && !L0.fixed[t] ? dw::from_double(A.x[t]) : dw::from_float(0.f));
                st(P, t, dw::from_float(0.f));
                st(Q, t, dw::from_float(0.f));
                acc[0] += bv * bv;
                acc[1] += rv * rv;
            }
        }
        block_sum<2>(acc, sm);
        if (!grid_sync<2, 0>(A.gs, A.partials, acc, 0.0)) return;
    }
    const double bnorm = sqrt(gs_result(A.gs, 0));
    double rr = gs_result(A.gs, 1);
    double rn = sqrt(rr), pq_prev = 1.0;
    int it = 0, conv = (rn <= A.eps * bnorm) ? 1 : 0, cycles = 0;
    // The cycle's input is r scaled by 1 / rs, rs the residual norm known when r was formed (the
    // current one before the first cycle, the previous one after), so the input is formed in
    // the update phase that forms r; z = rs V(r / rs).
    double rs = rn;
    if (!conv) {
        const float sc = (float)(1.0 / rs);
        for (long long n = tid; n < L0.nnodes; n += stride)
#pragma unroll
            for (int s = 0; s < T::nd; s++) {
                const long long t = n * T::nd + s;
                const float2 rv = R[t];
                const float bv = L0.fixed[t] ? 0.f : rv.x * sc + rv.y * sc;
                L0.b[t] = bv;
                L0.x[t] = L0.fixed[t] ? 0.f : A.omega * bv / L0.D[t];
            }
        if (!grid_barrier(A.gs, A.partials)) return;
    }
    for (; !conv && it < A.itmax; it++) {
        const bool tr = it == A.trace_iter;
        stamp(A, tr);
        // ---- preconditioner: one FP32 V-cycle; z = rs x (never stored); z.q_prev, z.r, p_prev.r
        const D rsD = dw::from_double(rs);
        D a3[3] = {dw::from_float(0.f), dw::from_float(0.f), dw::from_float(0.f)};
        auto on = [&](long long t, float xv) {
            const D zv = dw::mulf(rsD, xv);
            a3[0] = dw::add(a3[0], dw::mul(zv, ld(Q, t)));
            a3[1] = dw::add(a3[1], dw::mul(zv, ld(R, t)));
            a3[2] = dw::add(a3[2], dw::mul(ld(P, t), ld(R, t)));
        };
        if (!vcycle_fused<KIND>(A, B0, tid, stride, tr, on)) return;
        cycles++;
        double s3[3] = {0.0, 0.0, 0.0};
        dw::block_sum_dw<3>(a3, s3, sm);
        if (A.trace_steps) {
            __syncthreads();
            stamp(A, tr);
        }
        if (!grid_sync<3, 0>(A.gs, A.partials, s3, 0.0)) return;
        stamp(A, tr);
        const double beta = it > 0 ? gs_result(A.gs, 0) / pq_prev : 0.0;
        const double pr = gs_result(A.gs, 1) - beta * gs_result(A.gs, 2);
        const D betaD = dw::from_double(beta);
        // ---- p = z - beta p_prev and q = K p = rs K x - beta q_prev (K applied to the cycle's
        //      FP32 result, exact in double words), p.q
        D pqd[1] = {dw::from_float(0.f)};
        const float *X0 = L0.x;
        for (long long n = tid; n < L0.nnodes; n += stride) {
            D y[T::nd];
            applydw_x32<KIND>(A, X0, n, y);
#pragma unroll
            for (int s = 0; s < T::nd; s++) {
                const long long t = n * T::nd + s;
                const D pv = dw::sub(dw::mulf(rsD, X0[t]), dw::mul(betaD, ld(P, t)));
                const D qv = L0.fixed[t] ? dw::from_float(0.f) : dw::sub(dw::mul(rsD, y[s]), dw::mul(betaD, ld(Q, t)));
                st(P, t, pv);
                st(Q, t, qv);
                pqd[0] = dw::add(pqd[0], dw::mul(pv, qv));
            }
        }
        if (A.trace_steps) {
            __syncthreads();
            stamp(A, tr);
        }
        double pq[1] = {0.0};
        dw::block_sum_dw<1>(pqd, pq, sm);
        if (!grid_sync<1, 0>(A.gs, A.partials, pq, 0.0)) return;
        stamp(A, tr);
        const double pqv = gs_result(A.gs, 0);
        if (!(pqv > 0.0)) { it++; break; }
        const D alphaD = dw::from_double(pr / pqv);
        // ---- x += alpha p, r -= alpha q, |r|^2; the next cycle's input r / |r_prev| and its
        //      first sweep
        const float sc = (float)(1.0 / rn);
        D rad[1] = {dw::from_float(0.f)};
        // two nodes per pass, every load of both issued before the arithmetic
        for (long long n0 = tid; n0 < L0.nnodes; n0 += 2 * stride) {
            constexpr int nd = T::nd;
            const bool two = n0 + stride < L0.nnodes;
            float2 xv[2][nd], pv[2][nd], rv[2][nd], qv[2][nd];
            float dv[2][nd];
            unsigned char fx[2][nd];
#pragma unroll
            for (int h = 0; h < 2; h++)
#pragma unroll
                for (int s = 0; s < nd; s++) {
                    const long long t = (n0 + (h ? stride : 0)) * nd + s;
                    const bool on = h == 0 || two;
                    xv[h][s] = on ? X[t] : make_float2(0.f, 0.f);
                    pv[h][s] = on ? P[t] : make_float2(0.f, 0.f);
                    rv[h][s] = on ? R[t] : make_float2(0.f, 0.f);
                    qv[h][s] = on ? Q[t] : make_float2(0.f, 0.f);
                    dv[h][s] = on ? L0.D[t] : 1.f;
                    fx[h][s] = on ? L0.fixed[t] : 1;
                }
#pragma unroll
            for (int h = 0; h < 2; h++) {
                if (h == 1 && !two) break;
#pragma unroll
                for (int s = 0; s < nd; s++) {
                    const long long t = (n0 + (h ? stride : 0)) * nd + s;
                    st(X, t, dw::add(dw::make(xv[h][s].x, xv[h][s].y), dw::mul(alphaD, dw::make(pv[h][s].x, pv[h][s].y))));
                    const D r1 = dw::sub(dw::make(rv[h][s].x, rv[h][s].y), dw::mul(alphaD, dw::make(qv[h][s].x, qv[h][s].y)));
                    st(R, t, r1);
                    rad[0] = dw::add(rad[0], dw::sq(r1));
                    const float bv = fx[h][s] ? 0.f : r1.h * sc + r1.l * sc;
                    L0.b[t] = bv;
                    L0.x[t] = fx[h][s] ? 0.f : A.omega * bv / dv[h][s];
                }
            }
        }
        if (A.trace_steps) {
            __syncthreads();
            stamp(A, tr);
        }
        double ra[1] = {0.0};
        dw::block_sum_dw<1>(rad, ra, sm);
        if (!grid_sync<1, 0>(A.gs, A.partials, ra, 0.0)) return;
        stamp(A, tr);
        rs = rn;
        rr = gs_result(A.gs, 0);
        rn = sqrt(rr);
        pq_prev = pqv;
        if (rn <= A.eps * bnorm) { it++; conv = 1; break; }
        if (!isfinite(rr)) { it++; break; }
    }
    // ---- the solution in FP64 for the caller (own dofs)
    for (long long n = tid; n < L0.nnodes; n += stride)
#pragma unroll
        for (int s = 0; s < T::nd; s++) {
            const long long t = n * T::nd + s;
            A.x[t] = dw::to_double(ld(X, t));
        }
    if (tid == 0) {
        A.out[0] = it;
        A.out[1] = rr;
        A.out[2] = bnorm * bnorm;
        A.out[3] = conv;
        A.out[4] = cycles;
    }
}

// One V-cycle as a standalone preconditioner application (the learned
// solver's global stage): r32 = r, x = |r| V(r / |r|) in FP32.  Returns at
// once (every block) when *flags != 0.
template <int KIND>
__global__ void __launch_bounds__(kMgThreads, 1) mg_apply_kernel(MgFcgArgs A, const double *__restrict__ r,
                                                                 float *__restrict__ r32, float *__restrict__ xo,
                                                                 const int *flags) {
    using T = KT<KIND>;
    if (flags && *(volatile const int *)flags) return;
    grid_sync_init();
    __shared__ double sm[32 * 4];
    __shared__ Block0View B0;
    extern __shared__ __align__(16) unsigned char dsm[];
    block0_levels(A, B0, dsm);
    const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long stride = (long long)gridDim.x * blockDim.x;
    const MgLev &L0 = A.L[0];
    double acc[1] = {0.0};
    for (long long t = tid; t < L0.ndofs; t += stride) {
        const double rv = L0.fixed[t] ? 0.0 : r[t];
        r32[t] = (float)rv;
        acc[0] += rv * rv;
    }
    block_sum<1>(acc, sm);
    if (!grid_sync<1, 0>(A.gs, A.partials, acc, 0.0)) return;
    const double rn = sqrt(gs_result(A.gs, 0));
    if (!(rn > 0.0)) {
        for (long long t = tid; t < L0.ndofs; t += stride) xo[t] = 0.0f;
        return;
    }
    const float sc = (float)(1.0 / rn);
    for (long long n = tid; n < L0.nnodes; n += stride)
#pragma unroll
        for (int s = 0; s < T::nd; s++) {
            const long long t = n * T::nd + s;
            const float bv = L0.fixed[t] ? 0.f : (float)r[t] * sc;
            L0.b[t] = bv;
            L0.x[t] = L0.fixed[t] ? 0.f : A.omega * bv / L0.D[t];
        }
    if (!grid_barrier(A.gs, A.partials)) return;
    vcycle_fused<KIND>(A, B0, tid, stride, false,
                       [&](long long t, float xv) { xo[t] = L0.fixed[t] ? 0.0f : (float)(rn * (double)xv); });
}

// ------------------------------------------------------------------ host side
// levels at most this large run in one block: on the 1025 x 513-node MBB grid, block 0 from
// the 561-node level on takes 230 us per FCG iteration, from the 2,145-node level 267 us,
// from the 153-node level 242 us (a level on the grid costs two or six barriers, a level in
// block 0 runs one SM's worth of threads)
constexpr long long kSmallLevelNodes = 1024;

// first level (>= 1) that block 0 runs alone (PSF_MG_SMALL_NODES overrides the size)
static int mg_small_level(const MgHier *H) {
    const char *e = getenv("PSF_MG_SMALL_NODES");
    const long long lim = e && *e ? atoll(e) : kSmallLevelNodes;
    for (int l = 1; l < H->nlev - 1; l++)
        if (H->L[l].nnodes <= lim) return l;
    return H->nlev - 1;
}

constexpr size_t kMaxDynSmem = 200 * 1024;   // the MG kernels' dynamic shared memory limit (set once per setup)

// Block 0's shared-memory levels: from the coarsest level up, as many whole levels from
// lsmall on and the coarsest inverse as fit in PSF_MG_SMEM_KB (default 160) KB of dynamic
// shared memory.  The interface level lsmall, which the grid phases write and read in global
// memory, is copied in and out around block 0's part of the cycle.
// Fills a->lsm, a->smo, a->smo_ainv; returns the bytes.
static size_t mg_block0_layout(const Ctx *c, const MgHier *H, MgFcgArgs *a) {
    const int nd = c->ndof;
    a->nslot = (c->kind == PSF_H8_SOLID ? 27 : 9) * nd * nd;
    const char *e = getenv("PSF_MG_SMEM_KB");
    size_t budget = (size_t)(e ? atof(e) : 160.0) * 1024;
    if (budget > kMaxDynSmem) budget = kMaxDynSmem;
    auto al = [](size_t v) { return (v + 15) & ~(size_t)15; };
    auto level_bytes = [&](int l) {
        const MgLev &L = H->L[l];
        return al((size_t)L.nnodes * a->nslot * 4) + 5 * al((size_t)L.ndofs * 4) + al((size_t)L.ndofs);
    };
    const size_t ainv = al((size_t)H->nc * H->nc * 8);
    a->lsm = H->nlev;
    a->smo_ainv = -1;
    size_t total = ainv;
    if (total > budget) return 0;
    int lsm = H->nlev;
    // the interface level lsmall joins them only when PSF_MG_SMEM_IFACE=1: its 80 KB of
    // stencil at 1024x512 cost the grid phases more L1 than block 0 gains (236.6 vs 209.5 us
    // per FCG iteration)
    const char *ei = getenv("PSF_MG_SMEM_IFACE");
    const int lo = (ei && *ei == '1') ? a->lsmall : a->lsmall + 1;
    for (int l = H->nlev - 1; l >= lo && l >= 1; l--) {
        if (total + level_bytes(l) > budget) break;
        total += level_bytes(l);
        lsm = l;
    }
    size_t off = 0;
    a->smo_ainv = (int)off;
    off += ainv;
    for (int l = lsm; l < H->nlev; l++) {
        const MgLev &L = H->L[l];
        a->smo[l][0] = (int)off; off += al((size_t)L.nnodes * a->nslot * 4);
        for (int k = 1; k <= 5; k++) { a->smo[l][k] = (int)off; off += al((size_t)L.ndofs * 4); }
        a->smo[l][6] = (int)off; off += al((size_t)L.ndofs);
    }
    a->lsm = lsm;
    return off;
}

static psf_status mg_alloc(MgHier *H, Ctx *c, void **p, size_t bytes) {
    PSF_CUDA(cudaMalloc(p, bytes ? bytes : 1));
    PSF_CUDA(cudaMemsetAsync(*p, 0, bytes ? bytes : 1, c->stream));
    H->allocs.push_back(*p);
    return PSF_OK;
}

static KeF kef_of(const Ctx *c) {
    KeF k{};
    const int nk = c->nen * c->ndof;
    for (int q = 0; q < nk * nk; q++) k.v[q] = (float)c->Ke0_host[q];
    return k;
}

static psf_status mg_build_hierarchy(Ctx *c) {
    MgHier *H = new MgHier;
    c->mg = H;
    const bool is3d = c->kind == PSF_H8_SOLID;
    const int nd = c->ndof, nk = c->nen * c->ndof;
    MgLev &L0 = H->L[0];
    L0.nx = c->nx; L0.ny = c->ny; L0.nz = c->nz;
    L0.nnodes = c->nnodes; L0.ndofs = c->ndofs; L0.ne = c->ne;
    L0.K = nullptr; L0.Ep = c->Epadf; L0.D = c->Dl1f; L0.fixed = c->fixed;
    int nl = 1;
    while (nl < kMaxLev) {
        const MgLev &F = H->L[nl - 1];
        if (nl > 1 && F.ndofs <= kCoarseDofs) break;
        if (F.nx < 2 || F.ny < 2 || (is3d && F.nz < 2)) break;
        MgLev &Cc = H->L[nl];
        Cc.nx = (F.nx + 1) / 2; Cc.ny = (F.ny + 1) / 2; Cc.nz = is3d ? (F.nz + 1) / 2 : 0;
        Cc.nnodes = is3d ? (long long)(Cc.nx + 1) * (Cc.ny + 1) * (Cc.nz + 1) : (long long)(Cc.nx + 1) * (Cc.ny + 1);
        Cc.ndofs = Cc.nnodes * nd;
        Cc.ne = is3d ? (long long)Cc.nx * Cc.ny * Cc.nz : (long long)Cc.nx * Cc.ny;
        PSF_CHECK(mg_alloc(H, c, (void **)&Cc.K, sizeof(float) * Cc.ne * nk * nk));
        PSF_CHECK(mg_alloc(H, c, (void **)&Cc.S, sizeof(float) * Cc.nnodes * (is3d ? 27 : 9) * nd * nd));
        PSF_CHECK(mg_alloc(H, c, (void **)&Cc.D, sizeof(float) * Cc.ndofs));
        PSF_CHECK(mg_alloc(H, c, (void **)&Cc.fixed, Cc.ndofs));
        Cc.Ep = nullptr;
        nl++;
    }
    H->nlev = nl;
    for (int l = 0; l < nl; l++) {
        MgLev &L = H->L[l];
        PSF_CHECK(mg_alloc(H, c, (void **)&L.x, sizeof(float) * L.ndofs));
        PSF_CHECK(mg_alloc(H, c, (void **)&L.xt, sizeof(float) * L.ndofs));
        PSF_CHECK(mg_alloc(H, c, (void **)&L.r, sizeof(float) * L.ndofs));
        PSF_CHECK(mg_alloc(H, c, (void **)&L.b, sizeof(float) * L.ndofs));
    }
    if (nl < 2) { set_error("multigrid needs a grid of at least 2 elements per axis"); return PSF_BAD_INPUT; }
    H->nc = (int)H->L[nl - 1].ndofs;
    if (H->nc > 4096) { set_error("multigrid coarsest level too large for the dense solve (an axis of 1 element stops the coarsening: aspect ratio too large)"); return PSF_BAD_INPUT; }
    PSF_CHECK(mg_alloc(H, c, (void **)&H->Ac, sizeof(double) * (size_t)H->nc * H->nc));
    return PSF_OK;
}

template <int KIND>
static psf_status mg_setup_t(Ctx *c, MgHier *H) {
    KeF Ke = kef_of(c);
    for (int l = 1; l < H->nlev; l++) {
        MgLev &F = H->L[l - 1], &Cc = H->L[l];
        (coarse_fixed_kernel<KIND><<<grid_for(Cc.nnodes, 256, 65536), 256, 0, c->stream>>>(
             F, Cc),
         ::psf::note_launch());
        (galerkin_kernel<KIND><<<grid_for(Cc.ne, 64, 65536), 64, 0, c->stream>>>(
             F, Cc, l - 1, Ke),
         ::psf::note_launch());
        (coarse_stencil_kernel<KIND><<<grid_for(Cc.nnodes, 128, 65536), 128, 0, c->stream>>>(Cc), ::psf::note_launch());
        PSF_CUDA(cudaGetLastError());
    }
    MgLev &Lc = H->L[H->nlev - 1];
    const int n = H->nc;
    PSF_CUDA(cudaMemsetAsync(H->Ac, 0, sizeof(double) * (size_t)n * n, c->stream));
    (coarse_dense_kernel<KIND><<<grid_for(Lc.ne, 128, 4096), 128, 0, c->stream>>>(Lc, H->Ac, n), ::psf::note_launch());
    (dense_fix_identity<<<grid_for(n, 128), 128, 0, c->stream>>>(H->Ac, Lc.fixed, n), ::psf::note_launch());
    (gauss_jordan_kernel<<<1, 1024, 0, c->stream>>>(H->Ac, n), ::psf::note_launch());
    PSF_CUDA(cudaGetLastError());
    // the solver kernels may use all the dynamic shared memory a block can opt into (block 0's
    // levels, the fused levels' buffers); set here, outside any stream capture of their launches
    int dev = 0, optin = 0;
    PSF_CUDA(cudaGetDevice(&dev));
    PSF_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    size_t max_dyn = (size_t)optin;
    const void *fns[3] = {(const void *)mg_fcg_kernel<KIND>, (const void *)mg_fcg_dw_kernel<KIND>,
                          (const void *)mg_apply_kernel<KIND>};
    for (const void *fn : fns) {
        cudaFuncAttributes fa;
        PSF_CUDA(cudaFuncGetAttributes(&fa, fn));
        max_dyn = std::min(max_dyn, (size_t)optin - fa.sharedSizeBytes);
    }
    max_dyn &= ~(size_t)15;
    for (const void *fn : fns)
        PSF_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)max_dyn));
    H->max_dyn = max_dyn;
    return PSF_OK;
}

static psf_status mg_setup(Ctx *c) {
    if (!c->mg) PSF_CHECK(mg_build_hierarchy(c));
    MgHier *H = (MgHier *)c->mg;
    H->L[0].Ep = c->Epadf;
    H->L[0].D = c->Dl1f;
    switch (c->kind) {
    case PSF_Q4_PLANE_STRAIN: return mg_setup_t<0>(c, H);
    case PSF_Q4_HEAT: return mg_setup_t<1>(c, H);
    default: return mg_setup_t<2>(c, H);
    }
}

// Smoother of the V(2,2) cycle: degree-2 Chebyshev on [1/ratio, 1] in the l1-Jacobi
// preconditioned operator D^-1 A (the l1 row sums bound its spectrum by 1, so the upper
// end is rigorous).  Measured on the 1M-dof MBB trajectory (100 SIMP iterations, flexible
// CG to 1e-8): Krylov iterations 14,793 with two plain l1-Jacobi steps, 12,486 / 11,558 /
// 11,298 / 11,002 / 10,769 / 10,663 / 10,618 with ratio 3 / 6 / 8 / 12 / 20 / 30 / 50, at
// the same cost per cycle; on the 128x64x64 H8 cantilever (30 iterations) 2,778 with
// l1-Jacobi, 2,034 / 1,909 / 1,880 with ratio 8 / 20 / 40.  PSF_MG_CHEB=<ratio> overrides
// the default; a ratio <= 1 selects plain l1-Jacobi (omega = 1, convergent for any SPD
// operator).
constexpr double kChebRatio = 40.0;
static void mg_smoother(MgFcgArgs *a) {
    a->omega = 1.0f;
    a->sm_c2 = 0.0f;
    a->sm_c3 = 1.0f;
    const char *e = getenv("PSF_MG_CHEB");
    const double ratio = e ? atof(e) : kChebRatio;
    if (ratio > 1.0) {
        const double lo = 1.0 / ratio, hi = 1.0;
        const double theta = 0.5 * (hi + lo), delta = 0.5 * (hi - lo), sigma = theta / delta;
        const double rho0 = 1.0 / sigma, rho1 = 1.0 / (2.0 * sigma - rho0);
        a->omega = (float)(1.0 / theta);
        a->sm_c2 = (float)(rho1 * rho0);
        a->sm_c3 = (float)(2.0 * rho1 / delta);
    }
}

// Tiles of the fused grid levels for a launch of `blocks` blocks: per level the tile grid
// (at most one tile per block) whose grown tile (two rings) is smallest.  In 2D every grid
// level is fused (1025 x 513-node MBB: 209.5 us per FCG iteration, 221.2 us with the
// 65 x 33-node level in three phases, 270 us with none fused; 513 x 513-node heat sink: 105,
// 113 and 136 us); in 3D, where the rings are thicker in proportion, a level is fused when its
// grown tile holds at most 1.35x (level 0) or 3x (coarser levels) the own nodes (65 x 33 x 33
// nodes: 245 us either way, 254 us with every level fused).  PSF_MG_FUSE=0 runs every level in
// three phases, =2 fuses every grid level, =3 applies the size rule in 2D too.
// The buffers of a fused level go to dynamic shared memory, after block 0's levels
// (*smem bytes on entry, the launch's total on return), where both fit in max_dyn bytes.
static psf_status mg_tiles(Ctx *c, MgHier *H, MgFcgArgs *a, int blocks, size_t max_dyn, size_t *smem) {
    const bool is3d = c->kind == PSF_H8_SOLID;
    const char *e = getenv("PSF_MG_FUSE");
    const int mode = e && *e ? atoi(e) : 1;
    long long half = 0, half_sm = 0;
    const size_t off = (*smem + 15) & ~(size_t)15;
    const size_t avail = max_dyn > off ? max_dyn - off : 0;
    const char *ets = getenv("PSF_MG_TILE_SMEM");
    const bool tile_smem = !(ets && *ets == '0');   // 0: the tile buffers in global memory
    for (int l = 0; l < kMaxLev; l++) {
        a->fuse[l] = 0;
        a->tsm[l] = 0;
        for (int d = 0; d < 3; d++) a->tg[l][d] = a->ts[l][d] = 1;
    }
    for (int l = 0; l < a->lsmall && l < H->nlev - 1; l++) {
        const MgLev &L = H->L[l];
        const long long N[3] = {L.nx + 1, L.ny + 1, is3d ? L.nz + 1 : 1};
        long long best = -1;
        int bt[3] = {1, 1, 1};
        for (long long ti = 1; ti <= blocks && ti <= N[0]; ti++)
            for (long long tj = 1; ti * tj <= blocks && tj <= N[1]; tj++)
                for (long long tk = 1; ti * tj * tk <= blocks && tk <= N[2]; tk++) {
                    const long long si = (N[0] + ti - 1) / ti, sj = (N[1] + tj - 1) / tj, sk = (N[2] + tk - 1) / tk;
                    const long long cost = (si + 4) * (sj + 4) * (is3d ? sk + 4 : 1);
                    if (best < 0 || cost < best) {
                        best = cost;
                        bt[0] = (int)ti; bt[1] = (int)tj; bt[2] = (int)tk;
                    }
                }
        const long long s0 = (N[0] + bt[0] - 1) / bt[0], s1 = (N[1] + bt[1] - 1) / bt[1], s2 = (N[2] + bt[2] - 1) / bt[2];
        const double ratio = (double)best / (double)(s0 * s1 * s2);
        const bool by_size = ratio <= (l == 0 ? 1.35 : 3.0);
        const bool f = mode == 0 ? false : (mode == 2 || (mode == 1 && !is3d) ? true : by_size);
        a->fuse[l] = f ? 1 : 0;
        a->tg[l][0] = bt[0]; a->tg[l][1] = bt[1]; a->tg[l][2] = bt[2];
        a->ts[l][0] = (int)s0; a->ts[l][1] = (int)s1; a->ts[l][2] = (int)s2;
        if (!f) continue;
        const long long need = ((best * c->ndof) + 3) & ~3ll;   // floats per buffer, 16-byte multiple
        if (tile_smem && (size_t)need * 2 * sizeof(float) <= avail) {
            a->tsm[l] = 1;
            half_sm = std::max(half_sm, need);
        } else {
            half = std::max(half, need);
        }
    }
    half = (half + 31) & ~31ll;
    const size_t bytes = (size_t)blocks * 2 * (size_t)half * sizeof(float);
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    PSF_CUDA(cudaStreamIsCapturing(c->stream, &cap));
    if (bytes > H->tbuf_bytes && cap != cudaStreamCaptureStatusNone) {
        // no allocation inside a stream capture: the levels that would need global buffers
        // run in three phases
        for (int l = 0; l < kMaxLev; l++)
            if (a->fuse[l] && !a->tsm[l]) a->fuse[l] = 0;
        half = 0;
    } else if (bytes > H->tbuf_bytes) {
        PSF_CHECK(mg_alloc(H, c, (void **)&H->tbuf, bytes));
        H->tbuf_bytes = bytes;
    }
    a->tbuf = H->tbuf;
    a->tbuf_half = half;
    a->tsm_off = (int)off;
    a->tsm_half = (int)half_sm;
    if (half_sm > 0) *smem = off + (size_t)half_sm * 2 * sizeof(float);
    return PSF_OK;
}

template <int KIND>
static psf_status mg_fcg_t(Ctx *c, MgFcgArgs &a, double *h, bool dwords, size_t smem) {
    const void *fn = dwords ? (const void *)mg_fcg_dw_kernel<KIND> : (const void *)mg_fcg_kernel<KIND>;
    int per_sm = 0;
    PSF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kMgThreads, smem));
    if (per_sm < 1) { set_error("multigrid kernel does not fit on an SM"); return PSF_CUDA_ERROR; }
    int blocks = c->num_sms * (per_sm < 2 ? per_sm : 2);
    long long need = (c->nnodes + kMgThreads - 1) / kMgThreads;
    if (blocks > need) blocks = (int)need;
    if (blocks < 1) blocks = 1;
    PSF_CHECK(mg_tiles(c, (MgHier *)c->mg, &a, blocks, ((MgHier *)c->mg)->max_dyn, &smem));
    void *args[] = {&a};
    PSF_CUDA(cudaEventRecord(c->evk0, c->stream));
    PSF_CHECK(launch_coop(c, fn, blocks, kMgThreads, args, smem));
    PSF_CUDA(cudaEventRecord(c->evk1, c->stream));
    PSF_CHECK(read_sync_status(c));
    PSF_CHECK(add_kernel_time(c));
    PSF_CUDA(cudaMemcpyAsync(h, a.out, 5 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    PSF_CUDA(cudaStreamSynchronize(c->stream));
    return PSF_OK;
}

// PSF_SOLVE_IR_MG_F32: the whole solve in one persistent launch (a second one
// only if the FP64 true residual disagrees with the recurrence).  An FP32 inner
// solve inside FP64 iterative refinement was measured as the alternative: on the
// 1M-dof MBB trajectory it needed 5.7x the Krylov iterations and missed 1e-8 on
// some designs (the FP32 recurrence stalls at the SIMP contrast), so the flexible
// CG stays in FP64 with the FP32 V-cycle as its preconditioner.
psf_status mg_solve(Ctx *c, int itmax, double eps, bool warm, psf_solve_info *info) {
    PSF_CHECK(mg_setup(c));
    MgHier *H = (MgHier *)c->mg;
    MgFcgArgs *a = new MgFcgArgs;
    a->nlev = H->nlev;
    a->lsmall = mg_small_level(H);
    for (int l = 0; l < H->nlev; l++) a->L[l] = H->L[l];
    a->Ke = kef_of(c);
    const int nk = c->nen * c->ndof;
    for (int q = 0; q < nk * nk; q++) {
        a->Ke64.v[q] = c->Ke0_host[q];
        const float h = (float)c->Ke0_host[q];
        a->Kds.hi[q] = h;
        a->Kds.lo[q] = (float)(c->Ke0_host[q] - (double)h);
    }
    a->Ainv = H->Ac;
    a->nc = H->nc;
    mg_smoother(a);
    a->Ep64 = c->Epad;
    a->b = c->Fn;
    a->x = c->w64[5]; a->r = c->w64[6]; a->z = c->w64[7]; a->p = c->w64[1]; a->q = c->w64[2];
    a->itmax = itmax;
    a->eps = eps;
    a->gs = c->gs;
    a->partials = c->partials;
    a->out = c->scal + 12;
    // optional per-phase trace of the third iteration (PSF_MG_TRACE=<file>)
    const char *trace_path = getenv("PSF_MG_TRACE");
    a->trace = nullptr;
    a->trace_iter = 2;
    a->trace_steps = getenv("PSF_MG_TRACE_STEPS") ? 1 : 0;
    if (trace_path && *trace_path) {
        if (!H->trace) PSF_CHECK(mg_alloc(H, c, (void **)&H->trace, sizeof(unsigned long long) * 1001));
        PSF_CUDA(cudaMemsetAsync(H->trace, 0, sizeof(unsigned long long) * 1001, c->stream));
        a->trace = H->trace;
    }
    if (warm) PSF_CUDA(cudaMemcpyAsync(a->x, c->un, sizeof(double) * c->ndofs, cudaMemcpyDeviceToDevice, c->stream));
    a->warm = warm ? 1 : 0;
    // Krylov vectors in double words unless PSF_MG_FCG_F64=1 (FP64 vectors and operator)
    const char *f64env = getenv("PSF_MG_FCG_F64");
    const bool dwords = !(f64env && *f64env == '1');
    if (dwords && !H->xw) {
        const MgLev &L0 = H->L[0];
        H->npad = (c->kind == PSF_H8_SOLID) ? (long long)(L0.nx + 2) * (L0.ny + 2) * (L0.nz + 2)
                                            : (long long)(L0.nx + 2) * (L0.ny + 2);
        PSF_CHECK(mg_alloc(H, c, (void **)&H->xw, sizeof(float2) * c->ndofs));
        PSF_CHECK(mg_alloc(H, c, (void **)&H->rw, sizeof(float2) * c->ndofs));
        PSF_CHECK(mg_alloc(H, c, (void **)&H->pw, sizeof(float2) * c->ndofs));
        PSF_CHECK(mg_alloc(H, c, (void **)&H->qw, sizeof(float2) * c->ndofs));
        PSF_CHECK(mg_alloc(H, c, (void **)&H->Ew, sizeof(float2) * H->npad));
    }
    a->xw = H->xw; a->rw = H->rw; a->pw = H->pw; a->qw = H->qw; a->Ew = H->Ew; a->npad = H->npad;
    const size_t smem = mg_block0_layout(c, H, a);
    int total = 0, cycles = 0, launches = 0;
    bool ok = false;
    double h[5] = {0, 0, 0, 0, 0};
    psf_status st = PSF_OK;
    for (int pass = 0; pass < 3 && total < itmax; pass++) {
        a->itmax = itmax - total;
        switch (c->kind) {
        case PSF_Q4_PLANE_STRAIN: st = mg_fcg_t<0>(c, *a, h, dwords, smem); break;
        case PSF_Q4_HEAT: st = mg_fcg_t<1>(c, *a, h, dwords, smem); break;
        default: st = mg_fcg_t<2>(c, *a, h, dwords, smem); break;
        }
        if (st != PSF_OK) break;
        launches++;
        total += (int)h[0];
        cycles += (int)h[4];
        if (h[3] == 0.0) break;
        // confirm on the FP64 true residual; restart from x if the recurrence drifted
        double rn, bn;
        PSF_CHECK(residual64_check(c, c->Fn, a->x, c->w64[3], &rn, &bn));
        if (bn == 0.0 || rn <= eps * bn) { ok = true; break; }
        a->warm = 1;
    }
    delete a;
    if (st != PSF_OK) return st;
    if (trace_path && *trace_path && H->trace) {
        std::vector<unsigned long long> t(1001);
        PSF_CUDA(cudaMemcpy(t.data(), H->trace, sizeof(unsigned long long) * 1001, cudaMemcpyDeviceToHost));
        FILE *fh = fopen(trace_path, "a");
        if (fh) {
            fprintf(fh, "levels %d phases %llu ns:", H->nlev, t[0]);
            for (unsigned long long k = 1; k < t[0] && k < 1001; k++) fprintf(fh, " %llu", t[k + 1] - t[k]);
            fprintf(fh, "\n");
            fclose(fh);
        }
    }
    PSF_CUDA(cudaMemcpyAsync(c->un, c->w64[5], sizeof(double) * c->ndofs, cudaMemcpyDeviceToDevice, c->stream));
    PSF_CHECK(gather_reduced(c, c->un, c->u));
    info->iterations = total;
    info->outer_iterations = launches;
    info->rel_residual_recurrence = h[2] > 0 ? sqrt(h[1] / h[2]) : 0.0;
    return ok ? PSF_OK : PSF_NOT_CONVERGED;
}

psf_status mg_free(Ctx *c) {
    MgHier *H = (MgHier *)c->mg;
    if (!H) return PSF_OK;
    for (void *p : H->allocs) cudaFree(p);
    delete H;
    c->mg = nullptr;
    return PSF_OK;
}


}  // namespace psf

namespace psf {
// the Galerkin hierarchy of the current design (once per design, before mg_apply)
psf_status mg_prepare(Ctx *c) { return mg_setup(c); }

template <int KIND>
static psf_status mg_apply_t(Ctx *c, const double *r, float *r32, float *xo, const int *flags) {
    MgHier *H = (MgHier *)c->mg;
    MgFcgArgs *a = new MgFcgArgs;
    a->nlev = H->nlev;
    a->lsmall = mg_small_level(H);
    for (int l = 0; l < H->nlev; l++) a->L[l] = H->L[l];
    a->Ke = kef_of(c);
    const int nk = c->nen * c->ndof;
    for (int q = 0; q < nk * nk; q++) a->Ke64.v[q] = c->Ke0_host[q];
    a->Ainv = H->Ac;
    a->nc = H->nc;
    mg_smoother(a);
    const size_t smem = mg_block0_layout(c, H, a);
    a->Ep64 = c->Epad;
    a->gs = c->gs;
    a->partials = c->partials;
    a->trace = nullptr;
    a->trace_iter = -1;
    a->trace_steps = 0;
    int per_sm = 0;
    psf_status st = cuda_status(
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, mg_apply_kernel<KIND>, kMgThreads, smem), "occupancy");
    if (st == PSF_OK && per_sm < 1) {
        set_error("multigrid apply kernel does not fit on an SM");
        st = PSF_CUDA_ERROR;
    }
    if (st == PSF_OK) {
        int blocks = c->num_sms * (per_sm < 2 ? per_sm : 2);
        const long long need = (c->nnodes + kMgThreads - 1) / kMgThreads;
        if (blocks > need) blocks = (int)need;
        if (blocks < 1) blocks = 1;
        size_t sm2 = smem;
        st = mg_tiles(c, H, a, blocks, H->max_dyn, &sm2);
        void *args[] = {a, (void *)&r, (void *)&r32, (void *)&xo, (void *)&flags};
        if (st == PSF_OK) st = launch_coop(c, (const void *)mg_apply_kernel<KIND>, blocks, kMgThreads, args, sm2);
    }
    delete a;
    return st;
}

__global__ void widen_kernel(long long n, const float *__restrict__ a, double *__restrict__ b) {
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x)
        b[t] = (double)a[t];
}

psf_status mg_apply(Ctx *c, const double *r, float *r32, float *xo, const int *flags);

// z = |r| V(r / |r|) for a nodal r (fixed dofs zero): one V-cycle of the current design's
// hierarchy, the preconditioner of PSF_SOLVE_IR_MG_F32 on its own
psf_status mg_precondition(Ctx *c, const double *r, double *z) {
    PSF_CHECK(mg_prepare(c));
    PSF_CHECK(mg_apply(c, r, c->w32[0], c->w32[1], nullptr));
    (widen_kernel<<<grid_for(c->ndofs, 256, 65536), 256, 0, c->stream>>>(c->ndofs, c->w32[1], z), note_launch());
    PSF_CUDA(cudaGetLastError());
    return PSF_OK;
}

psf_status mg_apply(Ctx *c, const double *r, float *r32, float *xo, const int *flags) {
    if (!c->mg) {
        set_error("mg_apply: hierarchy not prepared");
        return PSF_BAD_INPUT;
    }
    switch (c->kind) {
        case PSF_Q4_PLANE_STRAIN: return mg_apply_t<0>(c, r, r32, xo, flags);
        case PSF_Q4_HEAT: return mg_apply_t<1>(c, r, r32, xo, flags);
        default: return mg_apply_t<2>(c, r, r32, xo, flags);
    }
}
}  // namespace psf
