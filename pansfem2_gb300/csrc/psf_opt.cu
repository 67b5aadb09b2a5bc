// psf_opt.cu -- density filter, compliance + sensitivities, OC and MMA updates.
//
// The density filter on a structured grid is a fixed stencil: the neighbour
// list of element i (every j with |cg_i - cg_j| <= R, ascending j, weight
// (R - d)/R; sample_optimize_density_oc.cpp:50-60) is the stencil clipped to the
// grid, visited in ascending element id, so each filtered value is summed in
// the reference's order.  OC and MMA run as persistent cooperative kernels:
// the bisection / interior-point loops with data-dependent trip counts stay
// on the device, every block computing the same scalars.
#include <cmath>
#include <cstdlib>
#include <cstdio>
#include <vector>

#include "psf_internal.cuh"

namespace psf {

constexpr int kMaxStencil = 1024;

struct Stencil {
    int n;
    int is3d;
    int nx, ny, nz;
    short di[kMaxStencil], dj[kMaxStencil], dk[kMaxStencil];
    double w[kMaxStencil];
};

__device__ __forceinline__ void elem_ijk(const Stencil &S, long long e, int &i, int &j, int &k) {
    if (S.is3d) {
        k = (int)(e % S.nz);
        long long r = e / S.nz;
        j = (int)(r % S.ny);
        i = (int)(r / S.ny);
    } else {
        k = 0;
        j = (int)(e % S.ny);
        i = (int)(e / S.ny);
    }
}

// sum_o w_o v[e + o] over in-grid offsets, in stencil (ascending element) order
__device__ __forceinline__ double stencil_sum(const Stencil &S, const double *__restrict__ v, int i, int j, int k) {
    double acc = 0.0;
    for (int o = 0; o < S.n; o++) {
        const int a = i + S.di[o], b = j + S.dj[o], q = k + S.dk[o];
        if (a < 0 || a >= S.nx || b < 0 || b >= S.ny) continue;
        if (S.is3d && (q < 0 || q >= S.nz)) continue;
        const long long e = S.is3d ? ((long long)S.ny * a + b) * S.nz + q : (long long)S.ny * a + b;
        acc += S.w[o] * v[e];
    }
    return acc;
}

namespace {

__global__ void wsum_kernel(const __grid_constant__ Stencil S, long long ne, double *wsum) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < ne; e += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        elem_ijk(S, e, i, j, k);
        double ws = 0.0;
        for (int o = 0; o < S.n; o++) {
            const int a = i + S.di[o], b = j + S.dj[o], q = k + S.dk[o];
            if (a < 0 || a >= S.nx || b < 0 || b >= S.ny) continue;
            if (S.is3d && (q < 0 || q >= S.nz)) continue;
            ws += S.w[o];
        }
        wsum[e] = ws;
    }
}

// GetFilteredVariables (DensityFilter.h:44-56) and GetFilteredSensitivitis
// (DensityFilter.h:59-71): both are sum_j w_ij v_j / wsum_i (the reference
// normalises sensitivities by wsum_i as well).
__global__ void filter_kernel(const __grid_constant__ Stencil S, long long ne, const double *__restrict__ in,
                              const double *__restrict__ wsum, double *__restrict__ out) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < ne; e += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        elem_ijk(S, e, i, j, k);
        out[e] = stencil_sum(S, in, i, j, k) / wsum[e];
    }
}

// filtered density, moduli E = E1 rho^p + E0 (1 - rho^p) (sample :123) and the
// volume sum sum_i scale1*rho_i/(vf*ne) (sample :99-105) in one pass
// HeavisideFilter.h:74 and :88 (the projection of the filtered density and its derivative)
__device__ __forceinline__ double heav_rho(double rt, double beta) {
    return 0.5 * (tanh(0.5 * beta) + tanh(beta * (rt - 0.5))) / tanh(0.5 * beta);
}
__device__ __forceinline__ double heav_drho(double rt, double beta) {
    const double t = tanh(beta * (rt - 0.5));
    return 0.5 * beta * (1.0 - t * t) / tanh(0.5 * beta);
}

__global__ void filter_moduli_kernel(const __grid_constant__ Stencil S, long long ne, const double *__restrict__ s,
                                     const double *__restrict__ wsum, double E1, double E0, double p, double vscale,
                                     double *__restrict__ rho, double *__restrict__ E, double *partials, int heav,
                                     double beta, double *__restrict__ dH) {
    __shared__ double sm[32];
    double acc[1] = {0.0};
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < ne; e += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        elem_ijk(S, e, i, j, k);
        double r = stencil_sum(S, s, i, j, k) / wsum[e];
        if (heav) {
            dH[e] = heav_drho(r, beta);
            r = heav_rho(r, beta);
        }
        rho[e] = r;
        const double rp = pow(r, p);
        E[e] = E1 * rp + E0 * (1.0 - rp);
        acc[0] += vscale * r;
    }
    block_sum<1>(acc, sm);
    if (threadIdx.x == 0) partials[blockIdx.x] = acc[0];
}

__global__ void moduli_kernel(long long ne, const double *rho, double E1, double E0, double p, double *E) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < ne; e += (long long)gridDim.x * blockDim.x) {
        const double rp = pow(rho[e], p);
        E[e] = E1 * rp + E0 * (1.0 - rp);
    }
}

__global__ void fill_kernel(long long n, double v, double *x) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x)
        x[e] = v;
}

// out = mul * (sum of the block partials, fixed order) + add
__global__ void sum_partials(const double *partials, int nb, double mul, double add, double *out) {
    const int lane = threadIdx.x;
    double a = 0.0;
    for (int b = lane; b < nb; b += 32) a += partials[b];
    a = warp_sum(a);
    if (lane == 0) *out = mul * a + add;
}

struct KeP {
    double v[576];
};

// q_e = u_e . Ke0 u_e; f += E_e q_e; dfdrho_e = -scale0*p*(E1 - E0)*rho^(p-1)*q_e
// (sample_optimize_density_oc.cpp:153-162; u.K u over the elements equals u.r)
template <int KIND>
__global__ void sens_kernel(int nx, int ny, int nz, long long ne, const __grid_constant__ KeP Ke,
                            const double *__restrict__ un, const double *__restrict__ rho,
                            const double *__restrict__ E, double scale0, double p, double E1, double E0,
                            double *__restrict__ dfdrho, double *partials) {
    constexpr bool is3d = KIND == PSF_H8_SOLID;
    constexpr int ndof = KIND == PSF_Q4_PLANE_STRAIN ? 2 : (KIND == PSF_Q4_HEAT ? 1 : 3);
    constexpr int nen = is3d ? 8 : 4, nk = nen * ndof;
    __shared__ double sm[32];
    double acc[1] = {0.0};
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < ne; e += (long long)gridDim.x * blockDim.x) {
        int i, j, k = 0;
        if (is3d) {
            k = (int)(e % nz);
            long long r = e / nz;
            j = (int)(r % ny);
            i = (int)(r / ny);
        } else {
            j = (int)(e % ny);
            i = (int)(e / ny);
        }
        double ue[nk];
#pragma unroll
        for (int q = 0; q < nen; q++) {
            const int qi = (q == 1 || q == 2 || q == 5 || q == 6), qj = (q == 2 || q == 3 || q == 6 || q == 7), qk = q >= 4;
            const long long m = is3d ? ((long long)(ny + 1) * (i + qi) + (j + qj)) * (nz + 1) + (k + qk)
                                     : (long long)(ny + 1) * (i + qi) + (j + qj);
#pragma unroll
            for (int b = 0; b < ndof; b++) ue[q * ndof + b] = un[m * ndof + b];
        }
        double qv = 0.0;
#pragma unroll
        for (int a = 0; a < nk; a++) {
            double v = 0.0;
#pragma unroll
            for (int b = 0; b < nk; b++) v += Ke.v[a * nk + b] * ue[b];
            qv += ue[a] * v;
        }
        dfdrho[e] = -scale0 * p * (-E0 + E1) * pow(rho[e], p - 1.0) * qv;
        acc[0] += E[e] * qv;
    }
    block_sum<1>(acc, sm);
    if (threadIdx.x == 0) partials[blockIdx.x] = acc[0];
}

// ------------------------------------------------------------------ OC (OC.h:76-107)
struct OcArgs {
    long long n;
    double *x, *xnew, *rho;
    const double *dfdx, *dgdx, *wsum;
    const double *vw;   // volume weights sum over e in N(j) of w_ej / wsum_e (oc_fact_kernel)
    double *bp, *cs;    // x (-dfdx / dgdx)^iota per element; two sets of chunk sums (oc_fact_kernel)
    double iota, lmin, lmax, leps, move, vscale, scale1;
    int heav;
    double beta;
    GridSync *gs;
    double *partials;
    double *out;   // out[0] = lambda, out[1] = bisection steps
};

__global__ void __launch_bounds__(256) oc_kernel(const __grid_constant__ Stencil S, OcArgs A) {
    grid_sync_init();
    __shared__ double sm[32];
    const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long stride = (long long)gridDim.x * blockDim.x;
    double l0 = A.lmin, l1 = A.lmax, lambda = 0.0;
    int steps = 0;
    while ((l1 - l0) / (l1 + l0) > A.leps) {
        lambda = 0.5 * (l1 + l0);
        steps++;
        for (long long e = tid; e < A.n; e += stride) {
            const double xe = A.x[e];
            double v = pow(-A.dfdx[e] / (A.dgdx[e] * lambda), A.iota) * xe;
            const double lo0 = (1.0 - A.move) * xe, hi0 = (1.0 + A.move) * xe;
            const double lo = (0.0 < lo0) ? lo0 : 0.0;      // std::max(T(), (1 - move) x)
            const double hi = (hi0 < 1.0) ? hi0 : 1.0;      // std::min(1.0, (1 + move) x)
            if (v < lo) v = lo;
            else if (v > hi) v = hi;
            A.xnew[e] = v;
        }
        if (!grid_barrier(A.gs, A.partials)) return;
        // the samples' constraint callback: filter x_new, sum the volume
        double acc[1] = {0.0};
        for (long long e = tid; e < A.n; e += stride) {
            int i, j, k;
            elem_ijk(S, e, i, j, k);
            double r = stencil_sum(S, A.xnew, i, j, k) / A.wsum[e];
            if (A.heav) r = heav_rho(r, A.beta);
            acc[0] += A.vscale * r;
        }
        block_sum<1>(acc, sm);
        if (!grid_sync<1, 0>(A.gs, A.partials, acc, 0.0)) return;
        const double g = gs_result(A.gs, 0) - 1.0 * A.scale1;
        if (g > 0.0) l0 = lambda;
        else l1 = lambda;
        if (steps > 4000) break;   // bisection of a finite interval ends long before this
    }
    for (long long e = tid; e < A.n; e += stride) A.x[e] = A.xnew[e];
    if (tid == 0) {
        A.out[0] = lambda;
        A.out[1] = steps;
    }
}

// OC without the Heaviside projection: the same bisection with the trial design formed as
// [x (-dfdx / dgdx)^iota] lambda^-iota (the power once per update) and the filtered volume
// sum_e (sum_j w_ej x_j) / wsum_e reordered as sum_j vw_j x_j, summed in the canonical chunk
// order (psf_common.cuh).  Each warp owns whole chunks, so a step is one pass and one grid
// barrier; the chunk sums alternate between two sets, so a set is rewritten only after a
// later barrier.  The batched OC (psf_batch.cu oc_batch) uses the same arithmetic and order,
// so both take the same bisection branches on the same inputs.  Against the reference's
// expression the trial designs differ by rounding only.
__global__ void __launch_bounds__(256) oc_fact_kernel(OcArgs A) {
    grid_sync_init();
    __shared__ double s_tot;
    const long long gtid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long gw = gtid >> 5, nw = ((long long)gridDim.x * blockDim.x) >> 5;
    const int lane = threadIdx.x & 31;
    const long long n = A.n, nc = (n + kChunk - 1) / kChunk;
    for (long long c = gw; c < nc; c += nw)
        for (long long e = c * kChunk + lane; e < n && e < (c + 1) * kChunk; e += 32) {
            const double b = -A.dfdx[e] / A.dgdx[e];
            A.bp[e] = A.x[e] * (A.iota == 0.5 ? sqrt(b) : pow(b, A.iota));
        }
    double l0 = A.lmin, l1 = A.lmax, lambda = 0.0;
    int steps = 0;
    while ((l1 - l0) / (l1 + l0) > A.leps && steps < 4000) {
        lambda = 0.5 * (l1 + l0);
        double *cs = A.cs + (steps & 1) * nc;
        steps++;
        const double li = A.iota == 0.5 ? 1.0 / sqrt(lambda) : pow(lambda, -A.iota);
        for (long long c = gw; c < nc; c += nw) {
            double acc = 0.0;
            for (long long e = c * kChunk + lane; e < n && e < (c + 1) * kChunk; e += 32) {
                const double xe = A.x[e];
                double v = A.bp[e] * li;
                const double lo0 = (1.0 - A.move) * xe, hi0 = (1.0 + A.move) * xe;
                const double lo = (0.0 < lo0) ? lo0 : 0.0;      // std::max(T(), (1 - move) x)
                const double hi = (hi0 < 1.0) ? hi0 : 1.0;      // std::min(1.0, (1 + move) x)
                if (v < lo) v = lo;
                else if (v > hi) v = hi;
                A.xnew[e] = v;
                acc += A.vw[e] * v;
            }
            acc = warp_xor_sum(acc);
            if (lane == 0) cs[c] = acc;
        }
        if (!grid_barrier(A.gs, A.partials)) return;
        if (threadIdx.x < 32) {
            const double tot = warp_canonical_sum(cs, nc);
            if (threadIdx.x == 0) s_tot = tot;
        }
        __syncthreads();
        const double g = s_tot * A.vscale - 1.0 * A.scale1;
        if (g > 0.0) l0 = lambda;
        else l1 = lambda;
    }
    for (long long c = gw; c < nc; c += nw)
        for (long long e = c * kChunk + lane; e < n && e < (c + 1) * kChunk; e += 32) A.x[e] = A.xnew[e];
    if (gtid == 0) {
        A.out[0] = lambda;
        A.out[1] = steps;
    }
}

// volume weights vw_j = sum over the in-grid stencil entries q of w_q / wsum_{j + q} (the
// stencil is symmetric, so this sums w_ej / wsum_e over the elements e whose filter holds j),
// in stencil order
__global__ void volume_weights_kernel(const __grid_constant__ Stencil S, long long ne, const double *__restrict__ wsum,
                                      double *__restrict__ vw) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < ne; e += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        elem_ijk(S, e, i, j, k);
        double acc = 0.0;
        for (int o = 0; o < S.n; o++) {
            const int a = i + S.di[o], b = j + S.dj[o], q = k + S.dk[o];
            if (a < 0 || a >= S.nx || b < 0 || b >= S.ny) continue;
            if (S.is3d && (q < 0 || q >= S.nz)) continue;
            const long long m = S.is3d ? ((long long)S.ny * a + b) * S.nz + q : (long long)S.ny * a + b;
            acc += S.w[o] / wsum[m];
        }
        vw[e] = acc;
    }
}

// ------------------------------------------------------------------ MMA and CONLIN, m = 1
// MMA (MMA.h:116-419) and CONLIN (CONLIN.h:91-365) solve their convex subproblem with the
// same primal-dual interior-point loop (Newton step on the (m+1) reduced system, step bound,
// backtracking on the KKT norm, eps reduction); they differ in the separable approximation:
//   MMA     f~_j = p_j / (U_j - x_j) + q_j / (x_j - L_j)   (moving asymptotes, history)
//   CONLIN  f~_j = p_j x_j + q_j / x_j                      (plain move limits)
// The kernel is templated on the approximation; everything between is shared.
struct MmaArgs {
    long long n;
    double *xk;                       // in: current design, out: next design
    const double *dfdx, *dgdx;
    double g;                         // constraint value
    double *L, *U, *xkm1, *xkm2;      // state
    double *w;                        // 17*n work
    int k;                            // outer counter
    double a0, a, c, d, xmin, xmax;
    double raa0, albefa, move, asyinit, asydecr, asyincr;
    int max_newton;
    GridSync *gs;
    double *partials;
    double *out;                      // out[0] = Newton steps, out[1] = final eps, out[2] = capped
};

__device__ __forceinline__ double dmax(double a, double b) { return (a < b) ? b : a; }   // std::max
__device__ __forceinline__ double dmin(double a, double b) { return (b < a) ? b : a; }   // std::min
__device__ __forceinline__ double sq(double v) { return v * v; }                          // pow(v, 2.0)
__device__ __forceinline__ double ad(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double mu_(double a, double b) { return __dmul_rn(a, b); }

template <bool kConlin>
__global__ void __launch_bounds__(256) mma_kernel(MmaArgs A) {
    grid_sync_init();
    __shared__ double sm[32 * 4];
    const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long stride = (long long)gridDim.x * blockDim.x;
    const long long n = A.n;
    double *al = A.w, *be = A.w + n, *p0 = A.w + 2 * n, *q0 = A.w + 3 * n, *p1 = A.w + 4 * n, *q1 = A.w + 5 * n,
           *x = A.w + 6 * n, *gsi = A.w + 7 * n, *ita = A.w + 8 * n, *G = A.w + 9 * n, *Dx = A.w + 10 * n,
           *dtx = A.w + 11 * n, *dx = A.w + 12 * n, *dgsi = A.w + 13 * n;
    double *dita = A.w + 14 * n;
    double *iam = A.w + 15 * n, *ibm = A.w + 16 * n;   // 1 / (x - alpha), 1 / (beta - x) at the Newton point
    const double xr = A.xmax - A.xmin;
    // ---- asymptotes, move limits, p/q, b (MMA.h:118-175), start point (:178-197);
    //      CONLIN: move limits, p/q, b (CONLIN.h:92-122), start point (:125-145)
    {
        double acc[1] = {0.0};
        for (long long j = tid; j < n; j += stride) {
            const double xj = A.xk[j];
            if constexpr (kConlin) {
                const double alj = dmax(A.xmin, xj - A.move * xr);
                const double bej = dmin(A.xmax, xj + A.move * xr);
                al[j] = alj;
                be[j] = bej;
                const double df = A.dfdx[j], dg = A.dgdx[j];
                const double x2 = sq(xj);
                const double p1j = dmax(dg, 0.0), q1j = dmax(-dg, 0.0) * x2;
                p0[j] = dmax(df, 0.0); q0[j] = dmax(-df, 0.0) * x2; p1[j] = p1j; q1[j] = q1j;
                acc[0] += p1j * xj + q1j / xj;
                const double x0 = 0.5 * (alj + bej);
                x[j] = x0;
                gsi[j] = dmax(1.0, 1.0 / (x0 - alj));
                ita[j] = dmax(1.0, 1.0 / (bej - x0));
                continue;
            }
            double L, U;
            if (A.k < 2) {
                L = xj - A.asyinit * xr;
                U = xj + A.asyinit * xr;
            } else {
                const double km1 = A.xkm1[j], km2 = A.xkm2[j];
                const double tmp = (xj - km1) * (km1 - km2);
                L = A.L[j];
                U = A.U[j];
                if (tmp < 0.0) {
                    L = xj - A.asydecr * (km1 - L);
                    U = xj + A.asydecr * (U - km1);
                } else if (tmp > 0.0) {
                    L = xj - A.asyincr * (km1 - L);
                    U = xj + A.asyincr * (U - km1);
                } else {
                    L = xj - (km1 - L);
                    U = xj + (U - km1);
                }
            }
            L = dmin(dmax(xj - 10.0 * xr, L), xj - 0.01 * xr);
            U = dmin(dmax(xj + 0.01 * xr, U), xj + 10.0 * xr);
            A.L[j] = L;
            A.U[j] = U;
            const double alj = dmax(dmax(A.xmin, L + A.albefa * (xj - L)), xj - A.move * xr);
            const double bej = dmin(dmin(A.xmax, U - A.albefa * (U - xj)), xj + A.move * xr);
            al[j] = alj;
            be[j] = bej;
            const double df = A.dfdx[j], dg = A.dgdx[j];
            const double dfp = dmax(df, 0.0), dfm = dmax(-df, 0.0), dgp = dmax(dg, 0.0), dgm = dmax(-dg, 0.0);
            const double ux = U - xj, xl = xj - L;
            const double p0j = sq(ux) * (1.001 * dfp + 0.001 * dfm + A.raa0 / xr);
            const double q0j = sq(xl) * (0.001 * dfp + 1.001 * dfm + A.raa0 / xr);
            const double p1j = sq(ux) * (1.001 * dgp + 0.001 * dgm + A.raa0 / xr);
            const double q1j = sq(xl) * (0.001 * dgp + 1.001 * dgm + A.raa0 / xr);
            p0[j] = p0j; q0[j] = q0j; p1[j] = p1j; q1[j] = q1j;
            acc[0] += p1j / ux + q1j / xl;
            const double x0 = 0.5 * (alj + bej);
            x[j] = x0;
            gsi[j] = dmax(1.0, 1.0 / (x0 - alj));
            ita[j] = dmax(1.0, 1.0 / (bej - x0));
        }
        block_sum<1>(acc, sm);
        if (!grid_sync<1, 0>(A.gs, A.partials, acc, 0.0)) return;
    }
    const double b = -A.g + gs_result(A.gs, 0);
    double eps = 1.0, y = 1.0, z = 1.0, zeta = 1.0, lam = 1.0, s = 1.0;
    double mu = dmax(1.0, 0.5 * A.c);
    int l = 0, capped = 0;
    for (; eps > 1.0e-7; l++) {
        if (l >= A.max_newton) { capped = 1; break; }
        // ---- phase 1: G, Dx, deltilx and the sums of the Newton system + KKT norm at w
        double acc[4] = {0.0, 0.0, 0.0, 0.0};
        // FP64 division is expensive on this part: one reciprocal per distinct
        // denominator (5 per element instead of 12); Dx is stored as 1/Dx
        for (long long j = tid; j < n; j += stride) {
            const double xj = x[j];
            const double plj = p0[j] + lam * p1[j], qlj = q0[j] + lam * q1[j];
            if constexpr (kConlin) {   // CONLIN.h:148-195
                const double xa = xj - al[j], bx = be[j] - xj;
                const double ix = 1.0 / xj, ia = 1.0 / xa, ib = 1.0 / bx;
                const double ix2 = ix * ix;
                const double Gj = p1[j] - q1[j] * ix2;
                const double Dxj = 2.0 * qlj * ix2 * ix + gsi[j] * ia + ita[j] * ib;
                const double iDx = 1.0 / Dxj;
                const double dtxj = plj - qlj * ix2 - eps * ia + eps * ib;
                G[j] = Gj; Dx[j] = iDx; dtx[j] = dtxj;
                iam[j] = ia; ibm[j] = ib;
                acc[0] += Gj * Gj * iDx;
                acc[1] += Gj * dtxj * iDx;
                acc[2] += p1[j] * xj + q1[j] * ix;
                acc[3] += sq(plj - qlj * ix2 - gsi[j] + ita[j]) + sq(gsi[j] * xa - eps) + sq(ita[j] * bx - eps);
                continue;
            }
            const double Lj = A.L[j], Uj = A.U[j];
            const double ux = Uj - xj, xl = xj - Lj, xa = xj - al[j], bx = be[j] - xj;
            const double iux = 1.0 / ux, ixl = 1.0 / xl, ia = 1.0 / xa, ib = 1.0 / bx;
            const double iux2 = iux * iux, ixl2 = ixl * ixl;
            const double Gj = p1[j] * iux2 - q1[j] * ixl2;
            const double Dxj = 2.0 * plj * iux2 * iux + 2.0 * qlj * ixl2 * ixl + gsi[j] * ia + ita[j] * ib;
            const double iDx = 1.0 / Dxj;
            const double dtxj = plj * iux2 - qlj * ixl2 - eps * ia + eps * ib;
            G[j] = Gj; Dx[j] = iDx; dtx[j] = dtxj;
            iam[j] = ia; ibm[j] = ib;
            acc[0] += Gj * Gj * iDx;
            acc[1] += Gj * dtxj * iDx;
            acc[2] += p1[j] * iux + q1[j] * ixl;
            acc[3] += sq(plj * iux2 - qlj * ixl2 - gsi[j] + ita[j]) + sq(gsi[j] * xa - eps) + sq(ita[j] * bx - eps);
        }
        block_sum<4>(acc, sm);
        if (!grid_sync<4, 0>(A.gs, A.partials, acc, 0.0)) return;
        const double SGG = gs_result(A.gs, 0), SGd = gs_result(A.gs, 1), Sg = gs_result(A.gs, 2),
                     Skkt = gs_result(A.gs, 3);
        // ---- scalars of the (m+1) system (MMA.h:226-285) and its solution (solvels, 2x2)
        const double Dy = A.d + mu / y, Dl = s / lam, dty = A.c + A.d * y - lam - eps / y;
        const double dtz = A.a0 - eps / z - (0.0 + lam * A.a);
        const double dtl = -A.a * z - y - b + eps / lam + Sg;
        const double Dly = Dl + 1.0 / Dy, dtly = dtl + dty / Dy;
        double M00 = SGG + Dly, M01 = A.a, M10 = A.a, M11 = -zeta / z;
        double B0 = dtly - SGd, B1 = dtz;
        // partial pivoting on column 0 (MMA.h:469-489), then elimination and back substitution
        if (fabs(M00) < fabs(M10)) {
            double t;
            t = B0; B0 = B1; B1 = t;
            t = M00; M00 = M10; M10 = t;
            t = M01; M01 = M11; M11 = t;
        }
        M11 -= M01 * M10 / M00;
        B1 -= B0 * M10 / M00;
        const double dz = B1 / M11;
        const double dl = (B0 - dz * M01) / M00;
        const double dy = dl / Dy - dty / Dy;
        const double dmu = -mu * dy / y - mu + eps / y;
        const double ds = -s * dl / lam - s + eps / lam;
        const double dzeta = -zeta * dz / z - zeta + eps / z;
        double tymax = 0.0;
        {
            double t = dmax(dmax(dmax(-1.01 * dy / y, -1.01 * dl / lam), -1.01 * dmu / mu), -1.01 * ds / s);
            if (tymax < t) tymax = t;
        }
        const double dw = sqrt(Skkt + sq(A.c + A.d * y - lam - mu) + sq(Sg - A.a * z - y + s - b) + sq(mu * y - eps) +
                               sq(lam * s - eps) + sq(A.a0 - zeta - (0.0 + lam * A.a)) + sq(zeta * z - eps));
        // ---- phase 2: Newton direction in x, step-length bound
        double tx = -INFINITY;
        for (long long j = tid; j < n; j += stride) {
            const double ia = iam[j], ib = ibm[j];   // x is unchanged since phase 1
            const double dxj = -(dtx[j] + G[j] * dl) * Dx[j];   // Dx holds 1/Dx
            const double dg = -gsi[j] * dxj * ia - gsi[j] + eps * ia;
            const double di = ita[j] * dxj * ib - ita[j] + eps * ib;
            dx[j] = dxj; dgsi[j] = dg; dita[j] = di;
            const double t = dmax(dmax(dmax(-1.01 * dxj * ia, 1.01 * dxj * ib), -1.01 * dg / gsi[j]), -1.01 * di / ita[j]);
            tx = fmax(tx, t);
        }
        tx = block_max(tx, sm);
        {
            double none[1] = {0.0};
            if (!grid_sync<0, 1>(A.gs, A.partials, none, tx)) return;
        }
        double txmax = 0.0;
        {
            const double t = gs_result_max(A.gs);
            if (txmax < t) txmax = t;
        }
        double tau = 1.0 / dmax(dmax(dmax(dmax(1.0, txmax), tymax), -1.01 * dz / z), -1.01 * dzeta / zeta);
        // ---- phase 3: backtracking on the KKT norm (MMA.h:371-391)
        double tau_used = tau, dw1 = 0.0, yp = y, lp = lam, mp = mu, sp = s, zp = z, zetap = zeta;
        for (int ll = 0; ll < 50; ll++) {
            tau_used = tau;
            yp = ad(y, mu_(tau, dy)); lp = ad(lam, mu_(tau, dl)); mp = ad(mu, mu_(tau, dmu));
            sp = ad(s, mu_(tau, ds)); zp = ad(z, mu_(tau, dz)); zetap = ad(zeta, mu_(tau, dzeta));
            double a2[2] = {0.0, 0.0};
            for (long long j = tid; j < n; j += stride) {
                const double xp = ad(x[j], mu_(tau, dx[j])), gp = ad(gsi[j], mu_(tau, dgsi[j])),
                             ip = ad(ita[j], mu_(tau, dita[j]));
                const double plj = p0[j] + lp * p1[j], qlj = q0[j] + lp * q1[j];
                if constexpr (kConlin) {   // CONLIN::KKTNorm (CONLIN.h:369-407) at the trial point
                    const double ixp = 1.0 / xp;
                    a2[0] += p1[j] * xp + q1[j] * ixp;
                    a2[1] += sq(plj - qlj * (ixp * ixp) - gp + ip) + sq(gp * (xp - al[j]) - eps) +
                             sq(ip * (be[j] - xp) - eps);
                    continue;
                }
                const double iux = 1.0 / (A.U[j] - xp), ixl = 1.0 / (xp - A.L[j]);
                a2[0] += p1[j] * iux + q1[j] * ixl;
                a2[1] += sq(plj * (iux * iux) - qlj * (ixl * ixl) - gp + ip) + sq(gp * (xp - al[j]) - eps) +
                         sq(ip * (be[j] - xp) - eps);
            }
            block_sum<2>(a2, sm);
            if (!grid_sync<2, 0>(A.gs, A.partials, a2, 0.0)) return;
            const double Sgt = gs_result(A.gs, 0), Skt = gs_result(A.gs, 1);
            dw1 = sqrt(Skt + sq(A.c + A.d * yp - lp - mp) + sq(Sgt - A.a * zp - yp + sp - b) + sq(mp * yp - eps) +
                       sq(lp * sp - eps) + sq(A.a0 - zetap - (0.0 + lp * A.a)) + sq(zetap * zp - eps));
            if (dw1 < dw) break;
            tau *= 0.5;
        }
        // ---- accept the last trial point (MMA.h:394-402); its KKT norm is dw1
        for (long long j = tid; j < n; j += stride) {
            x[j] = ad(x[j], mu_(tau_used, dx[j]));
            gsi[j] = ad(gsi[j], mu_(tau_used, dgsi[j]));
            ita[j] = ad(ita[j], mu_(tau_used, dita[j]));
        }
        y = yp; lam = lp; mu = mp; s = sp; z = zp; zeta = zetap;
        if (dw1 < 0.9 * eps) eps *= 0.1;
    }
    // ---- history and the new design (MMA.h:413-418; CONLIN keeps no history, CONLIN.h:361-364)
    for (long long j = tid; j < n; j += stride) {
        if constexpr (!kConlin) {
            A.xkm2[j] = A.xkm1[j];
            A.xkm1[j] = A.xk[j];
        }
        A.xk[j] = x[j];
    }
    if (tid == 0) {
        A.out[0] = l;
        A.out[1] = eps;
        A.out[2] = capped;
    }
}

}  // namespace

// ------------------------------------------------------------------ host side
static psf_status make_stencil(Ctx *c, Stencil *S) {
    S->is3d = c->kind == PSF_H8_SOLID;
    S->nx = c->nx; S->ny = c->ny; S->nz = c->nz;
    const double hx = c->lx / c->nx, hy = c->ly / c->ny, hz = S->is3d ? c->lz / c->nz : 1.0;
    const double R = c->R;
    const int rx = (int)floor(R / hx) + 1, ry = (int)floor(R / hy) + 1, rz = S->is3d ? (int)floor(R / hz) + 1 : 0;
    int n = 0;
    for (int a = -rx; a <= rx; a++)
        for (int b = -ry; b <= ry; b++)
            for (int q = -rz; q <= rz; q++) {
                // |cg_i - cg_j| of the reference: sqrt of the sum of pow(diff, 2.0)
                double d2 = 0.0;
                d2 += (a * hx) * (a * hx);
                d2 += (b * hy) * (b * hy);
                if (S->is3d) d2 += (q * hz) * (q * hz);
                const double d = sqrt(d2);
                if (d <= R) {
                    if (n >= kMaxStencil) { set_error("filter radius too large for the stencil table"); return PSF_BAD_INPUT; }
                    S->di[n] = (short)a; S->dj[n] = (short)b; S->dk[n] = (short)q;
                    S->w[n] = (R - d) / R;
                    n++;
                }
            }
    S->n = n;
    return PSF_OK;
}

static psf_status get_stencil(Ctx *c, Stencil *S) {
    if (c->filt_n <= 0) { set_error("filter not set up (psf_filter_setup / psf_simp_begin)"); return PSF_BAD_INPUT; }
    return make_stencil(c, S);
}

psf_status filter_setup(Ctx *c, double R) {
    if (!(R > 0)) { set_error("filter radius must be positive"); return PSF_BAD_INPUT; }
    c->R = R;
    Stencil *S = new Stencil;
    psf_status st = make_stencil(c, S);
    if (st != PSF_OK) { delete S; return st; }
    c->filt_n = S->n;
    (wsum_kernel<<<grid_for(c->ne, 256, 65536), 256, 0, c->stream>>>(*S, c->ne, c->filt_wsum), ::psf::note_launch());
    (volume_weights_kernel<<<grid_for(c->ne, 256, 65536), 256, 0, c->stream>>>(*S, c->ne, c->filt_wsum, c->filt_vw),
     ::psf::note_launch());
    delete S;
    PSF_CUDA(cudaGetLastError());
    return PSF_OK;
}

// SensitivityFilter (Sigmund, SensitivityFilter.h:38-50): sum_j w_ij s_j d_j / (wsum_i s_i);
// SensitivityFilter2 (Borrvall, :78-90): sum_j w_ij s_j d_j / sum_j w_ij s_j
__global__ void sens_filter_kernel(const __grid_constant__ Stencil S, long long ne, const double *__restrict__ s,
                                   const double *__restrict__ d, const double *__restrict__ wsum, int mode,
                                   double *__restrict__ out) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < ne; e += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        elem_ijk(S, e, i, j, k);
        double v = 0.0, ws = 0.0;
        for (int q = 0; q < S.n; q++) {
            const int a = i + S.di[q], b = j + S.dj[q], c = k + S.dk[q];
            if (a < 0 || a >= S.nx || b < 0 || b >= S.ny || (S.is3d && (c < 0 || c >= S.nz))) continue;
            const long long m = S.is3d ? ((long long)S.ny * a + b) * S.nz + c : (long long)S.ny * a + b;
            v += S.w[q] * s[m] * d[m];
            ws += S.w[q] * s[m];
        }
        out[e] = mode ? v / ws : v / (wsum[e] * s[e]);
    }
}

psf_status sensitivity_filter(Ctx *c, const double *s, const double *d, int mode, double *out) {
    Stencil *S = new Stencil;
    psf_status st = get_stencil(c, S);
    if (st == PSF_OK) {
        (sens_filter_kernel<<<grid_for(c->ne, 256, 65536), 256, 0, c->stream>>>(*S, c->ne, s, d, c->filt_wsum, mode,
                                                                                out), ::psf::note_launch());
        if (cudaGetLastError() != cudaSuccess) st = PSF_CUDA_ERROR;
    }
    delete S;
    return st;
}

__global__ void mul_kernel(long long n, const double *__restrict__ a, const double *__restrict__ b,
                           double *__restrict__ out) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x)
        out[e] = a[e] * b[e];
}

// projection of filtered densities in place: rt -> H(rt), dH = H'(rt) (HeavisideFilter.h:70, :84)
__global__ void heaviside_project_kernel(long long n, double beta, double *__restrict__ r, double *__restrict__ dH) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const double rt = r[e];
        dH[e] = heav_drho(rt, beta);
        r[e] = heav_rho(rt, beta);
    }
}

// HeavisideFilter::GetFilteredVariables (HeavisideFilter.h:61-74) on device arrays:
// rho = H(filter(s)); dH = H'(filter(s)) is kept for heaviside_back
psf_status heaviside_forward(Ctx *c, double beta, const double *s, double *rho) {
    PSF_CHECK(filter_apply(c, s, rho, false));
    (heaviside_project_kernel<<<grid_for(c->ne, 256, 65536), 256, 0, c->stream>>>(
         c->ne, beta, rho, c->dH),
     ::psf::note_launch());
    PSF_CUDA(cudaGetLastError());
    return PSF_OK;
}

// filtered sensitivity through the projection (HeavisideFilter.h:81-97):
// out_i = sum_j w_ij d_j dH_j / wsum_i
psf_status heaviside_back(Ctx *c, const double *d, double *out) {
    (mul_kernel<<<grid_for(c->ne, 256, 65536), 256, 0, c->stream>>>(c->ne, d, c->dH, c->tmp_ne), ::psf::note_launch());
    PSF_CUDA(cudaGetLastError());
    return filter_apply(c, c->tmp_ne, out, true);
}

psf_status filter_apply(Ctx *c, const double *in, double *out, bool backward) {
    (void)backward;   // both directions are the same stencil sum normalised by wsum_i
    Stencil *S = new Stencil;
    psf_status st = get_stencil(c, S);
    if (st == PSF_OK) {
        (filter_kernel<<<grid_for(c->ne, 256, 65536), 256, 0, c->stream>>>(
             *S, c->ne, in, c->filt_wsum, out),
         ::psf::note_launch());
        if (cudaGetLastError() != cudaSuccess) st = PSF_CUDA_ERROR;
    }
    delete S;
    return st;
}

// rho = filter(s), E = moduli(rho), scal[1] = g (volume constraint)
psf_status filter_moduli(Ctx *c, const double *s, double *rho, double *E, double E1, double E0, double p,
                         double vf, double scale1, double *g_dev) {
    Stencil *S = new Stencil;
    psf_status st = get_stencil(c, S);
    if (st != PSF_OK) { delete S; return st; }
    const int nb = grid_for(c->ne, 256, c->num_sms * 8);
    const double vscale = scale1 / (vf * (double)c->ne);
    (filter_moduli_kernel<<<nb, 256, 0, c->stream>>>(*S, c->ne, s, c->filt_wsum, E1, E0, p, vscale, rho, E, c->partials,
                                                    c->heav, c->beta, c->dH), ::psf::note_launch());
    delete S;
    (sum_partials<<<1, 32, 0, c->stream>>>(c->partials, nb, 1.0, -1.0 * scale1, g_dev), ::psf::note_launch());
    PSF_CUDA(cudaGetLastError());
    return PSF_OK;
}

psf_status moduli_from_rho(Ctx *c, const double *rho, double E1, double E0, double p, double *E_dev) {
    (moduli_kernel<<<grid_for(c->ne, 256, 65536), 256, 0, c->stream>>>(
         c->ne, rho, E1, E0, p, E_dev),
     ::psf::note_launch());
    PSF_CUDA(cudaGetLastError());
    return PSF_OK;
}

psf_status fill(Ctx *c, double *x, long long n, double v) {
    (fill_kernel<<<grid_for(n, 256, 65536), 256, 0, c->stream>>>(n, v, x), ::psf::note_launch());
    PSF_CUDA(cudaGetLastError());
    return PSF_OK;
}

psf_status compliance_sens(Ctx *c, const double *rho, double E1, double E0, double p, double scale0,
                           double *f_dev, double *dfdrho) {
    KeP *K = new KeP;
    const int nk = c->nen * c->ndof;
    for (int q = 0; q < nk * nk; q++) K->v[q] = c->Ke0_host[q];
    const int nb = grid_for(c->ne, 256, c->num_sms * 8);
    switch (c->kind) {
    case PSF_Q4_PLANE_STRAIN:
        (sens_kernel<0><<<nb, 256, 0, c->stream>>>(
             c->nx, c->ny, c->nz, c->ne, *K, c->un, rho, c->E, scale0, p, E1, E0, dfdrho, c->partials),
         ::psf::note_launch());
        break;
    case PSF_Q4_HEAT:
        (sens_kernel<1><<<nb, 256, 0, c->stream>>>(
             c->nx, c->ny, c->nz, c->ne, *K, c->un, rho, c->E, scale0, p, E1, E0, dfdrho, c->partials),
         ::psf::note_launch());
        break;
    default:
        (sens_kernel<2><<<nb, 256, 0, c->stream>>>(
             c->nx, c->ny, c->nz, c->ne, *K, c->un, rho, c->E, scale0, p, E1, E0, dfdrho, c->partials),
         ::psf::note_launch());
        break;
    }
    delete K;
    PSF_CUDA(cudaGetLastError());
    // f = scale0 * sum_e E_e q_e
    (sum_partials<<<1, 32, 0, c->stream>>>(c->partials, nb, scale0, 0.0, f_dev), ::psf::note_launch());
    PSF_CUDA(cudaGetLastError());
    return PSF_OK;
}

// the MMA / CONLIN element-wise arithmetic in double words (psf_optdw.cu) unless
// PSF_OPT_F64=1 asks for the FP64 kernel (read at every update)
static bool opt_use_dw() {
    const char *e = getenv("PSF_OPT_F64");
    return !(e && e[0] == '1');
}

static int coop_blocks_for(Ctx *c, const void *fn, int threads, long long work) {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, 0) != cudaSuccess || per_sm < 1) return 0;
    const int bps = c->opt_blocks_per_sm;   // psf_set_launch_shape(PSF_KERNEL_OPT)
    int blocks = c->num_sms * (per_sm < bps ? per_sm : bps);
    long long need = (work + threads - 1) / threads;
    if (blocks > need) blocks = (int)need;
    return blocks < 1 ? 1 : blocks;
}

psf_status oc_update(Ctx *c, double *x, const double *dfdx, const double *dgdx, double iota, double lmin,
                     double lmax, double leps, double move, double vf, double scale1, double *lambda) {
    Stencil *S = new Stencil;
    psf_status st = get_stencil(c, S);
    if (st != PSF_OK) { delete S; return st; }
    OcArgs A;
    A.n = c->ne;
    A.x = x;
    A.xnew = c->snew;
    A.rho = nullptr;
    A.dfdx = dfdx;
    A.dgdx = dgdx;
    A.wsum = c->filt_wsum;
    A.iota = iota; A.lmin = lmin; A.lmax = lmax; A.leps = leps; A.move = move;
    A.vscale = scale1 / (vf * (double)c->ne);
    A.scale1 = scale1;
    A.heav = c->heav;
    A.beta = c->beta;
    A.gs = c->gs;
    A.partials = c->partials;
    A.out = c->scal + 4;
    A.vw = c->filt_vw;
    A.bp = c->oc_bp;
    A.cs = c->oc_cs;
    if (c->heav) {
        const int blocks = coop_blocks_for(c, (const void *)oc_kernel, 256, c->ne);
        if (!blocks) { delete S; set_error("OC kernel does not fit"); return PSF_CUDA_ERROR; }
        void *args[] = {S, &A};
        st = launch_coop(c, (const void *)oc_kernel, blocks, 256, args);
    } else {
        const int blocks = coop_blocks_for(c, (const void *)oc_fact_kernel, 256, c->ne);
        if (!blocks) { delete S; set_error("OC kernel does not fit"); return PSF_CUDA_ERROR; }
        void *args[] = {&A};
        st = launch_coop(c, (const void *)oc_fact_kernel, blocks, 256, args);
    }
    delete S;
    PSF_CHECK(st);
    PSF_CHECK(read_sync_status(c));
    if (lambda) {
        PSF_CUDA(cudaMemcpyAsync(lambda, c->scal + 4, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
        PSF_CUDA(cudaStreamSynchronize(c->stream));
    }
    return PSF_OK;
}

psf_status mma_update(Ctx *c, double *x, double f, const double *dfdx, double g, const double *dgdx, int *newton) {
    if (!c->mma_ready) { set_error("psf_mma_update: call psf_mma_init first"); return PSF_BAD_INPUT; }
    if (opt_use_dw()) {
        bool done = false, capped = false;
        PSF_CHECK(mma_dw_update(c, false, x, dfdx, g, dgdx, newton, &capped, &done));
        if (done) {
            c->mma_prev = f;
            c->mma_k++;
            if (capped) { set_error("MMA interior-point loop hit its step cap"); return PSF_NOT_CONVERGED; }
            return PSF_OK;
        }
        c->opt_fp64_fallbacks++;
    }
    MmaArgs A;
    A.n = c->ne;
    A.xk = x;
    A.dfdx = dfdx;
    A.dgdx = dgdx;
    A.g = g;
    A.L = c->mma_L; A.U = c->mma_U; A.xkm1 = c->mma_xkm1; A.xkm2 = c->mma_xkm2;
    A.w = c->mma_work;
    A.k = c->mma_k;
    A.a0 = c->mma_a0; A.a = c->mma_a; A.c = c->mma_c; A.d = c->mma_d; A.xmin = c->mma_xmin; A.xmax = c->mma_xmax;
    A.raa0 = c->mma_raa0; A.albefa = c->mma_albefa; A.move = c->mma_move; A.asyinit = c->mma_asyinit;
    A.asydecr = c->mma_asydecr; A.asyincr = c->mma_asyincr;
    A.max_newton = 2000;
    A.gs = c->gs;
    A.partials = c->partials;
    A.out = c->scal + 4;
    const int blocks = coop_blocks_for(c, (const void *)mma_kernel<false>, 256, c->ne);
    if (!blocks) { set_error("MMA kernel does not fit"); return PSF_CUDA_ERROR; }
    void *args[] = {&A};
    PSF_CHECK(launch_coop(c, (const void *)mma_kernel<false>, blocks, 256, args));
    PSF_CHECK(read_sync_status(c));
    double h[3];
    PSF_CUDA(cudaMemcpyAsync(h, c->scal + 4, sizeof h, cudaMemcpyDeviceToHost, c->stream));
    PSF_CUDA(cudaStreamSynchronize(c->stream));
    if (newton) *newton = (int)h[0];
    c->mma_prev = f;
    c->mma_k++;
    if (h[2] != 0.0) { set_error("MMA interior-point loop hit its step cap"); return PSF_NOT_CONVERGED; }
    return PSF_OK;
}

psf_status conlin_update(Ctx *c, double *x, double f, const double *dfdx, double g, const double *dgdx, int *newton) {
    if (!c->cl_ready) { set_error("psf_conlin_update: call psf_conlin_init first"); return PSF_BAD_INPUT; }
    if (opt_use_dw()) {
        bool done = false, capped = false;
        PSF_CHECK(mma_dw_update(c, true, x, dfdx, g, dgdx, newton, &capped, &done));
        if (done) {
            c->cl_prev = f;
            c->cl_k++;
            if (capped) { set_error("CONLIN interior-point loop hit its step cap"); return PSF_NOT_CONVERGED; }
            return PSF_OK;
        }
        c->opt_fp64_fallbacks++;
    }
    MmaArgs A{};
    A.n = c->ne;
    A.xk = x;
    A.dfdx = dfdx;
    A.dgdx = dgdx;
    A.g = g;
    A.w = c->mma_work;
    A.k = c->cl_k;
    A.a0 = c->cl_a0; A.a = c->cl_a; A.c = c->cl_c; A.d = c->cl_d; A.xmin = c->cl_xmin; A.xmax = c->cl_xmax;
    A.move = c->cl_move;
    A.max_newton = 2000;
    A.gs = c->gs;
    A.partials = c->partials;
    A.out = c->scal + 4;
    const int blocks = coop_blocks_for(c, (const void *)mma_kernel<true>, 256, c->ne);
    if (!blocks) { set_error("CONLIN kernel does not fit"); return PSF_CUDA_ERROR; }
    void *args[] = {&A};
    PSF_CHECK(launch_coop(c, (const void *)mma_kernel<true>, blocks, 256, args));
    PSF_CHECK(read_sync_status(c));
    double h[3];
    PSF_CUDA(cudaMemcpyAsync(h, c->scal + 4, sizeof h, cudaMemcpyDeviceToHost, c->stream));
    PSF_CUDA(cudaStreamSynchronize(c->stream));
    if (newton) *newton = (int)h[0];
    c->cl_prev = f;
    c->cl_k++;
    if (h[2] != 0.0) { set_error("CONLIN interior-point loop hit its step cap"); return PSF_NOT_CONVERGED; }
    return PSF_OK;
}

}  // namespace psf
