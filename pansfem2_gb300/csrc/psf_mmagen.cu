// psf_mmagen.cu -- MMA<T> (MMA.h:18-509) on the device for any number of design
// variables n and 1 <= m <= 4 constraints, with per-variable bounds xmin / xmax.
//
// The object mirrors the reference class: MMA(n, m, a0, a, c, d, xmin, xmax)
// (MMA.h:64-90), SetParameters (:92-100), UpdateVariables (:116-419).  Svanberg's
// subproblem is solved by the same primal-dual interior-point iteration (the
// relaxed KKT system of his "5.9" equations), with the Newton step reduced to the
// (m+1) x (m+1) system in (lambda, z) when n > m (:260-291) or to the (n+1) x
// (n+1) system in (x, z) when n <= m (:292-330), both solved by Gaussian
// elimination with partial pivoting (solvels, :464-509), a fraction-to-boundary
// step bound and up to 50 halvings on the KKT norm (:343-391).
//
// n > m: one persistent cooperative kernel per update.  The per-variable terms
// run in parallel over the design variables, the sums the Newton system needs
// (the symmetric G D^-1 G^T block, G D^-1 deltilx, the constraint values and the
// KKT norm: m(m+1)/2 + 2m + 1 values) are folded by one grid barrier per phase,
// and every block solves the small system itself (same arithmetic, same answer).
// n <= m (at most 4 variables): one thread does the whole update.
// The per-element divisions of the reference are taken as reciprocals, so the
// result agrees with the reference to rounding (the tests hold it to 1e-7).
#include <cmath>
#include <vector>

#include "psf_internal.cuh"

namespace psf {
namespace mmagen {

constexpr int kMaxM = 4;
constexpr int kThreads = 256;

struct Params {
    int n, m, k;
    double a0, a[kMaxM], c[kMaxM], d[kMaxM];
    double raa0, albefa, move, asyinit, asydecr, asyincr;
    double g[kMaxM];                  // constraint values of this update
    const double *xmin, *xmax;        // per variable
    double *xk;                       // in: current design, out: next design
    const double *dfdx, *dgdx;        // dgdx: m x n, row-major
    double *L, *U, *xkm1, *xkm2;      // state
    double *w;                        // work, (14 + 3 kMaxM) n doubles
    int max_newton;
    GridSync *gs;
    double *partials;
    double *out;                      // out[0] Newton steps, out[1] final eps, out[2] capped
};

__device__ __forceinline__ double dmax(double a, double b) { return (a < b) ? b : a; }   // std::max
__device__ __forceinline__ double dmin(double a, double b) { return (b < a) ? b : a; }   // std::min
__device__ __forceinline__ double sq(double v) { return v * v; }

// solvels (MMA.h:464-509): Gaussian elimination with partial pivoting on column i, rows i..N-1
template <int N>
__device__ void solve_small(double (&A)[N][N], double (&b)[N], double (&x)[N], int n) {
    for (int i = 0; i < n - 1; i++) {
        double piv = fabs(A[i][i]);
        int pi = i;
        for (int j = i + 1; j < n; j++)
            if (piv < fabs(A[j][i])) { piv = fabs(A[j][i]); pi = j; }
        if (pi != i) {
            double t = b[i]; b[i] = b[pi]; b[pi] = t;
            for (int j = i; j < n; j++) { t = A[i][j]; A[i][j] = A[pi][j]; A[pi][j] = t; }
        }
        for (int j = i + 1; j < n; j++) {
            const double f = A[j][i] / A[i][i];
            for (int k = i + 1; k < n; k++) A[j][k] -= A[i][k] * f;
            b[j] -= b[i] * f;
        }
    }
    for (int i = n - 1; i >= 0; i--) {
        double v = b[i];
        for (int j = n - 1; j > i; j--) v -= x[j] * A[i][j];
        x[i] = v / A[i][i];
    }
}

// asymptotes (MMA.h:118-141), move limits (:143-149), p0 / q0 (:151-158), p / q and the
// constraint part of b (:160-172) of variable j; returns the start point's gsi, ita via x, ...
__device__ __forceinline__ void setup_var(const Params &P, long long j, double &L, double &U, double &al, double &be) {
    const double xj = P.xk[j], xr = P.xmax[j] - P.xmin[j];
    if (P.k < 2) {
        L = xj - P.asyinit * xr;
        U = xj + P.asyinit * xr;
    } else {
        const double km1 = P.xkm1[j], km2 = P.xkm2[j];
        const double tmp = (xj - km1) * (km1 - km2);
        L = P.L[j];
        U = P.U[j];
        if (tmp < 0.0) {
            L = xj - P.asydecr * (km1 - L);
            U = xj + P.asydecr * (U - km1);
        } else if (tmp > 0.0) {
            L = xj - P.asyincr * (km1 - L);
            U = xj + P.asyincr * (U - km1);
        } else {
            L = xj - (km1 - L);
            U = xj + (U - km1);
        }
    }
    L = dmin(dmax(xj - 10.0 * xr, L), xj - 0.01 * xr);
    U = dmin(dmax(xj + 0.01 * xr, U), xj + 10.0 * xr);
    al = dmax(dmax(P.xmin[j], L + P.albefa * (xj - L)), xj - P.move * xr);
    be = dmin(dmin(P.xmax[j], U - P.albefa * (U - xj)), xj + P.move * xr);
}
__device__ __forceinline__ void pq_of(double deriv, double ux, double xl, double raa, double &p, double &q) {
    const double dp = dmax(deriv, 0.0), dm = dmax(-deriv, 0.0);
    p = sq(ux) * (1.001 * dp + 0.001 * dm + raa);
    q = sq(xl) * (0.001 * dp + 1.001 * dm + raa);
}

// the n > m update, one persistent launch
template <int M>
__global__ void __launch_bounds__(kThreads) mma_gen_kernel(Params P) {
    grid_sync_init();
    __shared__ double sm[32 * (M * (M + 1) / 2 + 2 * M + 1)];
    constexpr int NSYM = M * (M + 1) / 2;
    constexpr int NS = NSYM + 2 * M + 1;   // Newton sums: sym(G G^T / Dx), G deltilx / Dx, g, KKT_x
    const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long stride = (long long)gridDim.x * blockDim.x;
    const long long n = P.n;
    double *al = P.w, *be = P.w + n, *p0 = P.w + 2 * n, *q0 = P.w + 3 * n, *x = P.w + 4 * n, *gsi = P.w + 5 * n,
           *ita = P.w + 6 * n, *iDx = P.w + 7 * n, *dtx = P.w + 8 * n, *dx = P.w + 9 * n, *dgsi = P.w + 10 * n,
           *dita = P.w + 11 * n, *iam = P.w + 12 * n, *ibm = P.w + 13 * n;
    double *pp = P.w + 14 * n, *qq = pp + (long long)kMaxM * n, *G = qq + (long long)kMaxM * n;   // [i][j]
    // ---- set-up, start point (MMA.h:178-197), b
    {
        double acc[M];
#pragma unroll
        for (int i = 0; i < M; i++) acc[i] = 0.0;
        for (long long j = tid; j < n; j += stride) {
            double L, U, a, b;
            setup_var(P, j, L, U, a, b);
            P.L[j] = L;
            P.U[j] = U;
            al[j] = a;
            be[j] = b;
            const double xj = P.xk[j], raa = P.raa0 / (P.xmax[j] - P.xmin[j]);
            const double ux = U - xj, xl = xj - L;
            pq_of(P.dfdx[j], ux, xl, raa, p0[j], q0[j]);
#pragma unroll
            for (int i = 0; i < M; i++) {
                double pij, qij;
                pq_of(P.dgdx[(long long)i * n + j], ux, xl, raa, pij, qij);
                pp[(long long)i * n + j] = pij;
                qq[(long long)i * n + j] = qij;
                acc[i] += pij / ux + qij / xl;
            }
            const double x0 = 0.5 * (a + b);
            x[j] = x0;
            gsi[j] = dmax(1.0, 1.0 / (x0 - a));
            ita[j] = dmax(1.0, 1.0 / (b - x0));
        }
        block_sum<M>(acc, sm);
        if (!grid_sync<M, 0>(P.gs, P.partials, acc, 0.0)) return;
    }
    double bb[M], y[M], lam[M], s[M], mu[M];
#pragma unroll
    for (int i = 0; i < M; i++) {
        bb[i] = -P.g[i] + gs_result(P.gs, i);
        y[i] = 1.0;
        lam[i] = 1.0;
        s[i] = 1.0;
        mu[i] = dmax(1.0, 0.5 * P.c[i]);
    }
    double eps = 1.0, z = 1.0, zeta = 1.0;
    int l = 0, capped = 0;
    for (; eps > 1.0e-7; l++) {
        if (l >= P.max_newton) { capped = 1; break; }
        // ---- phase 1: G, Dx, deltilx at w; the sums of the Newton system and the KKT norm
        double acc[NS];
#pragma unroll
        for (int q = 0; q < NS; q++) acc[q] = 0.0;
        for (long long j = tid; j < n; j += stride) {
            const double xj = x[j];
            double plj = p0[j], qlj = q0[j];
#pragma unroll
            for (int i = 0; i < M; i++) {
                plj += lam[i] * pp[(long long)i * n + j];
                qlj += lam[i] * qq[(long long)i * n + j];
            }
            const double ux = P.U[j] - xj, xl = xj - P.L[j], xa = xj - al[j], bx = be[j] - xj;
            const double iux = 1.0 / ux, ixl = 1.0 / xl, ia = 1.0 / xa, ib = 1.0 / bx;
            const double iux2 = iux * iux, ixl2 = ixl * ixl;
            double Gj[M];
#pragma unroll
            for (int i = 0; i < M; i++) {
                Gj[i] = pp[(long long)i * n + j] * iux2 - qq[(long long)i * n + j] * ixl2;
                G[(long long)i * n + j] = Gj[i];
                acc[NSYM + M + i] += pp[(long long)i * n + j] * iux + qq[(long long)i * n + j] * ixl;
            }
            const double Dxj = 2.0 * plj * iux2 * iux + 2.0 * qlj * ixl2 * ixl + gsi[j] * ia + ita[j] * ib;
            const double id = 1.0 / Dxj;
            const double dtxj = plj * iux2 - qlj * ixl2 - eps * ia + eps * ib;
            iDx[j] = id;
            dtx[j] = dtxj;
            iam[j] = ia;
            ibm[j] = ib;
            int q = 0;
#pragma unroll
            for (int i = 0; i < M; i++)
#pragma unroll
                for (int k = i; k < M; k++) acc[q++] += Gj[i] * Gj[k] * id;
#pragma unroll
            for (int i = 0; i < M; i++) acc[NSYM + i] += Gj[i] * dtxj * id;
            acc[NS - 1] += sq(plj * iux2 - qlj * ixl2 - gsi[j] + ita[j]) + sq(gsi[j] * xa - eps) + sq(ita[j] * bx - eps);
        }
        block_sum<NS>(acc, sm);
        if (!grid_sync<NS, 0>(P.gs, P.partials, acc, 0.0)) return;
        double S[NS];
#pragma unroll
        for (int q = 0; q < NS; q++) S[q] = gs_result(P.gs, q);
        // ---- scalars (MMA.h:226-257) and the (m+1) system (:260-291), solved in every block
        double Dy[M], dty[M], dtly[M], Dly[M];
        double dtz = P.a0 - eps / z;
#pragma unroll
        for (int i = 0; i < M; i++) dtz -= lam[i] * P.a[i];
        double A[M + 1][M + 1], B[M + 1], sol[M + 1];
        {
            int q = 0;
#pragma unroll
            for (int i = 0; i < M; i++)
#pragma unroll
                for (int k = i; k < M; k++, q++) { A[i][k] = S[q]; A[k][i] = S[q]; }
        }
#pragma unroll
        for (int i = 0; i < M; i++) {
            Dy[i] = P.d[i] + mu[i] / y[i];
            const double Dl = s[i] / lam[i];
            dty[i] = P.c[i] + P.d[i] * y[i] - lam[i] - eps / y[i];
            const double dtl = -P.a[i] * z - y[i] - bb[i] + eps / lam[i] + S[NSYM + M + i];
            Dly[i] = Dl + 1.0 / Dy[i];
            dtly[i] = dtl + dty[i] / Dy[i];
            A[i][i] += Dly[i];
            A[i][M] = P.a[i];
            A[M][i] = P.a[i];
            B[i] = dtly[i] - S[NSYM + i];
        }
        A[M][M] = -zeta / z;
        B[M] = dtz;
        solve_small<M + 1>(A, B, sol, M + 1);
        double dl[M], dy[M], dmu[M], ds[M];
        const double dz = sol[M];
        double tymax = 0.0;
#pragma unroll
        for (int i = 0; i < M; i++) {
            dl[i] = sol[i];
            dy[i] = dl[i] / Dy[i] - dty[i] / Dy[i];
            dmu[i] = -mu[i] * dy[i] / y[i] - mu[i] + eps / y[i];
            ds[i] = -s[i] * dl[i] / lam[i] - s[i] + eps / lam[i];
            const double t = dmax(dmax(dmax(-1.01 * dy[i] / y[i], -1.01 * dl[i] / lam[i]), -1.01 * dmu[i] / mu[i]),
                                  -1.01 * ds[i] / s[i]);
            if (tymax < t) tymax = t;
        }
        const double dzeta = -zeta * dz / z - zeta + eps / z;
        // KKT norm at w (MMA.h:421-461)
        double kkt = S[NS - 1];
        double lama = 0.0;
#pragma unroll
        for (int i = 0; i < M; i++) {
            kkt += sq(P.c[i] + P.d[i] * y[i] - lam[i] - mu[i]) + sq(S[NSYM + M + i] - P.a[i] * z - y[i] + s[i] - bb[i]) +
                   sq(mu[i] * y[i] - eps) + sq(lam[i] * s[i] - eps);
            lama += lam[i] * P.a[i];
        }
        kkt += sq(P.a0 - zeta - lama) + sq(zeta * z - eps);
        const double dw = sqrt(kkt);
        // ---- phase 2: the Newton direction in x, gsi, ita; the step bound (:293-357)
        double tx = -INFINITY;
        for (long long j = tid; j < n; j += stride) {
            double v = dtx[j];
#pragma unroll
            for (int i = 0; i < M; i++) v += G[(long long)i * n + j] * dl[i];
            const double dxj = -v * iDx[j];
            const double ia = iam[j], ib = ibm[j];
            const double dg = -gsi[j] * dxj * ia - gsi[j] + eps * ia;
            const double di = ita[j] * dxj * ib - ita[j] + eps * ib;
            dx[j] = dxj;
            dgsi[j] = dg;
            dita[j] = di;
            tx = fmax(tx, dmax(dmax(dmax(-1.01 * dxj * ia, 1.01 * dxj * ib), -1.01 * dg / gsi[j]), -1.01 * di / ita[j]));
        }
        tx = block_max(tx, sm);
        {
            double none[1] = {0.0};
            if (!grid_sync<0, 1>(P.gs, P.partials, none, tx)) return;
        }
        const double txmax = dmax(0.0, gs_result_max(P.gs));
        double tau = 1.0 / dmax(dmax(dmax(dmax(1.0, txmax), tymax), -1.01 * dz / z), -1.01 * dzeta / zeta);
        // ---- phase 3: halvings on the KKT norm (:371-391); w moves to the last trial point
        double dw1 = 0.0, yp[M], lp[M], mp[M], sp[M], zp = z, zetap = zeta, tau_used = tau;
        for (int ll = 0; ll < 50; ll++) {
            tau_used = tau;
#pragma unroll
            for (int i = 0; i < M; i++) {
                yp[i] = y[i] + tau * dy[i];
                lp[i] = lam[i] + tau * dl[i];
                mp[i] = mu[i] + tau * dmu[i];
                sp[i] = s[i] + tau * ds[i];
            }
            zp = z + tau * dz;
            zetap = zeta + tau * dzeta;
            double a2[M + 1];
#pragma unroll
            for (int i = 0; i <= M; i++) a2[i] = 0.0;
            for (long long j = tid; j < n; j += stride) {
                const double xp = x[j] + tau * dx[j], gp = gsi[j] + tau * dgsi[j], ip = ita[j] + tau * dita[j];
                double plj = p0[j], qlj = q0[j];
                const double iux = 1.0 / (P.U[j] - xp), ixl = 1.0 / (xp - P.L[j]);
#pragma unroll
                for (int i = 0; i < M; i++) {
                    const double pij = pp[(long long)i * n + j], qij = qq[(long long)i * n + j];
                    plj += lp[i] * pij;
                    qlj += lp[i] * qij;
                    a2[i] += pij * iux + qij * ixl;
                }
                a2[M] += sq(plj * (iux * iux) - qlj * (ixl * ixl) - gp + ip) + sq(gp * (xp - al[j]) - eps) +
                         sq(ip * (be[j] - xp) - eps);
            }
            block_sum<M + 1>(a2, sm);
            if (!grid_sync<M + 1, 0>(P.gs, P.partials, a2, 0.0)) return;
            double k1 = gs_result(P.gs, M), la = 0.0;
#pragma unroll
            for (int i = 0; i < M; i++) {
                k1 += sq(P.c[i] + P.d[i] * yp[i] - lp[i] - mp[i]) +
                      sq(gs_result(P.gs, i) - P.a[i] * zp - yp[i] + sp[i] - bb[i]) + sq(mp[i] * yp[i] - eps) +
                      sq(lp[i] * sp[i] - eps);
                la += lp[i] * P.a[i];
            }
            k1 += sq(P.a0 - zetap - la) + sq(zetap * zp - eps);
            dw1 = sqrt(k1);
            if (dw1 < dw) break;
            tau *= 0.5;
        }
        for (long long j = tid; j < n; j += stride) {
            x[j] = x[j] + tau_used * dx[j];
            gsi[j] = gsi[j] + tau_used * dgsi[j];
            ita[j] = ita[j] + tau_used * dita[j];
        }
#pragma unroll
        for (int i = 0; i < M; i++) {
            y[i] = yp[i];
            lam[i] = lp[i];
            mu[i] = mp[i];
            s[i] = sp[i];
        }
        z = zp;
        zeta = zetap;
        // the KKT norm at the new w is that of the last trial (MMA.h:405-411)
        if (dw1 < 0.9 * eps) eps *= 0.1;
        // every per-variable array is read and written by the thread that owns the variable, so the
        // next phase needs no barrier here
    }
    // ---- history and the new design (:414-418)
    for (long long j = tid; j < n; j += stride) {
        P.xkm2[j] = P.xkm1[j];
        P.xkm1[j] = P.xk[j];
        P.xk[j] = x[j];
    }
    if (tid == 0) {
        P.out[0] = l;
        P.out[1] = eps;
        P.out[2] = capped;
    }
}

// the n <= m update (n <= 4): the (n+1) system in (x, z) (MMA.h:292-330), one thread
__global__ void mma_small_kernel(Params P) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    const int n = P.n, m = P.m;
    double al[kMaxM], be[kMaxM], p0[kMaxM], q0[kMaxM], p[kMaxM][kMaxM], q[kMaxM][kMaxM], bb[kMaxM];
    double L[kMaxM], U[kMaxM], x[kMaxM], gsi[kMaxM], ita[kMaxM];
    for (int i = 0; i < m; i++) bb[i] = -P.g[i];
    for (int j = 0; j < n; j++) {
        setup_var(P, j, L[j], U[j], al[j], be[j]);
        const double xj = P.xk[j], raa = P.raa0 / (P.xmax[j] - P.xmin[j]);
        const double ux = U[j] - xj, xl = xj - L[j];
        pq_of(P.dfdx[j], ux, xl, raa, p0[j], q0[j]);
        for (int i = 0; i < m; i++) pq_of(P.dgdx[(long long)i * n + j], ux, xl, raa, p[i][j], q[i][j]);
    }
    for (int i = 0; i < m; i++)
        for (int j = 0; j < n; j++) {
            const double xj = P.xk[j];
            bb[i] += p[i][j] / (U[j] - xj) + q[i][j] / (xj - L[j]);
        }
    double y[kMaxM], lam[kMaxM], s[kMaxM], mu[kMaxM];
    for (int i = 0; i < m; i++) { y[i] = 1.0; lam[i] = 1.0; s[i] = 1.0; mu[i] = dmax(1.0, 0.5 * P.c[i]); }
    for (int j = 0; j < n; j++) {
        x[j] = 0.5 * (al[j] + be[j]);
        gsi[j] = dmax(1.0, 1.0 / (x[j] - al[j]));
        ita[j] = dmax(1.0, 1.0 / (be[j] - x[j]));
    }
    double eps = 1.0, z = 1.0, zeta = 1.0;
    // KKT norm (MMA.h:421-461) at a point
    auto kkt = [&](const double *xv, const double *yv, double zv, const double *lv, const double *gv, const double *iv,
                   const double *mv, double zev, const double *sv) {
        double norm = 0.0, g[kMaxM] = {0.0, 0.0, 0.0, 0.0}, la = 0.0;
        for (int j = 0; j < n; j++) {
            double pl = p0[j], ql = q0[j];
            for (int i = 0; i < m; i++) {
                pl += lv[i] * p[i][j];
                ql += lv[i] * q[i][j];
                g[i] += p[i][j] / (U[j] - xv[j]) + q[i][j] / (xv[j] - L[j]);
            }
            norm += sq(pl / sq(U[j] - xv[j]) - ql / sq(xv[j] - L[j]) - gv[j] + iv[j]);
            norm += sq(gv[j] * (xv[j] - al[j]) - eps);
            norm += sq(iv[j] * (be[j] - xv[j]) - eps);
        }
        for (int i = 0; i < m; i++) {
            norm += sq(P.c[i] + P.d[i] * yv[i] - lv[i] - mv[i]);
            norm += sq(g[i] - P.a[i] * zv - yv[i] + sv[i] - bb[i]);
            norm += sq(mv[i] * yv[i] - eps);
            norm += sq(lv[i] * sv[i] - eps);
            la += lv[i] * P.a[i];
        }
        norm += sq(P.a0 - zev - la);
        norm += sq(zev * zv - eps);
        return sqrt(norm);
    };
    int l = 0, capped = 0;
    for (; eps > 1.0e-7; l++) {
        if (l >= P.max_newton) { capped = 1; break; }
        double pl[kMaxM], ql[kMaxM], G[kMaxM][kMaxM], Dx[kMaxM], dtx[kMaxM];
        for (int j = 0; j < n; j++) {
            pl[j] = p0[j];
            ql[j] = q0[j];
            for (int i = 0; i < m; i++) { pl[j] += lam[i] * p[i][j]; ql[j] += lam[i] * q[i][j]; }
        }
        for (int i = 0; i < m; i++)
            for (int j = 0; j < n; j++) G[i][j] = p[i][j] / sq(U[j] - x[j]) - q[i][j] / sq(x[j] - L[j]);
        for (int j = 0; j < n; j++) {
            const double ux = U[j] - x[j], xl = x[j] - L[j];
            Dx[j] = 2.0 * pl[j] / (ux * ux * ux) + 2.0 * ql[j] / (xl * xl * xl) + gsi[j] / (x[j] - al[j]) + ita[j] / (be[j] - x[j]);
            dtx[j] = pl[j] / sq(ux) - ql[j] / sq(xl) - eps / (x[j] - al[j]) + eps / (be[j] - x[j]);
        }
        double Dy[kMaxM], Dl[kMaxM], dty[kMaxM], dtl[kMaxM], Dly[kMaxM], dtly[kMaxM];
        double dtz = P.a0 - eps / z;
        for (int i = 0; i < m; i++) dtz -= lam[i] * P.a[i];
        for (int i = 0; i < m; i++) {
            Dy[i] = P.d[i] + mu[i] / y[i];
            Dl[i] = s[i] / lam[i];
            dty[i] = P.c[i] + P.d[i] * y[i] - lam[i] - eps / y[i];
            dtl[i] = -P.a[i] * z - y[i] - bb[i] + eps / lam[i];
            for (int j = 0; j < n; j++) dtl[i] += p[i][j] / (U[j] - x[j]) + q[i][j] / (x[j] - L[j]);
            Dly[i] = Dl[i] + 1.0 / Dy[i];
            dtly[i] = dtl[i] + dty[i] / Dy[i];
        }
        double A[kMaxM + 1][kMaxM + 1], B[kMaxM + 1], sol[kMaxM + 1];
        for (int r = 0; r <= n; r++) for (int c = 0; c <= n; c++) A[r][c] = 0.0;
        for (int ii = 0; ii < n; ii++) {
            for (int jj = 0; jj < n; jj++)
                for (int kk = 0; kk < m; kk++) A[ii][jj] += G[kk][ii] * G[kk][jj] / Dly[kk];
            A[ii][ii] += Dx[ii];
            for (int jj = 0; jj < m; jj++) {
                A[ii][n] -= G[jj][ii] * P.a[jj] / Dly[jj];
                A[n][ii] -= G[jj][ii] * P.a[jj] / Dly[jj];
                A[n][n] += P.a[jj] * P.a[jj] / Dly[jj];
            }
        }
        A[n][n] += zeta / z;
        for (int ii = 0; ii < n; ii++) {
            B[ii] = -dtx[ii];
            for (int jj = 0; jj < m; jj++) B[ii] -= G[jj][ii] * dtly[jj] / Dly[jj];
        }
        B[n] = -dtz;
        for (int jj = 0; jj < m; jj++) B[n] += P.a[jj] * dtly[jj] / Dly[jj];
        solve_small<kMaxM + 1>(A, B, sol, n + 1);
        double dx[kMaxM], dz = sol[n], dl[kMaxM], dy[kMaxM], dmu[kMaxM], ds[kMaxM], dgsi[kMaxM], dita[kMaxM];
        for (int j = 0; j < n; j++) dx[j] = sol[j];
        for (int i = 0; i < m; i++) {
            dl[i] = -P.a[i] * dz / Dly[i] + dtly[i] / Dly[i];
            for (int j = 0; j < n; j++) dl[i] += G[i][j] * dx[j] / Dly[i];
            dy[i] = dl[i] / Dy[i] - dty[i] / Dy[i];
            dmu[i] = -mu[i] * dy[i] / y[i] - mu[i] + eps / y[i];
            ds[i] = -s[i] * dl[i] / lam[i] - s[i] + eps / lam[i];
        }
        for (int j = 0; j < n; j++) {
            dgsi[j] = -gsi[j] * dx[j] / (x[j] - al[j]) - gsi[j] + eps / (x[j] - al[j]);
            dita[j] = ita[j] * dx[j] / (be[j] - x[j]) - ita[j] + eps / (be[j] - x[j]);
        }
        const double dzeta = -zeta * dz / z - zeta + eps / z;
        double txmax = 0.0, tymax = 0.0;
        for (int j = 0; j < n; j++) {
            const double t = dmax(dmax(dmax(-1.01 * dx[j] / (x[j] - al[j]), 1.01 * dx[j] / (be[j] - x[j])),
                                       -1.01 * dgsi[j] / gsi[j]), -1.01 * dita[j] / ita[j]);
            if (txmax < t) txmax = t;
        }
        for (int i = 0; i < m; i++) {
            const double t = dmax(dmax(dmax(-1.01 * dy[i] / y[i], -1.01 * dl[i] / lam[i]), -1.01 * dmu[i] / mu[i]),
                                  -1.01 * ds[i] / s[i]);
            if (tymax < t) tymax = t;
        }
        double tau = 1.0 / dmax(dmax(dmax(dmax(1.0, txmax), tymax), -1.01 * dz / z), -1.01 * dzeta / zeta);
        const double dw = kkt(x, y, z, lam, gsi, ita, mu, zeta, s);
        double xp[kMaxM], yp[kMaxM], lp[kMaxM], gp[kMaxM], ip[kMaxM], mp[kMaxM], sp[kMaxM], zp = z, zetap = zeta;
        double dw1 = 0.0;
        for (int ll = 0; ll < 50; ll++) {
            for (int j = 0; j < n; j++) { xp[j] = x[j] + tau * dx[j]; gp[j] = gsi[j] + tau * dgsi[j]; ip[j] = ita[j] + tau * dita[j]; }
            for (int i = 0; i < m; i++) { yp[i] = y[i] + tau * dy[i]; lp[i] = lam[i] + tau * dl[i]; mp[i] = mu[i] + tau * dmu[i]; sp[i] = s[i] + tau * ds[i]; }
            zp = z + tau * dz;
            zetap = zeta + tau * dzeta;
            dw1 = kkt(xp, yp, zp, lp, gp, ip, mp, zetap, sp);
            if (dw1 < dw) break;
            tau *= 0.5;
        }
        for (int j = 0; j < n; j++) { x[j] = xp[j]; gsi[j] = gp[j]; ita[j] = ip[j]; }
        for (int i = 0; i < m; i++) { y[i] = yp[i]; lam[i] = lp[i]; mu[i] = mp[i]; s[i] = sp[i]; }
        z = zp;
        zeta = zetap;
        if (kkt(x, y, z, lam, gsi, ita, mu, zeta, s) < 0.9 * eps) eps *= 0.1;
    }
    for (int j = 0; j < n; j++) {
        P.L[j] = L[j];
        P.U[j] = U[j];
        P.xkm2[j] = P.xkm1[j];
        P.xkm1[j] = P.xk[j];
        P.xk[j] = x[j];
    }
    P.out[0] = l;
    P.out[1] = eps;
    P.out[2] = capped;
}

}  // namespace mmagen
}  // namespace psf

// ------------------------------------------------------------------ host object
using psf::mmagen::Params;

struct psf_mma {
    int n = 0, m = 0, k = 0;
    double a0 = 1.0, a[psf::mmagen::kMaxM] = {0}, c[psf::mmagen::kMaxM] = {0}, d[psf::mmagen::kMaxM] = {0};
    double raa0 = 1.0e-5, albefa = 0.1, move = 0.5, asyinit = 0.5, asydecr = 0.7, asyincr = 1.2, epsvalue = 1.0e-5;
    double *xmin = nullptr, *xmax = nullptr, *L = nullptr, *U = nullptr, *xkm1 = nullptr, *xkm2 = nullptr;
    double *w = nullptr, *x = nullptr, *dfdx = nullptr, *dgdx = nullptr, *out = nullptr, *partials = nullptr;
    psf::GridSync *gs = nullptr;
    cudaStream_t stream = nullptr;
    int num_sms = 0;
    std::vector<void *> allocs;
};

namespace {
psf_status mma_alloc(psf_mma *o, void **p, size_t bytes) {
    cudaError_t e = cudaMalloc(p, bytes ? bytes : 16);
    if (e != cudaSuccess) return psf::cuda_status(e, "cudaMalloc (MMA)");
    o->allocs.push_back(*p);
    return PSF_OK;
}
void mma_free(psf_mma *o) {
    if (!o) return;
    if (o->stream) cudaStreamSynchronize(o->stream);
    for (void *p : o->allocs) cudaFree(p);
    if (o->stream) cudaStreamDestroy(o->stream);
    delete o;
}

template <int M>
psf_status launch_gen(psf_mma *o, Params &P) {
    const void *fn = (const void *)psf::mmagen::mma_gen_kernel<M>;
    int per_sm = 0;
    PSF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, psf::mmagen::mma_gen_kernel<M>,
                                                           psf::mmagen::kThreads, 0));
    if (per_sm < 1) { psf::set_error("MMA kernel does not fit on an SM"); return PSF_CUDA_ERROR; }
    long long blocks = (long long)o->num_sms * (per_sm < 2 ? per_sm : 2);
    const long long need = (o->n + psf::mmagen::kThreads - 1) / psf::mmagen::kThreads;
    if (blocks > need) blocks = need;
    if (blocks < 1) blocks = 1;
    void *args[] = {&P};
    PSF_CUDA(cudaMemsetAsync(o->gs, 0, sizeof(psf::GridSync), o->stream));
    PSF_CUDA(cudaLaunchCooperativeKernel(fn, dim3((unsigned)blocks), dim3(psf::mmagen::kThreads), args, 0, o->stream));
    psf::note_launch();
    return PSF_OK;
}
}  // namespace

extern "C" {

psf_status psf_mma_create(int n, int m, double a0, const double *a, const double *c, const double *d,
                          const double *xmin, const double *xmax, psf_mma **out) {
    if (!out) { psf::set_error("psf_mma_create: null output"); return PSF_BAD_INPUT; }
    *out = nullptr;
    if (n < 1 || m < 1 || m > psf::mmagen::kMaxM || !a || !c || !d || !xmin || !xmax) {
        psf::set_error("psf_mma_create: need n >= 1, 1 <= m <= 4 and the a, c, d, xmin, xmax arrays");
        return PSF_BAD_INPUT;
    }
    for (int j = 0; j < n; j++)
        if (!(xmax[j] > xmin[j])) {
            psf::set_error("psf_mma_create: xmax must exceed xmin for every variable");
            return PSF_BAD_INPUT;
        }
    psf_mma *o = new psf_mma;
    o->n = n;
    o->m = m;
    o->a0 = a0;
    for (int i = 0; i < m; i++) { o->a[i] = a[i]; o->c[i] = c[i]; o->d[i] = d[i]; }
    int dev = 0;
    psf_status s = psf::cuda_status(cudaGetDevice(&dev), "cudaGetDevice");
    if (s == PSF_OK) s = psf::cuda_status(cudaDeviceGetAttribute(&o->num_sms, cudaDevAttrMultiProcessorCount, dev), "sms");
    if (s == PSF_OK) s = psf::cuda_status(cudaStreamCreateWithFlags(&o->stream, cudaStreamNonBlocking), "stream");
    const size_t nb = sizeof(double) * (size_t)n;
    for (double **p : {&o->xmin, &o->xmax, &o->L, &o->U, &o->xkm1, &o->xkm2, &o->x, &o->dfdx})
        if (s == PSF_OK) s = mma_alloc(o, (void **)p, nb);
    if (s == PSF_OK) s = mma_alloc(o, (void **)&o->dgdx, nb * psf::mmagen::kMaxM);
    if (s == PSF_OK) s = mma_alloc(o, (void **)&o->w, nb * (14 + 3 * psf::mmagen::kMaxM));
    if (s == PSF_OK) s = mma_alloc(o, (void **)&o->out, sizeof(double) * 4);
    if (s == PSF_OK) s = mma_alloc(o, (void **)&o->gs, sizeof(psf::GridSync));
    if (s == PSF_OK) s = mma_alloc(o, (void **)&o->partials, sizeof(double) * psf::kPartialSlots * 4096);
    if (s == PSF_OK) s = psf::cuda_status(cudaMemcpy(o->xmin, xmin, nb, cudaMemcpyHostToDevice), "copy");
    if (s == PSF_OK) s = psf::cuda_status(cudaMemcpy(o->xmax, xmax, nb, cudaMemcpyHostToDevice), "copy");
    // xkm1 = xkm2 = 0 (MMA.h:71-72), L = U = 0 until the first update sets them
    for (double *p : {o->xkm1, o->xkm2, o->L, o->U})
        if (s == PSF_OK) s = psf::cuda_status(cudaMemset(p, 0, nb), "memset");
    if (s != PSF_OK) {
        mma_free(o);
        return s;
    }
    *out = o;
    return PSF_OK;
}

psf_status psf_mma_set_parameters(psf_mma *o, double raa0, double albefa, double move, double asyinit, double asydecr,
                                  double asyincr, double epsvalue) {
    if (!o) { psf::set_error("psf_mma_set_parameters: null object"); return PSF_BAD_INPUT; }
    o->raa0 = raa0; o->albefa = albefa; o->move = move; o->asyinit = asyinit; o->asydecr = asydecr;
    o->asyincr = asyincr; o->epsvalue = epsvalue;
    return PSF_OK;
}

psf_status psf_mma_update_host(psf_mma *o, double *x, double f, const double *dfdx, const double *g,
                               const double *dgdx, int *newton_steps) {
    (void)f;   // the reference keeps f for IsConvergence only (MMA.h:414)
    if (!o || !x || !dfdx || !g || !dgdx) { psf::set_error("psf_mma_update_host: null argument"); return PSF_BAD_INPUT; }
    const size_t nb = sizeof(double) * (size_t)o->n;
    PSF_CUDA(cudaMemsetAsync(o->gs, 0, sizeof(psf::GridSync), o->stream));   // status read back below
    PSF_CUDA(cudaMemcpyAsync(o->x, x, nb, cudaMemcpyHostToDevice, o->stream));
    PSF_CUDA(cudaMemcpyAsync(o->dfdx, dfdx, nb, cudaMemcpyHostToDevice, o->stream));
    PSF_CUDA(cudaMemcpyAsync(o->dgdx, dgdx, nb * o->m, cudaMemcpyHostToDevice, o->stream));
    Params P{};
    P.n = o->n; P.m = o->m; P.k = o->k;
    P.a0 = o->a0;
    for (int i = 0; i < o->m; i++) { P.a[i] = o->a[i]; P.c[i] = o->c[i]; P.d[i] = o->d[i]; P.g[i] = g[i]; }
    P.raa0 = o->raa0; P.albefa = o->albefa; P.move = o->move; P.asyinit = o->asyinit; P.asydecr = o->asydecr;
    P.asyincr = o->asyincr;
    P.xmin = o->xmin; P.xmax = o->xmax; P.xk = o->x; P.dfdx = o->dfdx; P.dgdx = o->dgdx;
    P.L = o->L; P.U = o->U; P.xkm1 = o->xkm1; P.xkm2 = o->xkm2; P.w = o->w;
    P.max_newton = 2000;
    P.gs = o->gs; P.partials = o->partials; P.out = o->out;
    psf_status st = PSF_OK;
    if (o->n <= o->m) {
        (psf::mmagen::mma_small_kernel<<<1, 32, 0, o->stream>>>(P), psf::note_launch());
        st = psf::cuda_status(cudaGetLastError(), "mma_small_kernel");
    } else {
        switch (o->m) {
        case 1: st = launch_gen<1>(o, P); break;
        case 2: st = launch_gen<2>(o, P); break;
        case 3: st = launch_gen<3>(o, P); break;
        default: st = launch_gen<4>(o, P); break;
        }
    }
    PSF_CHECK(st);
    double h[3];
    int gst = 0;
    PSF_CUDA(cudaMemcpyAsync(h, o->out, sizeof h, cudaMemcpyDeviceToHost, o->stream));
    PSF_CUDA(cudaMemcpyAsync(&gst, &o->gs->status, sizeof(int), cudaMemcpyDeviceToHost, o->stream));
    PSF_CUDA(cudaMemcpyAsync(x, o->x, nb, cudaMemcpyDeviceToHost, o->stream));
    PSF_CUDA(cudaStreamSynchronize(o->stream));
    if (gst != 0) { psf::set_error("device-side grid barrier wait exceeded its limit"); return (psf_status)gst; }
    o->k++;
    if (newton_steps) *newton_steps = (int)h[0];
    if (h[2] != 0.0) { psf::set_error("MMA interior-point loop hit its step cap"); return PSF_NOT_CONVERGED; }
    return PSF_OK;
}

psf_status psf_mma_destroy(psf_mma *o) {
    mma_free(o);
    return PSF_OK;
}

}  // extern "C"
