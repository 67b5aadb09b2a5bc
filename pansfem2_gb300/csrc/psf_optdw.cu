// psf_optdw.cu -- the MMA / CONLIN interior-point loop with its element-wise
// arithmetic in double-word FP32 (psf_dw.cuh).
//
// The subproblem solvers of MMA.h:116-419 and CONLIN.h:91-365 spend their time in
// per-element expressions with five to nine divisions per Newton step.  On GB300
// those are FP64-pipe bound (about 170 FP64 instructions per element and step).  This
// kernel keeps the same loop, the same reductions (accumulated per thread in double
// words, then summed in FP64 in a fixed order) and the same scalar Newton system in
// FP64, but evaluates the element-wise terms on FP32 pairs: about 2^-48 relative
// precision, against the loop's 1e-7 stopping tolerance.
//
// Safety: the set-up phase (asymptotes, move limits, p/q, in FP64 as before) counts
// values outside the FP32 pair range [1e-30, 1e30]; every reduction is checked for a
// non-finite result.  Either case ends the kernel before any state is written
// (out[3] = 1) and the host reruns the update with the FP64 kernel.  The design,
// asymptotes and history are written only at the end of a successful run.
#include <cmath>

#include "psf_dw.cuh"
#include "psf_internal.cuh"

namespace psf {

namespace {

using dw::D;

struct MmaDwArgs {
    long long n;
    double *xk;                       // in: current design, out: next design
    const double *dfdx, *dgdx;
    double g;                         // constraint value
    double *L, *U, *xkm1, *xkm2;      // MMA state (unused by CONLIN)
    double *Lnew, *Unew;              // asymptotes of this update, copied to L / U at the end
    float2 *w;                        // 19 n double words
    int k;
    double a0, a, c, d, xmin, xmax;
    double raa0, albefa, move, asyinit, asydecr, asyincr;
    int max_newton;
    GridSync *gs;
    double *partials;
    double *out;                      // [0] Newton steps, [1] final eps, [2] capped, [3] needs the FP64 kernel
};

__device__ __forceinline__ double dmax(double a, double b) { return (a < b) ? b : a; }   // std::max
__device__ __forceinline__ double dmin(double a, double b) { return (b < a) ? b : a; }   // std::min
__device__ __forceinline__ double sq(double v) { return v * v; }

// outside the range where an FP32 pair keeps its precision
__device__ __forceinline__ int out_of_range(double v) {
    const double a = fabs(v);
    return !(a < 1e30) || (a != 0.0 && a < 1e-30);
}

__device__ __forceinline__ void dw_add_to(D &acc, D v) { acc = dw::add(acc, v); }

template <bool kConlin>
__global__ void __launch_bounds__(256) mma_dw_kernel(MmaDwArgs A) {
    grid_sync_init();
    __shared__ double sm[32 * 4];
    const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long stride = (long long)gridDim.x * blockDim.x;
    const long long n = A.n;
    float2 *al = A.w, *be = A.w + n, *p0 = A.w + 2 * n, *q0 = A.w + 3 * n, *p1 = A.w + 4 * n, *q1 = A.w + 5 * n,
           *X = A.w + 6 * n, *GS = A.w + 7 * n, *IT = A.w + 8 * n, *Gv = A.w + 9 * n, *Dx = A.w + 10 * n,
           *dtx = A.w + 11 * n, *dX = A.w + 12 * n, *dGS = A.w + 13 * n, *dIT = A.w + 14 * n,
           *iam = A.w + 15 * n, *ibm = A.w + 16 * n, *Lw = A.w + 17 * n, *Uw = A.w + 18 * n;
    const double xr = A.xmax - A.xmin;
    // ---- set-up in FP64: asymptotes, move limits, p/q, b (MMA.h:118-175 / CONLIN.h:92-122),
    //      start point (MMA.h:178-197 / CONLIN.h:125-145)
    {
        double acc[2] = {0.0, 0.0};
        for (long long j = tid; j < n; j += stride) {
            const double xj = A.xk[j];
            double alj, bej, p0j, q0j, p1j, q1j, L = 0.0, U = 0.0;
            const double df = A.dfdx[j], dg = A.dgdx[j];
            const double dfp = dmax(df, 0.0), dfm = dmax(-df, 0.0), dgp = dmax(dg, 0.0), dgm = dmax(-dg, 0.0);
            int bad = 0;
            if constexpr (kConlin) {
                alj = dmax(A.xmin, xj - A.move * xr);
                bej = dmin(A.xmax, xj + A.move * xr);
                const double x2 = sq(xj);
                p0j = dfp; q0j = dfm * x2; p1j = dgp; q1j = dgm * x2;
                acc[0] += p1j * xj + q1j / xj;
                bad |= out_of_range(xj) | (xj <= 0.0);
            } else {
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
                A.Lnew[j] = L;
                A.Unew[j] = U;
                alj = dmax(dmax(A.xmin, L + A.albefa * (xj - L)), xj - A.move * xr);
                bej = dmin(dmin(A.xmax, U - A.albefa * (U - xj)), xj + A.move * xr);
                const double ux = U - xj, xl = xj - L;
                p0j = sq(ux) * (1.001 * dfp + 0.001 * dfm + A.raa0 / xr);
                q0j = sq(xl) * (0.001 * dfp + 1.001 * dfm + A.raa0 / xr);
                p1j = sq(ux) * (1.001 * dgp + 0.001 * dgm + A.raa0 / xr);
                q1j = sq(xl) * (0.001 * dgp + 1.001 * dgm + A.raa0 / xr);
                acc[0] += p1j / ux + q1j / xl;
                bad |= out_of_range(L) | out_of_range(U) | out_of_range(ux) | out_of_range(xl);
                dw::st(Lw, j, dw::from_double(L));
                dw::st(Uw, j, dw::from_double(U));
            }
            const double x0 = 0.5 * (alj + bej);
            const double g0 = dmax(1.0, 1.0 / (x0 - alj)), i0 = dmax(1.0, 1.0 / (bej - x0));
            bad |= out_of_range(alj) | out_of_range(bej) | out_of_range(p0j) | out_of_range(q0j) |
                   out_of_range(p1j) | out_of_range(q1j) | out_of_range(x0) | out_of_range(g0) | out_of_range(i0) |
                   out_of_range(x0 - alj) | out_of_range(bej - x0);
            acc[1] += (double)bad;
            dw::st(al, j, dw::from_double(alj));
            dw::st(be, j, dw::from_double(bej));
            dw::st(p0, j, dw::from_double(p0j));
            dw::st(q0, j, dw::from_double(q0j));
            dw::st(p1, j, dw::from_double(p1j));
            dw::st(q1, j, dw::from_double(q1j));
            dw::st(X, j, dw::from_double(x0));
            dw::st(GS, j, dw::from_double(g0));
            dw::st(IT, j, dw::from_double(i0));
        }
        block_sum<2>(acc, sm);
        if (!grid_sync<2, 0>(A.gs, A.partials, acc, 0.0)) return;
    }
    if (gs_result(A.gs, 1) != 0.0 || !isfinite(gs_result(A.gs, 0))) {
        if (tid == 0) A.out[3] = 1.0;
        return;
    }
    const double b = -A.g + gs_result(A.gs, 0);
    const D c101 = dw::from_double(1.01);
    // The scalar recurrences of the interior point (the (m+1) Newton system, step bounds,
    // the backtracking decisions, eps) run in thread 0 of each block: every block sees the
    // same reduced sums, so all agree.  The element loops read the double-word scalars they
    // need from shared memory.  (Run redundantly by every thread, those few hundred FP64
    // instructions per step cost as much as the element work on GB300's FP64 pipe.)
    __shared__ float s_dw[12];   // lam, eps, dl, tau, lp, tau_used as double words
    __shared__ int s_ctl[2];     // [0] loop control / break flag, [1] non-finite reduction
    const bool lead = threadIdx.x == 0;
    double eps = 1.0, y = 1.0, z = 1.0, zeta = 1.0, lam = 1.0, s = 1.0;   // meaningful in the lead thread
    double mu = dmax(1.0, 0.5 * A.c);
    double dy = 0.0, dl = 0.0, dmu = 0.0, ds = 0.0, dz = 0.0, dzeta = 0.0, tymax = 0.0, dwn = 0.0;
    int l = 0, capped = 0;
    auto put = [&](int k, double v) {
        const D d = dw::from_double(v);
        s_dw[k] = d.h;
        s_dw[k + 1] = d.l;
    };
    auto get = [&](int k) { return dw::make(s_dw[k], s_dw[k + 1]); };
    auto bail = [&]() {
        if (tid == 0) A.out[3] = 1.0;
    };
    for (;; l++) {
        if (lead) {
            s_ctl[0] = (eps > 1.0e-7) ? (l >= A.max_newton ? 2 : 1) : 0;
            put(0, lam);
            put(2, eps);
        }
        __syncthreads();
        {
            const int ctl = s_ctl[0];
            if (ctl != 1) { capped = ctl == 2; break; }
        }
        const D lamD = get(0), epsD = get(2);
        // ---- phase 1: G, 1/Dx, deltilx and the sums of the Newton system + KKT norm at w.
        //      From the second step on it first takes the previous step's accepted trial point,
        //      x += tau dx (and the same for the multipliers), in the expressions of the trial.
        const bool pend = l > 0;
        const D tauA = get(10);
        D a0 = dw::from_float(0.f), a1 = a0, a2 = a0, a3 = a0;
        for (long long j = tid; j < n; j += stride) {
            D x = dw::ld(X, j), gsi = dw::ld(GS, j), ita = dw::ld(IT, j);
            if (pend) {
                x = dw::add(x, dw::mul(tauA, dw::ld(dX, j)));
                gsi = dw::add(gsi, dw::mul(tauA, dw::ld(dGS, j)));
                ita = dw::add(ita, dw::mul(tauA, dw::ld(dIT, j)));
                dw::st(X, j, x);
                dw::st(GS, j, gsi);
                dw::st(IT, j, ita);
            }
            const D P1 = dw::ld(p1, j), Q1 = dw::ld(q1, j);
            const D plj = dw::add(dw::ld(p0, j), dw::mul(lamD, P1)), qlj = dw::add(dw::ld(q0, j), dw::mul(lamD, Q1));
            const D xa = dw::sub(x, dw::ld(al, j)), bx = dw::sub(dw::ld(be, j), x);
            const D ia = dw::rcp(xa), ib = dw::rcp(bx);
            D Gj, curv, gpart, gval;
            if constexpr (kConlin) {   // CONLIN.h:148-195
                const D ix = dw::rcp(x), ix2 = dw::sq(ix);
                Gj = dw::sub(P1, dw::mul(Q1, ix2));
                curv = dw::mul(dw::mul(dw::scale2(qlj, 2.f), ix2), ix);
                gpart = dw::sub(plj, dw::mul(qlj, ix2));
                gval = dw::add(dw::mul(P1, x), dw::mul(Q1, ix));
            } else {                   // MMA.h:199-243
                const D iux = dw::rcp(dw::sub(dw::ld(Uw, j), x)), ixl = dw::rcp(dw::sub(x, dw::ld(Lw, j)));
                const D iux2 = dw::sq(iux), ixl2 = dw::sq(ixl);
                Gj = dw::sub(dw::mul(P1, iux2), dw::mul(Q1, ixl2));
                curv = dw::add(dw::mul(dw::mul(dw::scale2(plj, 2.f), iux2), iux),
                               dw::mul(dw::mul(dw::scale2(qlj, 2.f), ixl2), ixl));
                gpart = dw::sub(dw::mul(plj, iux2), dw::mul(qlj, ixl2));
                gval = dw::add(dw::mul(P1, iux), dw::mul(Q1, ixl));
            }
            const D iDx = dw::rcp(dw::add(dw::add(curv, dw::mul(gsi, ia)), dw::mul(ita, ib)));
            const D dtxj = dw::add(dw::sub(gpart, dw::mul(epsD, ia)), dw::mul(epsD, ib));
            dw::st(Gv, j, Gj);
            dw::st(Dx, j, iDx);
            dw::st(dtx, j, dtxj);
            dw::st(iam, j, ia);
            dw::st(ibm, j, ib);
            dw_add_to(a0, dw::mul(dw::mul(Gj, Gj), iDx));
            dw_add_to(a1, dw::mul(dw::mul(Gj, dtxj), iDx));
            dw_add_to(a2, gval);
            const D k1 = dw::add(dw::sub(gpart, gsi), ita);
            const D k2 = dw::sub(dw::mul(gsi, xa), epsD), k3 = dw::sub(dw::mul(ita, bx), epsD);
            dw_add_to(a3, dw::add(dw::add(dw::sq(k1), dw::sq(k2)), dw::sq(k3)));
        }
        D av[4] = {a0, a1, a2, a3};
        double acc[4] = {0.0, 0.0, 0.0, 0.0};
        dw::block_sum_dw<4>(av, acc, sm);
        if (!grid_sync<4, 0>(A.gs, A.partials, acc, 0.0)) return;
        if (lead) {
            const double SGG = gs_result(A.gs, 0), SGd = gs_result(A.gs, 1), Sg = gs_result(A.gs, 2),
                         Skkt = gs_result(A.gs, 3);
            s_ctl[1] = !(isfinite(SGG) && isfinite(SGd) && isfinite(Sg) && isfinite(Skkt));
            // ---- the (m+1) system (MMA.h:226-285 / CONLIN.h:197-291), solvels on 2x2
            const double Dy = A.d + mu / y, Dl = s / lam, dty = A.c + A.d * y - lam - eps / y;
            const double dtz = A.a0 - eps / z - (0.0 + lam * A.a);
            const double dtl = -A.a * z - y - b + eps / lam + Sg;
            const double Dly = Dl + 1.0 / Dy, dtly = dtl + dty / Dy;
            double M00 = SGG + Dly, M01 = A.a, M10 = A.a, M11 = -zeta / z;
            double B0 = dtly - SGd, B1 = dtz;
            if (fabs(M00) < fabs(M10)) {
                double t;
                t = B0; B0 = B1; B1 = t;
                t = M00; M00 = M10; M10 = t;
                t = M01; M01 = M11; M11 = t;
            }
            M11 -= M01 * M10 / M00;
            B1 -= B0 * M10 / M00;
            dz = B1 / M11;
            dl = (B0 - dz * M01) / M00;
            dy = dl / Dy - dty / Dy;
            dmu = -mu * dy / y - mu + eps / y;
            ds = -s * dl / lam - s + eps / lam;
            dzeta = -zeta * dz / z - zeta + eps / z;
            tymax = 0.0;
            const double t = dmax(dmax(dmax(-1.01 * dy / y, -1.01 * dl / lam), -1.01 * dmu / mu), -1.01 * ds / s);
            if (tymax < t) tymax = t;
            dwn = sqrt(Skkt + sq(A.c + A.d * y - lam - mu) + sq(Sg - A.a * z - y + s - b) + sq(mu * y - eps) +
                       sq(lam * s - eps) + sq(A.a0 - zeta - (0.0 + lam * A.a)) + sq(zeta * z - eps));
            put(4, dl);
        }
        __syncthreads();
        if (s_ctl[1]) { bail(); return; }
        // ---- phase 2: Newton direction in x, step-length bound (MMA.h:286-360)
        const D dlD = get(4);
        D txd = dw::from_float(-INFINITY);
        for (long long j = tid; j < n; j += stride) {
            const D ia = dw::ld(iam, j), ib = dw::ld(ibm, j), gsi = dw::ld(GS, j), ita = dw::ld(IT, j);
            const D dxj = dw::neg(dw::mul(dw::add(dw::ld(dtx, j), dw::mul(dw::ld(Gv, j), dlD)), dw::ld(Dx, j)));
            const D dg = dw::add(dw::sub(dw::neg(dw::mul(dw::mul(gsi, dxj), ia)), gsi), dw::mul(epsD, ia));
            const D di = dw::add(dw::sub(dw::mul(dw::mul(ita, dxj), ib), ita), dw::mul(epsD, ib));
            dw::st(dX, j, dxj);
            dw::st(dGS, j, dg);
            dw::st(dIT, j, di);
            const D cdx = dw::mul(c101, dxj);
            const D t = dw::max(dw::max(dw::max(dw::neg(dw::mul(cdx, ia)), dw::mul(cdx, ib)),
                                        dw::neg(dw::div(dw::mul(c101, dg), gsi))),
                                dw::neg(dw::div(dw::mul(c101, di), ita)));
            txd = dw::max(txd, t);
        }
        double tx = dw::block_max_dw(txd, sm);
        {
            double none[1] = {0.0};
            if (!grid_sync<0, 1>(A.gs, A.partials, none, tx)) return;
        }
        // ---- phase 3: backtracking on the KKT norm (MMA.h:371-391 / CONLIN.h:323-339)
        double tau = 0.0, tau_used = 0.0, dw1 = 0.0, yp = y, lp = lam, mp = mu, sp = s, zp = z, zetap = zeta;
        if (lead) {
            const double t = gs_result_max(A.gs);
            s_ctl[1] = !isfinite(t);
            double txmax = 0.0;
            if (txmax < t) txmax = t;
            tau = 1.0 / dmax(dmax(dmax(dmax(1.0, txmax), tymax), -1.01 * dz / z), -1.01 * dzeta / zeta);
        }
        for (int ll = 0; ll < 50; ll++) {
            if (lead) {
                tau_used = tau;
                yp = y + tau * dy; lp = lam + tau * dl; mp = mu + tau * dmu;
                sp = s + tau * ds; zp = z + tau * dz; zetap = zeta + tau * dzeta;
                put(6, tau);
                put(8, lp);
            }
            __syncthreads();
            if (s_ctl[1]) { bail(); return; }
            const D tauD = get(6), lpD = get(8);
            D b0 = dw::from_float(0.f), b1 = b0;
            for (long long j = tid; j < n; j += stride) {
                const D xp = dw::add(dw::ld(X, j), dw::mul(tauD, dw::ld(dX, j)));
                const D gp = dw::add(dw::ld(GS, j), dw::mul(tauD, dw::ld(dGS, j)));
                const D ip = dw::add(dw::ld(IT, j), dw::mul(tauD, dw::ld(dIT, j)));
                const D P1 = dw::ld(p1, j), Q1 = dw::ld(q1, j);
                const D plj = dw::add(dw::ld(p0, j), dw::mul(lpD, P1)), qlj = dw::add(dw::ld(q0, j), dw::mul(lpD, Q1));
                D gpart;
                if constexpr (kConlin) {
                    const D ix = dw::rcp(xp);
                    dw_add_to(b0, dw::add(dw::mul(P1, xp), dw::mul(Q1, ix)));
                    gpart = dw::sub(plj, dw::mul(qlj, dw::sq(ix)));
                } else {
                    const D iux = dw::rcp(dw::sub(dw::ld(Uw, j), xp)), ixl = dw::rcp(dw::sub(xp, dw::ld(Lw, j)));
                    dw_add_to(b0, dw::add(dw::mul(P1, iux), dw::mul(Q1, ixl)));
                    gpart = dw::sub(dw::mul(plj, dw::sq(iux)), dw::mul(qlj, dw::sq(ixl)));
                }
                const D k1 = dw::add(dw::sub(gpart, gp), ip);
                const D k2 = dw::sub(dw::mul(gp, dw::sub(xp, dw::ld(al, j))), epsD);
                const D k3 = dw::sub(dw::mul(ip, dw::sub(dw::ld(be, j), xp)), epsD);
                dw_add_to(b1, dw::add(dw::add(dw::sq(k1), dw::sq(k2)), dw::sq(k3)));
            }
            D bv[2] = {b0, b1};
            double a2v[2] = {0.0, 0.0};
            dw::block_sum_dw<2>(bv, a2v, sm);
            if (!grid_sync<2, 0>(A.gs, A.partials, a2v, 0.0)) return;
            if (lead) {
                const double Sgt = gs_result(A.gs, 0), Skt = gs_result(A.gs, 1);
                s_ctl[1] = !(isfinite(Sgt) && isfinite(Skt));
                dw1 = sqrt(Skt + sq(A.c + A.d * yp - lp - mp) + sq(Sgt - A.a * zp - yp + sp - b) + sq(mp * yp - eps) +
                           sq(lp * sp - eps) + sq(A.a0 - zetap - (0.0 + lp * A.a)) + sq(zetap * zp - eps));
                s_ctl[0] = dw1 < dwn;
                if (!(dw1 < dwn)) tau *= 0.5;
            }
            __syncthreads();
            if (s_ctl[1]) { bail(); return; }
            if (s_ctl[0]) break;
        }
        // ---- accept the last trial point: its step length goes to the next phase 1 (or to the
        //      final pass), which applies it element by element with the trial's expressions
        if (lead) {
            put(10, tau_used);
            y = yp; lam = lp; mu = mp; s = sp; z = zp; zeta = zetap;
            if (dw1 < 0.9 * eps) eps *= 0.1;
        }
        __syncthreads();   // every thread has read the backtracking's s_ctl before the lead rewrites it
    }
    // ---- history, asymptotes and the new design (MMA.h:413-418; CONLIN.h:361-364), with the
    //      last accepted step applied to x
    const bool pend = l > 0;
    const D tauA = get(10);
    for (long long j = tid; j < n; j += stride) {
        if constexpr (!kConlin) {
            A.xkm2[j] = A.xkm1[j];
            A.xkm1[j] = A.xk[j];
            A.L[j] = A.Lnew[j];
            A.U[j] = A.Unew[j];
        }
        D x = dw::ld(X, j);
        if (pend) x = dw::add(x, dw::mul(tauA, dw::ld(dX, j)));
        A.xk[j] = dw::to_double(x);
    }
    if (tid == 0) {
        A.out[0] = l;
        A.out[1] = eps;
        A.out[2] = capped;
        A.out[3] = 0.0;
    }
}

}  // namespace

static int coop_blocks_dw(Ctx *c, const void *fn, int threads, long long work) {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, 0) != cudaSuccess || per_sm < 1) return 0;
    const int bps = c->opt_blocks_per_sm;   // psf_set_launch_shape(PSF_KERNEL_OPT)
    int blocks = c->num_sms * (per_sm < bps ? per_sm : bps);
    long long need = (work + threads - 1) / threads;
    if (blocks > need) blocks = (int)need;
    return blocks < 1 ? 1 : blocks;
}

// One MMA (conlin = false) or CONLIN update with the double-word kernel.  *done is
// false when the data left the double-word range: nothing was written and the
// caller runs the FP64 kernel.
psf_status mma_dw_update(Ctx *c, bool conlin, double *x, const double *dfdx, double g, const double *dgdx,
                         int *newton, bool *capped, bool *done) {
    *done = false;
    MmaDwArgs A{};
    A.n = c->ne;
    A.xk = x;
    A.dfdx = dfdx;
    A.dgdx = dgdx;
    A.g = g;
    double *wd = c->mma_work;   // 21 n doubles: 19 n double words, then Lnew, Unew
    A.w = (float2 *)wd;
    A.Lnew = wd + 19 * c->ne;
    A.Unew = wd + 20 * c->ne;
    if (conlin) {
        A.k = c->cl_k;
        A.a0 = c->cl_a0; A.a = c->cl_a; A.c = c->cl_c; A.d = c->cl_d; A.xmin = c->cl_xmin; A.xmax = c->cl_xmax;
        A.move = c->cl_move;
    } else {
        A.L = c->mma_L; A.U = c->mma_U; A.xkm1 = c->mma_xkm1; A.xkm2 = c->mma_xkm2;
        A.k = c->mma_k;
        A.a0 = c->mma_a0; A.a = c->mma_a; A.c = c->mma_c; A.d = c->mma_d; A.xmin = c->mma_xmin; A.xmax = c->mma_xmax;
        A.raa0 = c->mma_raa0; A.albefa = c->mma_albefa; A.move = c->mma_move; A.asyinit = c->mma_asyinit;
        A.asydecr = c->mma_asydecr; A.asyincr = c->mma_asyincr;
    }
    A.max_newton = 2000;
    A.gs = c->gs;
    A.partials = c->partials;
    A.out = c->scal + 4;
    const void *fn = conlin ? (const void *)mma_dw_kernel<true> : (const void *)mma_dw_kernel<false>;
    const int blocks = coop_blocks_dw(c, fn, 256, c->ne);
    if (!blocks) { set_error("double-word MMA kernel does not fit"); return PSF_CUDA_ERROR; }
    void *args[] = {&A};
    PSF_CHECK(launch_coop(c, fn, blocks, 256, args));
    PSF_CHECK(read_sync_status(c));
    double h[4];
    PSF_CUDA(cudaMemcpyAsync(h, c->scal + 4, sizeof h, cudaMemcpyDeviceToHost, c->stream));
    PSF_CUDA(cudaStreamSynchronize(c->stream));
    if (h[3] != 0.0) return PSF_OK;   // out of range: the caller falls back
    *done = true;
    if (newton) *newton = (int)h[0];
    *capped = h[2] != 0.0;
    return PSF_OK;
}

}  // namespace psf
