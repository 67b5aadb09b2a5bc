// psf_learned.cu -- PSF_SOLVE_IR_LEARNED_F32: flexible CG in FP64 whose
// preconditioner is a learned two-level cycle, plus the harvesting of training
// pairs from the method's own solves and the training loop of the network.
//
// Preconditioner z = M(r) (FP32 smoothing, bf16 network):
//   x = l1-Jacobi sweeps (nu_pre) on K x = r from x = 0
//   r1 = r - K x;  s = rms(D^-1/2 r1) over the free dofs
//   x += D^-1/2 * s * U(rho, D^-1/2 r1 / s)      (the U-Net correction)
//   x = l1-Jacobi sweeps (nu_post);  z = x in FP64
// with D the l1 row sums of K (the smoother of the multigrid solver).  The
// network is trained to map (density, D^-1/2 r1 / s) to D^1/2 K^-1 r1 / s, so
// an exact network makes M exact.  FCG(1) in FP64 around it
// (beta = -(z . q_prev) / (p_prev . q_prev)) tolerates the nonlinear
// preconditioner; the FP64 true residual decides convergence, and after a
// stall the solve falls back to FP64 Jacobi PCG from the current iterate.
//
// One FCG iteration is ~30 kernels (smoothing, 15 convolutions, 3 upsamplings,
// FP64 operator, updates) captured once as a CUDA graph and replayed; every
// kernel returns at once when the device-side "done" flag is set, so replays
// past convergence cost only launch latency.  Reductions are per-block
// partials of a fixed grid folded in a fixed order: deterministic.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "psf_ebe.cuh"
#include "psf_internal.cuh"
#include "psf_unet.cuh"

// training pairs on the device (one slot per pair)
struct psf_trainset {
    int H = 0, W = 0, cap = 0, n = 0;
    double out_scale = 0.0;   // rms of the stored targets (0: not computed for the current pairs)
    int scale_n = 0;          // pair count out_scale was computed over
    int kind = -1, nd = 0;    // problem kind of the harvested pairs (Q4 only)
    float Ke[64];             // element matrix (E = 1) of the grid, for the energy loss
    psf::unet::bf16 *in = nullptr;   // cap x H x W x 8: network input (density, rhat, zeros)
    float *tgt = nullptr;            // cap x H x W x 2: D^1/2 K^-1 r1 / s
    float *mask = nullptr;           // cap x H x W x 2: free dofs, weighted 1 / mean(tgt^2) per pair
    float *rhat = nullptr;           // cap x H x W x 2: D^-1/2 r1 / s in fp32
    float *isd = nullptr;            // cap x H x W x 2: D^-1/2 (0 on fixed dofs)
    float *epad = nullptr;           // cap x (H+1)(W+1): zero-padded element moduli
    double *cden = nullptr;          // cap: tgt . rhat, the energy of the exact correction
};

namespace psf {

using unet::bf16;

constexpr int kLpBlocks = 608;
constexpr int kLpThreads = 256;
constexpr int kGraphIters = 4;   // FCG iterations per host check
constexpr int kMaxBatchAngle = 16;   // training batch limit of the scale-free loss

// scalar slots
enum { S_SCALE = 0, S_ZQ, S_PQPREV, S_PQ, S_RP, S_RR, S_BB, S_EPS2, S_FIRST, S_OMEGA, S_NSC = 16 };
// flag slots
enum { F_DONE = 0, F_ITERS, F_NONFINITE, F_LIMIT, F_ITMAX, F_N = 8 };

struct Learned {
    unet::Net *net = nullptr;
    int pre_mg = 0;   // pre-stage: 0 = nu_pre l1-Jacobi sweeps, 1 = one multigrid V-cycle
    int nu_pre = 2, nu_post = 2, use_net = 1;
    int fallback_after = 0;
    int ref_iters = 0;   // iterations of the last converged learned solve (the stall reference)
    float *r32 = nullptr, *xa = nullptr, *xb = nullptr, *r1 = nullptr, *isd = nullptr, *rho = nullptr;
    bf16 *nnin = nullptr;
    double *part = nullptr, *sc = nullptr;
    int *flags = nullptr, *hflags = nullptr;
    double *hsc = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    float graph_scale = 0.0f;
    size_t graph_nodes = 0;   // kernel nodes of the captured graph (kGraphIters FCG iterations)
    float inv_e1 = 1.0f;   // 1 / E1 of the design (density features)
    float *dcorr = nullptr;   // the network's correction in x space (before its step length)
    std::vector<void *> allocs;
};

// ------------------------------------------------------------------ device pieces
__device__ __forceinline__ bool lp_done(const int *flags) { return *(volatile const int *)flags != 0; }

// fold kLpBlocks partials of NV values (fixed order); every thread gets the result
template <int NV>
__device__ __forceinline__ void fold_parts(const double *part, double (&out)[NV]) {
    __shared__ double s_out[NV];
    if (threadIdx.x < 32) {
#pragma unroll
        for (int v = 0; v < NV; v++) {
            double a = 0.0;
            for (int i = threadIdx.x; i < kLpBlocks; i += 32) a += part[i * NV + v];
            a = warp_sum(a);
            if (threadIdx.x == 0) s_out[v] = a;
        }
    }
    __syncthreads();
#pragma unroll
    for (int v = 0; v < NV; v++) out[v] = s_out[v];
    __syncthreads();
}

template <int NV>
__device__ __forceinline__ void write_parts(double (&v)[NV], double *part) {
    __shared__ double sm[32 * NV];
    block_sum<NV>(v, sm);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < NV; k++) part[blockIdx.x * NV + k] = v[k];
    }
}

// r32 = r; x = r / D (the first sweep from zero)
__global__ void lp_first_kernel(long long nd, const double *__restrict__ r, const float *__restrict__ D,
                                const unsigned char *__restrict__ fixed, float *__restrict__ r32,
                                float *__restrict__ x, const int *flags) {
    if (lp_done(flags)) return;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nd; i += (long long)gridDim.x * blockDim.x) {
        const float rv = fixed[i] ? 0.0f : (float)r[i];
        r32[i] = rv;
        x[i] = fixed[i] ? 0.0f : rv / D[i];
    }
}

// xout = xin + (r32 - K xin) / D on free dofs
template <int KIND>
__global__ void lp_sweep_kernel(Geo g, KeT<float> Ke, const float *__restrict__ Ep, const float *__restrict__ D,
                                const unsigned char *__restrict__ fixed, const float *__restrict__ r32,
                                const float *__restrict__ xin, float *__restrict__ xout, const int *flags) {
    if (lp_done(flags)) return;
    constexpr int nd = ndof_of<KIND>();
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < g.nnodes;
         n += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        node_ijk<KIND>(g, n, i, j, k);
        float y[nd];
        ebe_node<float, KIND>(g, Ke, Ep, i, j, k, [&](long long a) { return xin[a]; }, y);
#pragma unroll
        for (int a = 0; a < nd; a++) {
            const long long d = n * nd + a;
            xout[d] = fixed[d] ? 0.0f : xin[d] + (r32[d] - y[a]) / D[d];
        }
    }
}

// r1 = r32 - K x; partial sum of (D^-1/2 r1)^2
template <int KIND>
__global__ void __launch_bounds__(kLpThreads) lp_resid_kernel(Geo g, KeT<float> Ke, const float *__restrict__ Ep,
                                                              const unsigned char *__restrict__ fixed,
                                                              const float *__restrict__ r32,
                                                              const float *__restrict__ x,
                                                              const float *__restrict__ isd, float *__restrict__ r1,
                                                              double *part, const int *flags) {
    if (lp_done(flags)) return;
    constexpr int nd = ndof_of<KIND>();
    double v[1] = {0.0};
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < g.nnodes;
         n += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        node_ijk<KIND>(g, n, i, j, k);
        float y[nd];
        ebe_node<float, KIND>(g, Ke, Ep, i, j, k, [&](long long a) { return x[a]; }, y);
#pragma unroll
        for (int a = 0; a < nd; a++) {
            const long long d = n * nd + a;
            const float rv = fixed[d] ? 0.0f : r32[d] - y[a];
            r1[d] = rv;
            const double t = (double)(isd[d] * rv);
            v[0] += t * t;
        }
    }
    write_parts<1>(v, part);
}

// network input: density, D^-1/2 r1 / s per dof, zeros; s = rms over the free dofs
// channels: 0 node density, 1-2 D^-1/2 r1 / s per dof, 3-6 (E / E1)^(1/3) of the four
// surrounding elements (the local operator; 0 outside the grid), 7 zero
template <int KIND>
__global__ void __launch_bounds__(kLpThreads) nn_prep_kernel(long long nnodes, long long nfree,
                                                             const double *__restrict__ part,
                                                             const float *__restrict__ r1,
                                                             const float *__restrict__ isd,
                                                             const float *__restrict__ rho, bf16 *__restrict__ nnin,
                                                             double *sc, const int *flags, int ny,
                                                             const float *__restrict__ epad, float inv_e1) {
    if (lp_done(flags)) return;
    constexpr int nd = ndof_of<KIND>();
    double ss[1];
    fold_parts<1>(part, ss);
    double s = nfree > 0 ? sqrt(ss[0] / (double)nfree) : 0.0;
    if (!(s > 0.0) || !isfinite(s)) s = 1.0;
    if (blockIdx.x == 0 && threadIdx.x == 0) sc[S_SCALE] = s;
    const float is = (float)(1.0 / s);
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < nnodes;
         n += (long long)gridDim.x * blockDim.x) {
        float c[8] = {rho[n], 0, 0, 0, 0, 0, 0, 0};
        const int i = (int)(n / (ny + 1)), j = (int)(n % (ny + 1));
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const int ei = i - 1 + (q >> 1), ej = j - 1 + (q & 1);
            const float e = epad[(long long)(ei + 1) * (ny + 2) + (ej + 1)];
            c[3 + q] = e > 0.0f ? cbrtf(e * inv_e1) : 0.0f;
        }
#pragma unroll
        for (int a = 0; a < nd && a < 2; a++) c[1 + a] = isd[n * nd + a] * r1[n * nd + a] * is;
        uint4 o;
        bf16 *h = reinterpret_cast<bf16 *>(&o);
#pragma unroll
        for (int q = 0; q < 8; q++) h[q] = __float2bfloat16_rn(c[q]);
        *reinterpret_cast<uint4 *>(nnin + n * 8) = o;
    }
}

// the correction d = D^-1/2 * s * out on the free dofs
template <int KIND>
__global__ void nn_apply_kernel(long long nnodes, const float *__restrict__ out, const float *__restrict__ isd,
                                const double *sc, float oscale, float *__restrict__ d, const int *flags) {
    if (lp_done(flags)) return;
    constexpr int nd = ndof_of<KIND>();
    const float s = (float)sc[S_SCALE] * oscale;
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < nnodes;
         n += (long long)gridDim.x * blockDim.x) {
#pragma unroll
        for (int a = 0; a < nd; a++) d[n * nd + a] = a < 2 ? isd[n * nd + a] * s * out[n * 2 + a] : 0.0f;
    }
}

// partial sums of d . r1 and d . K d (the energy-optimal step length of the correction)
template <int KIND>
__global__ void __launch_bounds__(kLpThreads) nn_step_kernel(Geo g, KeT<float> Ke, const float *__restrict__ Ep,
                                                             const unsigned char *__restrict__ fixed,
                                                             const float *__restrict__ d,
                                                             const float *__restrict__ r1, double *part,
                                                             const int *flags) {
    if (lp_done(flags)) return;
    constexpr int nd = ndof_of<KIND>();
    double v[2] = {0.0, 0.0};
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < g.nnodes;
         n += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        node_ijk<KIND>(g, n, i, j, k);
        float y[nd];
        ebe_node<float, KIND>(g, Ke, Ep, i, j, k, [&](long long a) { return d[a]; }, y);
#pragma unroll
        for (int a = 0; a < nd; a++) {
            const long long t = n * nd + a;
            if (fixed[t]) continue;
            v[0] += (double)d[t] * r1[t];
            v[1] += (double)d[t] * y[a];
        }
    }
    write_parts<2>(v, part);
}

// x += omega d with omega = (d . r1) / (d . K d), 0 when the correction has no energy
__global__ void __launch_bounds__(kLpThreads) nn_add_kernel(long long nd, const double *part,
                                                            const float *__restrict__ d, float *__restrict__ x,
                                                            double *sc, const int *flags) {
    if (lp_done(flags)) return;
    double v[2];
    fold_parts<2>(part, v);
    const double om = (v[1] > 0.0 && isfinite(v[0] / v[1])) ? v[0] / v[1] : 0.0;
    if (blockIdx.x == 0 && threadIdx.x == 0) sc[S_OMEGA] = om;
    const float w = (float)om;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < nd; t += (long long)gridDim.x * blockDim.x)
        x[t] += w * d[t];
}

// last step of the preconditioner: optional sweep, z = x in FP64, partial z . q_prev
template <int KIND>
__global__ void __launch_bounds__(kLpThreads) lp_last_kernel(Geo g, KeT<float> Ke, const float *__restrict__ Ep,
                                                             const float *__restrict__ D,
                                                             const unsigned char *__restrict__ fixed,
                                                             const float *__restrict__ r32,
                                                             const float *__restrict__ xin, int sweep,
                                                             double *__restrict__ z, const double *__restrict__ qprev,
                                                             double *part, const int *flags) {
    if (lp_done(flags)) return;
    constexpr int nd = ndof_of<KIND>();
    double v[1] = {0.0};
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < g.nnodes;
         n += (long long)gridDim.x * blockDim.x) {
        float y[nd];
#pragma unroll
        for (int a = 0; a < nd; a++) y[a] = 0.0f;
        if (sweep) {
            int i, j, k;
            node_ijk<KIND>(g, n, i, j, k);
            ebe_node<float, KIND>(g, Ke, Ep, i, j, k, [&](long long a) { return xin[a]; }, y);
        }
#pragma unroll
        for (int a = 0; a < nd; a++) {
            const long long d = n * nd + a;
            float xv = xin[d];
            if (sweep) xv += (r32[d] - y[a]) / D[d];
            const double zv = fixed[d] ? 0.0 : (double)xv;
            z[d] = zv;
            v[0] += zv * qprev[d];
        }
    }
    write_parts<1>(v, part);
}

// p = z + beta p, beta = -(z . q_prev) / (p_prev . q_prev) (0 on the first iteration)
__global__ void __launch_bounds__(kLpThreads) fcg_dir_kernel(long long nd, const double *__restrict__ part,
                                                             const double *__restrict__ z, double *__restrict__ p,
                                                             double *sc, const int *flags) {
    if (lp_done(flags)) return;
    double zq[1];
    fold_parts<1>(part, zq);
    const bool first = sc[S_FIRST] != 0.0;
    const double pqp = sc[S_PQPREV];
    const double beta = (first || pqp == 0.0) ? 0.0 : -zq[0] / pqp;
    if (blockIdx.x == 0 && threadIdx.x == 0) sc[S_ZQ] = zq[0];
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nd; i += (long long)gridDim.x * blockDim.x)
        p[i] = z[i] + (first ? 0.0 : beta * p[i]);
}

// q = K p (FP64); partials of p . q and r . p
template <int KIND>
__global__ void __launch_bounds__(kLpThreads) fcg_op_kernel(Geo g, KeT<double> Ke, const double *__restrict__ Ep,
                                                            const unsigned char *__restrict__ fixed,
                                                            const double *__restrict__ p, double *__restrict__ q,
                                                            const double *__restrict__ r, double *part,
                                                            const int *flags) {
    if (lp_done(flags)) return;
    constexpr int nd = ndof_of<KIND>();
    double v[2] = {0.0, 0.0};
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < g.nnodes;
         n += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        node_ijk<KIND>(g, n, i, j, k);
        double y[nd];
        ebe_node<double, KIND>(g, Ke, Ep, i, j, k, [&](long long a) { return p[a]; }, y);
#pragma unroll
        for (int a = 0; a < nd; a++) {
            const long long d = n * nd + a;
            const double qv = fixed[d] ? 0.0 : y[a];
            q[d] = qv;
            v[0] += p[d] * qv;
            v[1] += r[d] * p[d];
        }
    }
    write_parts<2>(v, part);
}

// alpha = (r . p) / (p . q); x += alpha p; r -= alpha q; partial |r|^2
__global__ void __launch_bounds__(kLpThreads) fcg_step_kernel(long long nd, const double *__restrict__ part_in,
                                                              const double *__restrict__ p,
                                                              const double *__restrict__ q, double *__restrict__ x,
                                                              double *__restrict__ r, double *part_out, double *sc,
                                                              const int *flags) {
    if (lp_done(flags)) return;
    double pr[2];
    fold_parts<2>(part_in, pr);
    const double alpha = pr[0] != 0.0 ? pr[1] / pr[0] : 0.0;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        sc[S_PQ] = pr[0];
        sc[S_RP] = pr[1];
    }
    double v[1] = {0.0};
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nd; i += (long long)gridDim.x * blockDim.x) {
        x[i] += alpha * p[i];
        const double rv = r[i] - alpha * q[i];
        r[i] = rv;
        v[0] += rv * rv;
    }
    write_parts<1>(v, part_out);
}

// one block: convergence test on the recurrence residual, iteration count, bookkeeping
__global__ void fcg_check_kernel(const double *part, double *sc, int *flags) {
    if (lp_done(flags)) return;
    double rr[1];
    fold_parts<1>(part, rr);
    if (threadIdx.x == 0) {
        sc[S_RR] = rr[0];
        sc[S_PQPREV] = sc[S_PQ];
        sc[S_FIRST] = 0.0;
        const int it = flags[F_ITERS] + 1;
        flags[F_ITERS] = it;
        if (!isfinite(rr[0]) || !isfinite(sc[S_PQ])) {
            flags[F_NONFINITE] = 1;
            flags[F_DONE] = 1;
        } else if (rr[0] <= sc[S_EPS2] * sc[S_BB]) {
            flags[F_DONE] = 1;
        } else if (it >= flags[F_ITMAX]) {
            flags[F_LIMIT] = 1;
            flags[F_DONE] = 1;
        }
    }
}

// r = b - K x (FP64) and |b|^2 into the partials (2 values)
template <int KIND>
__global__ void __launch_bounds__(kLpThreads) lp_residual_kernel(Geo g, KeT<double> Ke, const double *__restrict__ Ep,
                                                                 const unsigned char *__restrict__ fixed,
                                                                 const double *__restrict__ b,
                                                                 const double *__restrict__ x, double *__restrict__ r,
                                                                 double *part) {
    constexpr int nd = ndof_of<KIND>();
    double v[2] = {0.0, 0.0};
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < g.nnodes;
         n += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        node_ijk<KIND>(g, n, i, j, k);
        double y[nd];
        ebe_node<double, KIND>(g, Ke, Ep, i, j, k, [&](long long a) { return x[a]; }, y);
#pragma unroll
        for (int a = 0; a < nd; a++) {
            const long long d = n * nd + a;
            const double rv = fixed[d] ? 0.0 : b[d] - y[a];
            r[d] = rv;
            v[0] += rv * rv;
            v[1] += fixed[d] ? 0.0 : b[d] * b[d];
        }
    }
    write_parts<2>(v, part);
}

__global__ void lp_start_kernel(const double *part, double eps, int itmax, double *sc, int *flags) {
    double v[2];
    fold_parts<2>(part, v);
    if (threadIdx.x == 0) {
        sc[S_RR] = v[0];
        sc[S_BB] = v[1];
        sc[S_EPS2] = eps * eps;
        sc[S_FIRST] = 1.0;
        sc[S_PQPREV] = 0.0;
        flags[F_ITERS] = 0;
        flags[F_NONFINITE] = 0;
        flags[F_LIMIT] = 0;
        flags[F_ITMAX] = itmax;
        flags[F_DONE] = (v[1] == 0.0 || v[0] <= eps * eps * v[1]) ? 1 : 0;
    }
}

// node density feature: mean over the 4 surrounding elements of (E / E1)^(1/3) (padding counts as 0)
__global__ void rho_node_kernel(int nx, int ny, const double *__restrict__ Epad, double E1, float *__restrict__ rho) {
    const long long nn = (long long)(nx + 1) * (ny + 1);
    const double inv = E1 > 0.0 ? 1.0 / E1 : 1.0;
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < nn; n += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(n / (ny + 1)), j = (int)(n % (ny + 1));
        double s = 0.0;
        for (int di = -1; di <= 0; di++)
            for (int dj = -1; dj <= 0; dj++) {
                const double e = Epad[(long long)(i + di + 1) * (ny + 2) + (j + dj + 1)];
                s += e > 0.0 ? cbrt(e * inv) : 0.0;
            }
        rho[n] = (float)(0.25 * s);
    }
}

// D^-1/2 on free dofs, 0 on fixed
__global__ void isd_kernel(long long nd, const float *__restrict__ D, const unsigned char *__restrict__ fixed,
                           float *__restrict__ isd) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nd; i += (long long)gridDim.x * blockDim.x)
        isd[i] = (fixed[i] || !(D[i] > 0.0f)) ? 0.0f : rsqrtf(D[i]);
}

// ------------------------------------------------------------------ host
template <class T>
static psf_status lp_alloc(Learned *L, T **p, size_t n) {
    void *q = nullptr;
    cudaError_t e = cudaMalloc(&q, std::max<size_t>(n, 1) * sizeof(T));
    if (e != cudaSuccess) return cuda_status(e, "cudaMalloc (learned preconditioner)");
    L->allocs.push_back(q);
    *p = reinterpret_cast<T *>(q);
    return PSF_OK;
}

psf_status learned_free(Ctx *c) {
    Learned *L = (Learned *)c->learned;
    if (!L) return PSF_OK;
    if (L->exec) cudaGraphExecDestroy(L->exec);
    if (L->graph) cudaGraphDestroy(L->graph);
    for (void *p : L->allocs) cudaFree(p);
    if (L->hflags) cudaFreeHost(L->hflags);
    if (L->hsc) cudaFreeHost(L->hsc);
    delete L;
    c->learned = nullptr;
    return PSF_OK;
}

static Geo lp_geo(const Ctx *c) {
    Geo g;
    g.nx = c->nx;
    g.ny = c->ny;
    g.nz = c->nz;
    g.nnodes = c->nnodes;
    return g;
}

template <class T>
static KeT<T> lp_ke(const Ctx *c) {
    KeT<T> k{};
    const int nk = c->nen * c->ndof;
    for (int q = 0; q < nk * nk; q++) k.v[q] = (T)c->Ke0_host[q];
    return k;
}

psf_status learned_attach(Ctx *c, unet::Net *net, int pre_mg, int nu_pre, int nu_post, int use_net,
                          int fallback_after) {
    if (c->kind == PSF_H8_SOLID) {
        set_error("learned preconditioner: 2D grids only (Q4 plane strain, Q4 heat)");
        return PSF_BAD_INPUT;
    }
    if (use_net && (!net || net->H[0] != c->nx + 1 || net->W[0] != c->ny + 1)) {
        set_error("learned preconditioner: the network grid must be (nx+1) x (ny+1) nodes");
        return PSF_BAD_INPUT;
    }
    if (nu_pre < 1 || nu_pre > 8 || nu_post < 0 || nu_post > 8) {
        set_error("learned preconditioner: 1 <= nu_pre <= 8, 0 <= nu_post <= 8");
        return PSF_BAD_INPUT;
    }
    if (pre_mg && c->kind == PSF_H8_SOLID) {
        set_error("learned preconditioner: 2D grids only");
        return PSF_BAD_INPUT;
    }
    if (!c->learned) {
        Learned *L = new Learned();
        c->learned = L;
        const size_t nd = c->ndofs;
        psf_status s = PSF_OK;
        if (s == PSF_OK) s = lp_alloc(L, &L->r32, nd);
        if (s == PSF_OK) s = lp_alloc(L, &L->xa, nd);
        if (s == PSF_OK) s = lp_alloc(L, &L->xb, nd);
        if (s == PSF_OK) s = lp_alloc(L, &L->r1, nd);
        if (s == PSF_OK) s = lp_alloc(L, &L->dcorr, nd);
        if (s == PSF_OK) s = lp_alloc(L, &L->isd, nd);
        if (s == PSF_OK) s = lp_alloc(L, &L->rho, c->nnodes);
        if (s == PSF_OK) s = lp_alloc(L, &L->nnin, (size_t)c->nnodes * 8);
        if (s == PSF_OK) s = lp_alloc(L, &L->part, (size_t)kLpBlocks * 4);
        if (s == PSF_OK) s = lp_alloc(L, &L->sc, S_NSC);
        if (s == PSF_OK) s = lp_alloc(L, &L->flags, F_N);
        if (s == PSF_OK) s = cuda_status(cudaMallocHost(&L->hflags, sizeof(int) * F_N), "cudaMallocHost");
        if (s == PSF_OK) s = cuda_status(cudaMallocHost(&L->hsc, sizeof(double) * S_NSC), "cudaMallocHost");
        if (s != PSF_OK) {
            learned_free(c);
            return s;
        }
    }
    Learned *L = (Learned *)c->learned;
    if (L->net != net || L->nu_pre != nu_pre || L->nu_post != nu_post || L->use_net != use_net ||
        L->pre_mg != pre_mg) {
        if (L->exec) cudaGraphExecDestroy(L->exec);
        if (L->graph) cudaGraphDestroy(L->graph);
        L->exec = nullptr;
        L->graph = nullptr;
    }
    L->net = net;
    L->pre_mg = pre_mg ? 1 : 0;
    L->nu_pre = nu_pre;
    L->nu_post = nu_post;
    L->use_net = use_net;
    L->fallback_after = fallback_after;
    return PSF_OK;
}

// per-solve inputs of the preconditioner that depend on the design: D^-1/2 and the density feature
static psf_status lp_refresh(Ctx *c, Learned *L) {
    const int gb = 4 * std::max(c->num_sms, 1);
    (isd_kernel<<<gb, 256, 0, c->stream>>>(c->ndofs, c->Dl1f, c->fixed, L->isd), ::psf::note_launch());
    const double E1 = c->simp_ready && c->prm.E1 > 0 ? c->prm.E1 : 1.0;
    L->inv_e1 = (float)(1.0 / E1);
    (rho_node_kernel<<<gb, 256, 0, c->stream>>>(c->nx, c->ny, c->Epad, E1, L->rho), ::psf::note_launch());
    PSF_CUDA(cudaGetLastError());
    return PSF_OK;
}

psf_status mg_prepare(Ctx *c);                                                        // psf_mg.cu
psf_status mg_apply(Ctx *c, const double *r, float *r32, float *xo, const int *flags);  // psf_mg.cu

// pre-stage of M: r32 = r and x (returned in *cur; *oth is the other buffer)
template <int KIND>
static psf_status lp_pre(Ctx *c, Learned *L, const double *r, const int *fl, float **cur, float **oth) {
    cudaStream_t st = c->stream;
    *cur = L->xa;
    *oth = L->xb;
    if (L->pre_mg) return mg_apply(c, r, L->r32, L->xa, fl);
    const Geo g = lp_geo(c);
    const KeT<float> Kf = lp_ke<float>(c);
    (lp_first_kernel<<<kLpBlocks, kLpThreads, 0, st>>>(
         c->ndofs, r, c->Dl1f, c->fixed, L->r32, L->xa, fl),
     ::psf::note_launch());
    for (int k = 1; k < L->nu_pre; k++) {
        (lp_sweep_kernel<KIND><<<kLpBlocks, kLpThreads, 0, st>>>(g, Kf, c->Epadf, c->Dl1f, c->fixed, L->r32, *cur,
                                                               *oth, fl), ::psf::note_launch());
        std::swap(*cur, *oth);
    }
    PSF_CUDA(cudaGetLastError());
    return PSF_OK;
}

// z = M(r) and the partial sums of z . qprev
template <int KIND>
static psf_status lp_precond(Ctx *c, Learned *L, const double *r, double *z, const double *qprev, const int *fl) {
    cudaStream_t st = c->stream;
    const Geo g = lp_geo(c);
    const KeT<float> Kf = lp_ke<float>(c);
    float *cur, *oth;
    PSF_CHECK(lp_pre<KIND>(c, L, r, fl, &cur, &oth));
    if (L->use_net) {
        (lp_resid_kernel<KIND><<<kLpBlocks, kLpThreads, 0, st>>>(g, Kf, c->Epadf, c->fixed, L->r32, cur, L->isd, L->r1,
                                                               L->part, fl), ::psf::note_launch());
        (nn_prep_kernel<KIND><<<kLpBlocks, kLpThreads, 0, st>>>(c->nnodes, c->nfree, L->part, L->r1, L->isd, L->rho,
                                                              L->nnin, L->sc, fl, c->ny, c->Epadf, L->inv_e1),
                                                              ::psf::note_launch());
        L->net->stream = st;
        L->net->skip = fl;
        PSF_CHECK(L->net->forward(1, L->nnin));
        (nn_apply_kernel<KIND><<<kLpBlocks, kLpThreads, 0, st>>>(c->nnodes, L->net->out32, L->isd, L->sc,
                                                               L->net->out_scale, L->dcorr, fl), ::psf::note_launch());
        (nn_step_kernel<KIND><<<kLpBlocks, kLpThreads, 0, st>>>(
             g, Kf, c->Epadf, c->fixed, L->dcorr, L->r1, L->part, fl),
         ::psf::note_launch());
        (nn_add_kernel<<<kLpBlocks, kLpThreads, 0, st>>>(
             c->ndofs, L->part, L->dcorr, cur, L->sc, fl),
         ::psf::note_launch());
    }
    for (int k = 1; k < L->nu_post; k++) {
        (lp_sweep_kernel<KIND><<<kLpBlocks, kLpThreads, 0, st>>>(
             g, Kf, c->Epadf, c->Dl1f, c->fixed, L->r32, cur, oth, fl),
         ::psf::note_launch());
        std::swap(cur, oth);
    }
    (lp_last_kernel<KIND><<<kLpBlocks, kLpThreads, 0, st>>>(g, Kf, c->Epadf, c->Dl1f, c->fixed, L->r32, cur,
                                                          L->nu_post > 0 ? 1 : 0, z, qprev, L->part, fl),
                                                          ::psf::note_launch());
    PSF_CUDA(cudaGetLastError());
    return PSF_OK;
}

// preconditioner z = M(r) followed by the FCG step; recorded into the capture stream
template <int KIND>
static psf_status lp_iteration(Ctx *c, Learned *L, double *x, double *r, double *z, double *p, double *q) {
    cudaStream_t st = c->stream;
    const Geo g = lp_geo(c);
    const KeT<double> Kd = lp_ke<double>(c);
    const long long nd = c->ndofs;
    const int *fl = L->flags;
    PSF_CHECK(lp_precond<KIND>(c, L, r, z, q, fl));
    (fcg_dir_kernel<<<kLpBlocks, kLpThreads, 0, st>>>(nd, L->part, z, p, L->sc, fl), ::psf::note_launch());
    (fcg_op_kernel<KIND><<<kLpBlocks, kLpThreads, 0, st>>>(
         g, Kd, c->Epad, c->fixed, p, q, r, L->part, fl),
     ::psf::note_launch());
    // the step writes |r|^2 partials into the upper half so that the (p.q, r.p) partials stay readable
    (fcg_step_kernel<<<kLpBlocks, kLpThreads, 0, st>>>(
         nd, L->part, p, q, x, r, L->part + 2 * kLpBlocks, L->sc, fl),
     ::psf::note_launch());
    (fcg_check_kernel<<<1, 32, 0, st>>>(L->part + 2 * kLpBlocks, L->sc, L->flags), ::psf::note_launch());
    PSF_CUDA(cudaGetLastError());
    return PSF_OK;
}

template <int KIND>
static psf_status lp_build_graph(Ctx *c, Learned *L, double *x, double *r, double *z, double *p, double *q) {
    if (L->exec) return PSF_OK;
    cudaStream_t st = c->stream;
    PSF_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    psf_status s = PSF_OK;
    for (int k = 0; k < kGraphIters && s == PSF_OK; k++) s = lp_iteration<KIND>(c, L, x, r, z, p, q);
    cudaGraph_t gph = nullptr;
    cudaError_t e = cudaStreamEndCapture(st, &gph);
    if (s != PSF_OK) {
        if (gph) cudaGraphDestroy(gph);
        return s;
    }
    if (e != cudaSuccess) return cuda_status(e, "cudaStreamEndCapture (learned FCG)");
    e = cudaGraphInstantiate(&L->exec, gph, 0);
    if (e != cudaSuccess) {
        cudaGraphDestroy(gph);
        return cuda_status(e, "cudaGraphInstantiate (learned FCG)");
    }
    L->graph = gph;
    L->graph_nodes = 0;
    cudaGraphGetNodes(gph, nullptr, &L->graph_nodes);
    return PSF_OK;
}

psf_status pcg_ebe_fallback(Ctx *c, const double *b, double *x, int itmax, double eps, int *iters, bool *conv);  // psf_solve.cu

template <int KIND>
static psf_status learned_solve_t(Ctx *c, int itmax, double eps, bool warm, psf_solve_info *info) {
    Learned *L = (Learned *)c->learned;
    cudaStream_t st = c->stream;
    double *x = c->w64[5], *r = c->w64[6], *z = c->w64[7], *p = c->w64[1], *q = c->w64[2];
    const Geo g = lp_geo(c);
    const KeT<double> Kd = lp_ke<double>(c);
    PSF_CHECK(lp_refresh(c, L));
    if (L->pre_mg) PSF_CHECK(mg_prepare(c));
    if (warm)
        PSF_CUDA(cudaMemcpyAsync(x, c->un, sizeof(double) * c->ndofs, cudaMemcpyDeviceToDevice, st));
    else
        PSF_CUDA(cudaMemsetAsync(x, 0, sizeof(double) * c->ndofs, st));
    PSF_CUDA(cudaMemsetAsync(p, 0, sizeof(double) * c->ndofs, st));
    PSF_CUDA(cudaMemsetAsync(q, 0, sizeof(double) * c->ndofs, st));
    // the output scale is a kernel parameter of the captured graph: recapture when it changed
    if (L->exec && L->net && L->graph_scale != L->net->out_scale) {
        cudaGraphExecDestroy(L->exec);
        cudaGraphDestroy(L->graph);
        L->exec = nullptr;
        L->graph = nullptr;
    }
    if (L->net) L->graph_scale = L->net->out_scale;
    PSF_CHECK(lp_build_graph<KIND>(c, L, x, r, z, p, q));
    // automatic stall limit: twice the iterations of the last converged learned solve (at least 100)
    int limit = L->fallback_after > 0 ? L->fallback_after : std::max(100, 2 * L->ref_iters);
    if (L->ref_iters == 0 && L->fallback_after == 0) limit = std::max(limit, 400);
    if (L->fallback_after < 0) limit = itmax;
    limit = std::min(limit, itmax);
    const bool allow_fallback = L->fallback_after >= 0;
    int total = 0, passes = 0;
    bool ok = false, stalled = false;
    double rn = 0.0, bn = 0.0;
    long long glaunch = 0;
    PSF_CUDA(cudaEventRecord(c->evk0, st));
    for (int pass = 0; pass < 3 && total < limit; pass++) {
        passes++;
        (lp_residual_kernel<KIND><<<kLpBlocks, kLpThreads, 0, st>>>(
             g, Kd, c->Epad, c->fixed, c->Fn, x, r, L->part),
         ::psf::note_launch());
        (lp_start_kernel<<<1, 32, 0, st>>>(L->part, eps, limit - total, L->sc, L->flags), ::psf::note_launch());
        PSF_CUDA(cudaGetLastError());
        for (;;) {
            for (int k = 0; k < 2; k++) PSF_CUDA(cudaGraphLaunch(L->exec, st));
            glaunch += 2;
            note_launch(2 * (long long)L->graph_nodes);
            PSF_CUDA(cudaMemcpyAsync(L->hflags, L->flags, sizeof(int) * F_N, cudaMemcpyDeviceToHost, st));
            PSF_CUDA(cudaStreamSynchronize(st));
            if (L->hflags[F_DONE]) break;
        }
        total += L->hflags[F_ITERS];
        if (L->hflags[F_NONFINITE]) {
            stalled = true;
            break;
        }
        if (L->hflags[F_LIMIT]) {
            stalled = true;
            break;
        }
        // FP64 true residual decides
        PSF_CHECK(residual64_pub(c, c->Fn, x, c->w64[3], &rn, &bn));
        if (bn == 0.0 || rn <= eps * bn) {
            ok = true;
            break;
        }
    }
    PSF_CUDA(cudaEventRecord(c->evk1, st));
    PSF_CUDA(cudaEventSynchronize(c->evk1));
    float ms = 0.f;
    PSF_CUDA(cudaEventElapsedTime(&ms, c->evk0, c->evk1));
    c->ksec += ms * 1e-3;
    // kernels launched: residual + start per pass, every node of every graph launch (the
    // iterations after convergence skip their work on the device flag but still launch)
    c->klaunch += 2 * passes + (int)(glaunch * (long long)L->graph_nodes);
    int fb_iters = 0;
    if (!ok && allow_fallback && (stalled || total >= limit)) {
        // fallback: FP64 Jacobi PCG from the current iterate (zero start if the iterate is not finite)
        if (L->hflags[F_NONFINITE]) PSF_CUDA(cudaMemsetAsync(x, 0, sizeof(double) * c->ndofs, st));
        bool conv = false;
        PSF_CHECK(pcg_ebe_fallback(c, c->Fn, x, std::max(itmax - total, 1), eps, &fb_iters, &conv));
        ok = conv;
        info->fell_back = 1;
    } else if (ok) {
        L->ref_iters = total;
    }
    PSF_CUDA(cudaMemcpyAsync(c->un, x, sizeof(double) * c->ndofs, cudaMemcpyDeviceToDevice, st));
    PSF_CHECK(gather_reduced(c, c->un, c->u));
    PSF_CUDA(cudaMemcpyAsync(L->hsc, L->sc, sizeof(double) * S_NSC, cudaMemcpyDeviceToHost, st));
    PSF_CUDA(cudaStreamSynchronize(st));
    info->iterations = total + fb_iters;
    info->outer_iterations = passes;
    info->rel_residual_recurrence = L->hsc[S_BB] > 0 ? sqrt(L->hsc[S_RR] / L->hsc[S_BB]) : 0.0;
    return ok ? PSF_OK : PSF_NOT_CONVERGED;
}

psf_status learned_solve(Ctx *c, int itmax, double eps, bool warm, psf_solve_info *info) {
    if (!c->learned) {
        set_error("psf_solve: no learned preconditioner attached (psf_learned_attach)");
        return PSF_BAD_INPUT;
    }
    switch (c->kind) {
        case PSF_Q4_PLANE_STRAIN: return learned_solve_t<PSF_Q4_PLANE_STRAIN>(c, itmax, eps, warm, info);
        case PSF_Q4_HEAT: return learned_solve_t<PSF_Q4_HEAT>(c, itmax, eps, warm, info);
        default: set_error("learned preconditioner: 2D grids only"); return PSF_BAD_INPUT;
    }
}

// ------------------------------------------------------------------ training pairs
// per-sample weight 1 / mean(target^2) folded into the mask: every pair counts with its relative error
__global__ void tgt_kernel(long long nnodes, int nd, const double *__restrict__ e, const float *__restrict__ isd,
                           const double *sc, float *__restrict__ tgt, float *__restrict__ mask, double *part) {
    const double s = sc[S_SCALE];
    double v[2] = {0.0, 0.0};
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < nnodes;
         n += (long long)gridDim.x * blockDim.x) {
        for (int a = 0; a < 2; a++) {
            float t = 0.0f, m = 0.0f;
            if (a < nd && isd[n * nd + a] > 0.0f) {
                t = (float)(e[n * nd + a] / ((double)isd[n * nd + a] * s));
                m = 1.0f;
            }
            tgt[n * 2 + a] = t;
            mask[n * 2 + a] = m;
            v[0] += (double)t * t;
            v[1] += m;
        }
    }
    write_parts<2>(v, part);
}

__global__ void mask_scale_kernel(long long n, const double *part, float *__restrict__ mask) {
    double v[2];
    fold_parts<2>(part, v);
    const float w = (v[0] > 0.0 && v[1] > 0.0) ? (float)(v[1] / v[0]) : 1.0f;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        mask[i] *= w;
}

// rms of the targets over the masked entries (partials per block; folded by the host)
__global__ void __launch_bounds__(kLpThreads) tgt_rms_kernel(long long n, const float *__restrict__ tgt,
                                                             const float *__restrict__ mask, double *part) {
    double v[2] = {0.0, 0.0};
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        if (mask[i] > 0.0f) {
            v[0] += (double)tgt[i] * tgt[i];
            v[1] += 1.0;
        }
    write_parts<2>(v, part);
}

__global__ void scale_copy_kernel(long long n, const float *__restrict__ a, float s, float *__restrict__ b) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        b[i] = a[i] * s;
}

__global__ void f32_to_f64_kernel(long long n, const float *__restrict__ a, double *__restrict__ b) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        b[i] = (double)a[i];
}

psf_status mg_solve(Ctx *c, int itmax, double eps, bool warm, psf_solve_info *info);  // psf_mg.cu

// energy-loss data of a pair: rhat = D^-1/2 r1 / s, isd in [P][2] layout, partial sums of tgt . rhat
__global__ void __launch_bounds__(kLpThreads) pair_extra_kernel(long long nnodes, int nd, const float *__restrict__ r1,
                                                                const float *__restrict__ isd, const double *sc,
                                                                const float *__restrict__ tgt,
                                                                float *__restrict__ rhat, float *__restrict__ isd2,
                                                                double *part) {
    const double is = 1.0 / sc[S_SCALE];
    double v[1] = {0.0};
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < nnodes;
         n += (long long)gridDim.x * blockDim.x)
        for (int a = 0; a < 2; a++) {
            float rh = 0.0f, id = 0.0f;
            if (a < nd) {
                id = isd[n * nd + a];
                rh = (float)(id * r1[n * nd + a] * is);
            }
            rhat[n * 2 + a] = rh;
            isd2[n * 2 + a] = id;
            v[0] += (double)tgt[n * 2 + a] * rh;
        }
    write_parts<1>(v, part);
}

// energy loss of a batch (the norm flexible CG minimises): per sample
//   L_b = 1 + (y . K^ y - 2 y . rhat) / c_b,   y = oscale * out,  K^ = D^-1/2 K D^-1/2,
// which is the K-norm error of the correction relative to that of the exact one
// (c_b = t . rhat = t . K^ t); gradient d(mean_b L_b)/d out = 2 oscale (K^ y - rhat) / (c_b B).
template <int KIND>
__global__ void __launch_bounds__(kLpThreads) energy_kernel(int nx, int ny, KeT<float> Ke, int B,
                                                            const float *__restrict__ out,
                                                            const float *__restrict__ rhat,
                                                            const float *__restrict__ isd,
                                                            const float *__restrict__ epad,
                                                            const double *__restrict__ cden, float oscale,
                                                            float *__restrict__ gout, double *part) {
    constexpr int nd = ndof_of<KIND>();
    const long long P = (long long)(nx + 1) * (ny + 1), Pe = (long long)(nx + 2) * (ny + 2);
    Geo g;
    g.nx = nx;
    g.ny = ny;
    g.nz = 0;
    g.nnodes = P;
    double v[1] = {0.0};
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < (long long)B * P;
         idx += (long long)gridDim.x * blockDim.x) {
        const int b = (int)(idx / P);
        const long long n = idx - (long long)b * P;
        const float *yb = out + (size_t)b * P * 2, *ib = isd + (size_t)b * P * 2, *rb = rhat + (size_t)b * P * 2;
        int i, j, k;
        node_ijk<KIND>(g, n, i, j, k);
        float kv[nd];
        ebe_node<float, KIND>(g, Ke, epad + (size_t)b * Pe, i, j, k,
                              [&](long long a) {
                                  const long long m = a / nd;
                                  const int d = (int)(a - m * nd);
                                  return ib[m * 2 + d] * oscale * yb[m * 2 + d];
                              },
                              kv);
        const double ic = 1.0 / cden[b];
#pragma unroll
        for (int a = 0; a < 2; a++) {
            float gr = 0.0f;
            if (a < nd && ib[n * 2 + a] > 0.0f) {
                const float yh = oscale * yb[n * 2 + a];
                const float kh = ib[n * 2 + a] * kv[a < nd ? a : 0];
                const float rh = rb[n * 2 + a];
                gr = (float)(2.0 * ((double)kh - rh) * ic * oscale / B);
                v[0] += ((double)yh * kh - 2.0 * (double)yh * rh) * ic;
            }
            gout[(size_t)b * P * 2 + n * 2 + a] = gr;
        }
    }
    write_parts<1>(v, part);
}

// the scale-free form of the energy loss (the solver rescales the correction by its
// energy-optimal step omega): per sample L_b = 1 - (y . rhat)^2 / ((y . K^ y) c_b), the
// K-norm error left by the best multiple of the correction.  Pass 1: K^ y into ky and the
// per-block, per-sample partial sums of y . rhat and y . K^ y.
template <int KIND>
__global__ void __launch_bounds__(kLpThreads) angle_ab_kernel(int nx, int ny, KeT<float> Ke, int B,
                                                              const float *__restrict__ out,
                                                              const float *__restrict__ rhat,
                                                              const float *__restrict__ isd,
                                                              const float *__restrict__ epad, float oscale,
                                                              float *__restrict__ ky, double *part) {
    constexpr int nd = ndof_of<KIND>();
    const long long P = (long long)(nx + 1) * (ny + 1), Pe = (long long)(nx + 2) * (ny + 2);
    Geo g;
    g.nx = nx;
    g.ny = ny;
    g.nz = 0;
    g.nnodes = P;
    double acc[kMaxBatchAngle][2];
#pragma unroll
    for (int b = 0; b < kMaxBatchAngle; b++) acc[b][0] = acc[b][1] = 0.0;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < (long long)B * P;
         idx += (long long)gridDim.x * blockDim.x) {
        const int b = (int)(idx / P);
        const long long n = idx - (long long)b * P;
        const float *yb = out + (size_t)b * P * 2, *ib = isd + (size_t)b * P * 2, *rb = rhat + (size_t)b * P * 2;
        int i, j, k;
        node_ijk<KIND>(g, n, i, j, k);
        float kv[nd];
        ebe_node<float, KIND>(g, Ke, epad + (size_t)b * Pe, i, j, k,
                              [&](long long q) {
                                  const long long m = q / nd;
                                  const int d = (int)(q - m * nd);
                                  return ib[m * 2 + d] * oscale * yb[m * 2 + d];
                              },
                              kv);
        double a = 0.0, bs = 0.0;
#pragma unroll
        for (int c = 0; c < 2; c++) {
            float kh = 0.0f;
            if (c < nd && ib[n * 2 + c] > 0.0f) {
                kh = ib[n * 2 + c] * kv[c < nd ? c : 0];
                const double yh = (double)oscale * yb[n * 2 + c];
                a += yh * rb[n * 2 + c];
                bs += yh * kh;
            }
            ky[(size_t)b * P * 2 + n * 2 + c] = kh;
        }
#pragma unroll
        for (int q = 0; q < kMaxBatchAngle; q++)
            if (q == b) {
                acc[q][0] += a;
                acc[q][1] += bs;
            }
    }
    // per-sample block sums in a fixed order (deterministic)
    __shared__ double sm[64];
    for (int b = 0; b < B; b++) {
        double v[2] = {acc[0][0], acc[0][1]};
#pragma unroll
        for (int q = 1; q < kMaxBatchAngle; q++)
            if (q == b) {
                v[0] = acc[q][0];
                v[1] = acc[q][1];
            }
        block_sum<2>(v, sm);
        if (threadIdx.x == 0) {
            part[(size_t)blockIdx.x * 2 * kMaxBatchAngle + 2 * b] = v[0];
            part[(size_t)blockIdx.x * 2 * kMaxBatchAngle + 2 * b + 1] = v[1];
        }
    }
}

// pass 2: fold the partials (fixed block order), the gradient
// dL_b/dy = oscale (-2 A / (c B) rhat + 2 A^2 / (c B^2) K^ y) / nbatch, and the mean loss
__global__ void __launch_bounds__(kLpThreads) angle_grad_kernel(long long P, int B, const double *part,
                                                                const double *__restrict__ cden,
                                                                const float *__restrict__ rhat,
                                                                const float *__restrict__ ky,
                                                                const float *__restrict__ isd, float oscale,
                                                                float *__restrict__ gout, double *loss) {
    __shared__ double sAB[kMaxBatchAngle * 2];
    if (threadIdx.x < 2 * B) {
        double v = 0.0;
        for (int blk = 0; blk < kLpBlocks; blk++) v += part[(size_t)blk * 2 * kMaxBatchAngle + threadIdx.x];
        sAB[threadIdx.x] = v;
    }
    __syncthreads();
    if (blockIdx.x == 0 && threadIdx.x == 0 && loss) {
        double l = 0.0;
        for (int b = 0; b < B; b++) {
            const double A = sAB[2 * b], Bb = sAB[2 * b + 1], c = cden[b];
            l += (Bb > 0.0 && c > 0.0) ? 1.0 - A * A / (c * Bb) : 1.0;
        }
        *loss = l / B;
    }
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < (long long)B * P * 2;
         idx += (long long)gridDim.x * blockDim.x) {
        const int b = (int)(idx / (P * 2));
        const double A = sAB[2 * b], Bb = sAB[2 * b + 1], c = cden[b];
        float gr = 0.0f;
        if (isd[idx] > 0.0f && Bb > 0.0 && c > 0.0) {
            const double d = -2.0 * A / (c * Bb) * rhat[idx] + 2.0 * A * A / (c * Bb * Bb) * ky[idx];
            gr = (float)(d * oscale / B);
        }
        gout[idx] = gr;
    }
}

__global__ void energy_loss_kernel(const double *part, int B, double *out) {
    double v[1];
    fold_parts<1>(part, v);
    if (threadIdx.x == 0) *out = 1.0 + v[0] / B;
}

__global__ void fold_to_kernel(const double *part, double *out) {
    double v[1];
    fold_parts<1>(part, v);
    if (threadIdx.x == 0) *out = v[0];
}

// one training pair from residual r (FP64 nodal): input (density, scaled r1), target D^1/2 K^-1 r1 / s
template <int KIND>
static psf_status harvest_pair(Ctx *c, Learned *L, const double *r, double *rhs64, double *e64, psf_trainset *ts,
                               size_t slot) {
    const size_t P = (size_t)ts->H * ts->W, Pe = (size_t)(ts->H + 1) * (ts->W + 1);
    bf16 *in_out = ts->in + slot * P * 8;
    float *tgt_out = ts->tgt + slot * P * 2, *mask_out = ts->mask + slot * P * 2;
    cudaStream_t st = c->stream;
    const Geo g = lp_geo(c);
    const KeT<float> Kf = lp_ke<float>(c);
    const long long nd = c->ndofs;
    PSF_CUDA(cudaMemsetAsync(L->flags, 0, sizeof(int) * F_N, st));
    float *cur, *oth;
    if (L->pre_mg) PSF_CHECK(mg_prepare(c));
    PSF_CHECK(lp_pre<KIND>(c, L, r, L->flags, &cur, &oth));
    (lp_resid_kernel<KIND><<<kLpBlocks, kLpThreads, 0, st>>>(g, Kf, c->Epadf, c->fixed, L->r32, cur, L->isd, L->r1,
                                                           L->part, L->flags), ::psf::note_launch());
    (nn_prep_kernel<KIND><<<kLpBlocks, kLpThreads, 0, st>>>(c->nnodes, c->nfree, L->part, L->r1, L->isd, L->rho, in_out,
                                                          L->sc, L->flags, c->ny, c->Epadf, L->inv_e1),
                                                          ::psf::note_launch());
    (f32_to_f64_kernel<<<kLpBlocks, kLpThreads, 0, st>>>(nd, L->r1, rhs64), ::psf::note_launch());
    PSF_CUDA(cudaGetLastError());
    // e = K^-1 r1 with the multigrid FCG to 1e-8 (its right-hand side is the context's nodal load vector)
    double *Fn_saved = c->Fn;
    c->Fn = rhs64;
    psf_solve_info inf{};
    psf_status s = mg_solve(c, 20000, 1e-8, false, &inf);
    c->Fn = Fn_saved;
    if (s == PSF_NOT_CONVERGED) return PSF_NOT_CONVERGED;   // the caller skips this pair
    if (s != PSF_OK) return s;
    PSF_CUDA(cudaMemcpyAsync(e64, c->un, sizeof(double) * nd, cudaMemcpyDeviceToDevice, st));
    (tgt_kernel<<<kLpBlocks, kLpThreads, 0, st>>>(
         c->nnodes, c->ndof, e64, L->isd, L->sc, tgt_out, mask_out, L->part),
     ::psf::note_launch());
    (mask_scale_kernel<<<kLpBlocks, kLpThreads, 0, st>>>(c->nnodes * 2, L->part, mask_out), ::psf::note_launch());
    (pair_extra_kernel<<<kLpBlocks, kLpThreads, 0, st>>>(c->nnodes, c->ndof, L->r1, L->isd, L->sc, tgt_out,
                                                        ts->rhat + slot * P * 2, ts->isd + slot * P * 2, L->part),
                                                        ::psf::note_launch());
    (fold_to_kernel<<<1, 32, 0, st>>>(L->part, ts->cden + slot), ::psf::note_launch());
    PSF_CUDA(cudaMemcpyAsync(ts->epad + slot * Pe, c->Epadf, sizeof(float) * Pe, cudaMemcpyDeviceToDevice, st));
    PSF_CUDA(cudaGetLastError());
    return PSF_OK;
}

}  // namespace psf

// ------------------------------------------------------------------ C ABI: training set, harvest, training

extern "C" {

psf_status psf_trainset_destroy(psf_trainset *t);

psf_status psf_trainset_create(int H, int W, int capacity, psf_trainset **out) {
    if (!out || H < 9 || W < 9 || capacity < 1) return PSF_BAD_INPUT;
    *out = nullptr;
    psf_trainset *t = new psf_trainset();
    t->H = H;
    t->W = W;
    t->cap = capacity;
    const size_t P = (size_t)H * W;
    const size_t Pe = (size_t)(H + 1) * (W + 1);
    cudaError_t e = cudaMalloc(&t->in, sizeof(psf::unet::bf16) * P * 8 * capacity);
    if (e == cudaSuccess) e = cudaMalloc(&t->tgt, sizeof(float) * P * 2 * capacity);
    if (e == cudaSuccess) e = cudaMalloc(&t->mask, sizeof(float) * P * 2 * capacity);
    if (e == cudaSuccess) e = cudaMalloc(&t->rhat, sizeof(float) * P * 2 * capacity);
    if (e == cudaSuccess) e = cudaMalloc(&t->isd, sizeof(float) * P * 2 * capacity);
    if (e == cudaSuccess) e = cudaMalloc(&t->epad, sizeof(float) * Pe * capacity);
    if (e == cudaSuccess) e = cudaMalloc(&t->cden, sizeof(double) * capacity);
    if (e != cudaSuccess) {
        psf_trainset_destroy(t);
        return psf::cuda_status(e, "psf_trainset_create");
    }
    *out = t;
    return PSF_OK;
}

psf_status psf_trainset_destroy(psf_trainset *t) {
    if (t) {
        for (void *p : {(void *)t->in, (void *)t->tgt, (void *)t->mask, (void *)t->rhat, (void *)t->isd,
                        (void *)t->epad, (void *)t->cden})
            if (p) cudaFree(p);
        delete t;
    }
    return PSF_OK;
}

int psf_trainset_size(const psf_trainset *t) { return t ? t->n : 0; }

}  // extern "C"

namespace psf {
psf_status learned_harvest(Ctx *c, psf_trainset *ts, int npairs, const int *iters, int niters) {
    if (!ts || npairs < 1 || ts->H != c->nx + 1 || ts->W != c->ny + 1 || c->kind == PSF_H8_SOLID) {
        set_error("psf_learned_harvest: the training set grid must be (nx+1) x (ny+1) nodes of a 2D problem");
        return PSF_BAD_INPUT;
    }
    if (ts->kind >= 0 && ts->kind != c->kind) {
        set_error("psf_learned_harvest: the training set holds pairs of another problem kind");
        return PSF_BAD_INPUT;
    }
    ts->kind = c->kind;
    ts->nd = c->ndof;
    for (int q = 0; q < 64; q++) ts->Ke[q] = q < (int)c->Ke0_host.size() ? (float)c->Ke0_host[q] : 0.0f;
    if (!c->learned) PSF_CHECK(learned_attach(c, nullptr, 1, 2, 1, 0, 0));
    Learned *L = (Learned *)c->learned;
    PSF_CHECK(lp_refresh(c, L));
    cudaStream_t st = c->stream;
    const size_t P = (size_t)ts->H * ts->W;
    double *rbuf = c->w64[3], *rhs = c->w64[4];
    double *ebuf = nullptr, *un_saved = nullptr;
    PSF_CUDA(cudaMalloc(&ebuf, sizeof(double) * c->ndofs));
    PSF_CUDA(cudaMalloc(&un_saved, sizeof(double) * c->ndofs));
    PSF_CUDA(cudaMemcpyAsync(un_saved, c->un, sizeof(double) * c->ndofs, cudaMemcpyDeviceToDevice, st));
    psf_status s = PSF_OK;
    for (int k = 0; k < npairs && s == PSF_OK; k++) {
        if (ts->n >= ts->cap) break;
        // residual of the mixed-precision multigrid FCG after `it` iterations from zero
        const int it = (iters && niters > 0) ? iters[k % niters] : (k % 4) * 2;
        psf_solve_info inf{};
        if (it > 0) {
            s = mg_solve(c, it, 1e-30, false, &inf);
            if (s == PSF_NOT_CONVERGED) s = PSF_OK;
        } else {
            s = cuda_status(cudaMemsetAsync(c->un, 0, sizeof(double) * c->ndofs, st), "memset");
        }
        double rn, bn;
        if (s == PSF_OK) s = residual64_pub(c, c->Fn, c->un, rbuf, &rn, &bn);
        if (s != PSF_OK) break;
        const size_t slot = (size_t)ts->n;
        switch (c->kind) {
            case PSF_Q4_PLANE_STRAIN: s = harvest_pair<PSF_Q4_PLANE_STRAIN>(c, L, rbuf, rhs, ebuf, ts, slot); break;
            default: s = harvest_pair<PSF_Q4_HEAT>(c, L, rbuf, rhs, ebuf, ts, slot);
        }
        if (s == PSF_OK) ts->n++;
        else if (s == PSF_NOT_CONVERGED) s = PSF_OK;   // no exact target for this residual: skip the pair
    }
    cudaMemcpyAsync(c->un, un_saved, sizeof(double) * c->ndofs, cudaMemcpyDeviceToDevice, st);
    if (s == PSF_OK) s = gather_reduced(c, c->un, c->u);
    cudaStreamSynchronize(st);
    cudaFree(ebuf);
    cudaFree(un_saved);
    return s;
}
}  // namespace psf

extern "C" {

psf_status psf_learned_train(psf_unet *u, psf_trainset *ts, int steps, int batch, float lr, uint64_t seed,
                             int loss_mode, double *loss_hist) {
    if (!u || !ts || steps < 1 || batch < 1 || ts->n < 1 || loss_mode < 0 || loss_mode > 2) return PSF_BAD_INPUT;
    if (loss_mode == 2 && batch > psf::kMaxBatchAngle) {
        psf::set_error("psf_learned_train: the scale-free loss takes batches of at most 16");
        return PSF_BAD_INPUT;
    }
    psf::unet::Net &net = u->net;
    if (net.H[0] != ts->H || net.W[0] != ts->W || batch > net.cap) {
        psf::set_error("psf_learned_train: network grid or batch capacity does not match the training set");
        return PSF_BAD_INPUT;
    }
    const size_t P = (size_t)ts->H * ts->W, Pe = (size_t)(ts->H + 1) * (ts->W + 1);
    float *tgt = nullptr, *mask = nullptr, *rhat = nullptr, *isdb = nullptr, *epad = nullptr;
    double *dl = nullptr, *cden = nullptr, *epart = nullptr;
    PSF_CUDA(cudaMalloc(&tgt, sizeof(float) * (P * 2 * batch * 4 + Pe * batch)));
    mask = tgt + P * 2 * batch;
    rhat = mask + P * 2 * batch;
    isdb = rhat + P * 2 * batch;
    epad = isdb + P * 2 * batch;
    PSF_CUDA(cudaMalloc(&cden, sizeof(double) * (batch + 2 * (size_t)psf::kLpBlocks * psf::kMaxBatchAngle)));
    epart = cden + batch;
    psf::KeT<float> Kf{};
    for (int q = 0; q < 64; q++) Kf.v[q] = ts->Ke[q];
    PSF_CUDA(cudaMalloc(&dl, sizeof(double) * (size_t)steps * 2));
    cudaStream_t st = net.stream;
    // global target scale: the network learns targets of unit rms, the preconditioner scales back
    if (ts->scale_n != ts->n || !(ts->out_scale > 0.0)) {
        double *part = nullptr;
        PSF_CUDA(cudaMalloc(&part, sizeof(double) * 2 * psf::kLpBlocks));
        (psf::tgt_rms_kernel<<<psf::kLpBlocks, psf::kLpThreads, 0, st>>>((long long)ts->n * P * 2, ts->tgt, ts->mask,
                                                                        part), ::psf::note_launch());
        std::vector<double> h(2 * psf::kLpBlocks);
        cudaError_t e = cudaMemcpyAsync(h.data(), part, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        cudaFree(part);
        if (e != cudaSuccess) return psf::cuda_status(e, "target scale");
        double a = 0.0, m = 0.0;
        for (int b = 0; b < psf::kLpBlocks; b++) {
            a += h[2 * b];
            m += h[2 * b + 1];
        }
        ts->out_scale = (m > 0.0 && a > 0.0) ? sqrt(a / m) : 1.0;
        ts->scale_n = ts->n;
    }
    net.out_scale = (float)ts->out_scale;
    uint64_t rs = seed ? seed : 1;
    auto rnd = [&rs]() {
        rs ^= rs << 13;
        rs ^= rs >> 7;
        rs ^= rs << 17;
        return rs;
    };
    psf_status s = PSF_OK;
    const int warm = std::max(1, steps / 20);
    for (int k = 0; k < steps && s == PSF_OK; k++) {
        for (int b = 0; b < batch && s == PSF_OK; b++) {
            const size_t i = (size_t)(rnd() % (uint64_t)ts->n);
            s = psf::cuda_status(cudaMemcpyAsync(net.t[0] + b * P * 8, ts->in + i * P * 8, sizeof(psf::unet::bf16) * P * 8,
                                                 cudaMemcpyDeviceToDevice, st), "copy");
            if (s == PSF_OK) {
                (psf::scale_copy_kernel<<<psf::kLpBlocks, psf::kLpThreads, 0, st>>>(
                    (long long)P * 2, ts->tgt + i * P * 2, (float)(1.0 / ts->out_scale), tgt + b * P * 2),
                    ::psf::note_launch());
                s = psf::cuda_status(cudaGetLastError(), "scale_copy_kernel");
            }
            if (s == PSF_OK)
                s = psf::cuda_status(cudaMemcpyAsync(mask + b * P * 2, ts->mask + i * P * 2, sizeof(float) * P * 2,
                                                     cudaMemcpyDeviceToDevice, st), "copy");
            if (s == PSF_OK && loss_mode >= 1) {
                s = psf::cuda_status(cudaMemcpyAsync(rhat + b * P * 2, ts->rhat + i * P * 2, sizeof(float) * P * 2,
                                                     cudaMemcpyDeviceToDevice, st), "copy");
                if (s == PSF_OK)
                    s = psf::cuda_status(cudaMemcpyAsync(isdb + b * P * 2, ts->isd + i * P * 2, sizeof(float) * P * 2,
                                                         cudaMemcpyDeviceToDevice, st), "copy");
                if (s == PSF_OK)
                    s = psf::cuda_status(cudaMemcpyAsync(epad + b * Pe, ts->epad + i * Pe, sizeof(float) * Pe,
                                                         cudaMemcpyDeviceToDevice, st), "copy");
                if (s == PSF_OK)
                    s = psf::cuda_status(cudaMemcpyAsync(cden + b, ts->cden + i, sizeof(double),
                                                         cudaMemcpyDeviceToDevice, st), "copy");
            }
        }
        // linear warm-up, then cosine decay to 5% of lr
        const double fr = (double)k / steps;
        double lrk = lr * (0.05 + 0.95 * 0.5 * (1.0 + cos(3.141592653589793 * fr)));
        if (k < warm) lrk = lr * (k + 1) / (double)warm;
        if (s == PSF_OK) s = net.forward(batch, nullptr);
        if (s == PSF_OK && loss_mode == 0) s = net.loss_grad(batch, tgt, mask, dl + steps + k, dl + k);
        if (s == PSF_OK && loss_mode == 1) {
            const int nx = ts->H - 1, ny = ts->W - 1;
            if (ts->kind == PSF_Q4_HEAT)
                (psf::energy_kernel<PSF_Q4_HEAT><<<psf::kLpBlocks, psf::kLpThreads, 0, st>>>(
                    nx, ny, Kf, batch, net.out32, rhat, isdb, epad, cden, net.out_scale, net.g[psf::unet::kTensors - 1],
                    epart), ::psf::note_launch());
            else
                (psf::energy_kernel<PSF_Q4_PLANE_STRAIN><<<psf::kLpBlocks, psf::kLpThreads, 0, st>>>(
                    nx, ny, Kf, batch, net.out32, rhat, isdb, epad, cden, net.out_scale, net.g[psf::unet::kTensors - 1],
                    epart), ::psf::note_launch());
            (psf::energy_loss_kernel<<<1, 32, 0, st>>>(epart, batch, dl + k), ::psf::note_launch());
            s = psf::cuda_status(cudaGetLastError(), "energy loss");
        }
        if (s == PSF_OK && loss_mode == 2) {
            const int nx = ts->H - 1, ny = ts->W - 1;
            float *ky = tgt;   // the MSE target buffer is free in this mode
            if (ts->kind == PSF_Q4_HEAT)
                (psf::angle_ab_kernel<PSF_Q4_HEAT><<<psf::kLpBlocks, psf::kLpThreads, 0, st>>>(
                    nx, ny, Kf, batch, net.out32, rhat, isdb, epad, net.out_scale, ky, epart), ::psf::note_launch());
            else
                (psf::angle_ab_kernel<PSF_Q4_PLANE_STRAIN><<<psf::kLpBlocks, psf::kLpThreads, 0, st>>>(
                    nx, ny, Kf, batch, net.out32, rhat, isdb, epad, net.out_scale, ky, epart), ::psf::note_launch());
            (psf::angle_grad_kernel<<<psf::kLpBlocks, psf::kLpThreads, 0, st>>>(
                (long long)P, batch, epart, cden, rhat, ky, isdb, net.out_scale, net.g[psf::unet::kTensors - 1],
                dl + k), ::psf::note_launch());
            s = psf::cuda_status(cudaGetLastError(), "scale-free energy loss");
        }
        if (s == PSF_OK) s = net.backward(batch, nullptr);
        if (s == PSF_OK) s = net.adam((float)lrk);
    }
    if (s == PSF_OK) s = net.check_err();
    if (s == PSF_OK && loss_hist)
        s = psf::cuda_status(cudaMemcpy(loss_hist, dl, sizeof(double) * steps, cudaMemcpyDeviceToHost), "copy");
    cudaFree(tgt);
    cudaFree(dl);
    cudaFree(cden);
    return s;
}

}  // extern "C"

namespace psf {
// z = M(r) once, outside any graph (reduced vectors in, reduced out)
template <int KIND>
static psf_status learned_apply_t(Ctx *c, const double *r_red, double *z_red) {
    Learned *L = (Learned *)c->learned;
    cudaStream_t st = c->stream;
    PSF_CHECK(lp_refresh(c, L));
    double *r = c->w64[3], *z = c->w64[4], *q0 = c->w64[0];
    double *red = nullptr;
    PSF_CUDA(cudaMalloc(&red, sizeof(double) * std::max<long long>(c->nfree, 1)));
    psf_status s0 = cuda_status(cudaMemcpyAsync(red, r_red, sizeof(double) * c->nfree, cudaMemcpyHostToDevice, st),
                                "copy");
    if (s0 == PSF_OK) s0 = scatter_reduced(c, red, r);
    if (s0 != PSF_OK) {
        cudaFree(red);
        return s0;
    }
    PSF_CUDA(cudaMemsetAsync(q0, 0, sizeof(double) * c->ndofs, st));
    PSF_CUDA(cudaMemsetAsync(L->flags, 0, sizeof(int) * F_N, st));
    if (L->pre_mg) {
        psf_status sp = mg_prepare(c);
        if (sp != PSF_OK) {
            cudaFree(red);
            return sp;
        }
    }
    psf_status sq = lp_precond<KIND>(c, L, r, z, q0, L->flags);
    if (sq != PSF_OK) {
        cudaFree(red);
        return sq;
    }
    psf_status s = cuda_status(cudaGetLastError(), "learned apply");
    if (s == PSF_OK) s = gather_reduced(c, z, red);
    if (s == PSF_OK)
        s = cuda_status(cudaMemcpyAsync(z_red, red, sizeof(double) * c->nfree, cudaMemcpyDeviceToHost, st), "copy");
    if (s == PSF_OK) s = cuda_status(cudaStreamSynchronize(st), "sync");
    cudaFree(red);
    if (s == PSF_OK && L->use_net) s = L->net->check_err();
    return s;
}
}  // namespace psf

extern "C" {

psf_status psf_learned_apply(psf_ctx *h, const double *r, double *z) {
    if (!h || !r || !z) return PSF_BAD_INPUT;
    psf::Ctx *c = &h->c;
    if (!c->learned) {
        psf::set_error("psf_learned_apply: no learned preconditioner attached");
        return PSF_BAD_INPUT;
    }
    switch (c->kind) {
        case PSF_Q4_PLANE_STRAIN: return psf::learned_apply_t<PSF_Q4_PLANE_STRAIN>(c, r, z);
        case PSF_Q4_HEAT: return psf::learned_apply_t<PSF_Q4_HEAT>(c, r, z);
        default: return PSF_BAD_INPUT;
    }
}

psf_status psf_learned_attach(psf_ctx *h, psf_unet *net, int pre_mg, int nu_pre, int nu_post, int use_net,
                              int fallback_after) {
    if (!h) return PSF_BAD_INPUT;
    return psf::learned_attach(&h->c, net ? &net->net : nullptr, pre_mg, nu_pre, nu_post, use_net, fallback_after);
}

psf_status psf_learned_harvest(psf_ctx *h, psf_trainset *ts, int npairs, const int *iters, int niters) {
    if (!h) return PSF_BAD_INPUT;
    return psf::learned_harvest(&h->c, ts, npairs, iters, niters);
}

}  // extern "C"

extern "C" {

psf_status psf_learned_eval(psf_unet *u, psf_trainset *ts, int first, int count, int mode, double *mean_rel_energy) {
    if (!u || !ts || !mean_rel_energy || first < 0 || count < 1 || first + count > ts->n || mode < 1 || mode > 2)
        return PSF_BAD_INPUT;
    psf::unet::Net &net = u->net;
    if (net.H[0] != ts->H || net.W[0] != ts->W) {
        psf::set_error("psf_learned_eval: network grid does not match the training set");
        return PSF_BAD_INPUT;
    }
    const size_t P = (size_t)ts->H * ts->W, Pe = (size_t)(ts->H + 1) * (ts->W + 1);
    const int B = net.cap;
    double *dl = nullptr, *part = nullptr;
    float *ky = nullptr;
    PSF_CUDA(cudaMalloc(&dl, sizeof(double) * ((size_t)count + 2 * (size_t)psf::kLpBlocks * psf::kMaxBatchAngle)));
    part = dl + count;
    PSF_CUDA(cudaMalloc(&ky, sizeof(float) * P * 2));
    psf::KeT<float> Kf{};
    for (int q = 0; q < 64; q++) Kf.v[q] = ts->Ke[q];
    cudaStream_t st = net.stream;
    psf_status s = PSF_OK;
    const int nx = ts->H - 1, ny = ts->W - 1;
    std::vector<double> h(count);
    for (int i0 = 0; i0 < count && s == PSF_OK; i0 += B) {
        const int nb = std::min(B, count - i0);
        const size_t i = (size_t)(first + i0);
        // consecutive pairs: the trainset slots are already laid out as a batch
        s = psf::cuda_status(cudaMemcpyAsync(net.t[0], ts->in + i * P * 8, sizeof(psf::unet::bf16) * P * 8 * nb,
                                             cudaMemcpyDeviceToDevice, st), "copy");
        if (s == PSF_OK) s = net.forward(nb, nullptr);
        for (int b = 0; b < nb && s == PSF_OK; b++) {
            const size_t j = i + b;
            float *gsc = net.g[psf::unet::kTensors - 1];   // scratch: the output gradient is not needed
            if (mode == 1) {
                if (ts->kind == PSF_Q4_HEAT)
                    (psf::energy_kernel<PSF_Q4_HEAT><<<psf::kLpBlocks, psf::kLpThreads, 0, st>>>(
                        nx, ny, Kf, 1, net.out32 + b * P * 2, ts->rhat + j * P * 2, ts->isd + j * P * 2,
                        ts->epad + j * Pe, ts->cden + j, net.out_scale, gsc, part), ::psf::note_launch());
                else
                    (psf::energy_kernel<PSF_Q4_PLANE_STRAIN><<<psf::kLpBlocks, psf::kLpThreads, 0, st>>>(
                        nx, ny, Kf, 1, net.out32 + b * P * 2, ts->rhat + j * P * 2, ts->isd + j * P * 2,
                        ts->epad + j * Pe, ts->cden + j, net.out_scale, gsc, part), ::psf::note_launch());
                (psf::energy_loss_kernel<<<1, 32, 0, st>>>(part, 1, dl + i0 + b), ::psf::note_launch());
            } else {
                if (ts->kind == PSF_Q4_HEAT)
                    (psf::angle_ab_kernel<PSF_Q4_HEAT><<<psf::kLpBlocks, psf::kLpThreads, 0, st>>>(
                        nx, ny, Kf, 1, net.out32 + b * P * 2, ts->rhat + j * P * 2, ts->isd + j * P * 2,
                        ts->epad + j * Pe, net.out_scale, ky, part), ::psf::note_launch());
                else
                    (psf::angle_ab_kernel<PSF_Q4_PLANE_STRAIN><<<psf::kLpBlocks, psf::kLpThreads, 0, st>>>(
                        nx, ny, Kf, 1, net.out32 + b * P * 2, ts->rhat + j * P * 2, ts->isd + j * P * 2,
                        ts->epad + j * Pe, net.out_scale, ky, part), ::psf::note_launch());
                (psf::angle_grad_kernel<<<psf::kLpBlocks, psf::kLpThreads, 0, st>>>(
                    (long long)P, 1, part, ts->cden + j, ts->rhat + j * P * 2, ky, ts->isd + j * P * 2, net.out_scale,
                    gsc, dl + i0 + b), ::psf::note_launch());
            }
            s = psf::cuda_status(cudaGetLastError(), "energy loss");
        }
    }
    if (s == PSF_OK) s = net.check_err();
    if (s == PSF_OK) s = psf::cuda_status(cudaMemcpy(h.data(), dl, sizeof(double) * count, cudaMemcpyDeviceToHost), "copy");
    cudaFree(dl);
    cudaFree(ky);
    if (s != PSF_OK) return s;
    double m = 0.0;
    for (double v : h) m += v;
    *mean_rel_energy = m / count;
    return PSF_OK;
}

}  // extern "C"
