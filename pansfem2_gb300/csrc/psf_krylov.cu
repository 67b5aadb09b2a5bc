// psf_krylov.cu -- the remaining Krylov solvers of CG.h on the device: ScalingBiCGSTAB
// (CG.h:457-495), BiCGSTAB2 (:196-253), and the ILU(0) family: ILU0 (:257-284),
// PreILU0 (:288-315), ILU0CG (:319-352), ILU0BiCGSTAB (:356-391).
//
// These solvers are not on the SIMP hot path, so they are written for exactness rather
// than speed: the CSR product is one thread per row summing in column order, the vector
// updates keep the reference's expression order, and this file is compiled without FMA
// contraction, so everything except the dot products (tree order instead of sequential)
// rounds as the reference does.  ILU(0) is level-scheduled: the rows are grouped by the
// depth of their dependence on earlier rows (lower pattern, for the factor and the
// forward solve) or later rows (upper pattern, backward solve), the levels computed
// once on the host from the pattern; one block walks the levels with a block barrier
// between them, every row of a level by its own thread, each row's sums in the
// reference's order (so the factor and the triangular solves are bit-exact with it).
#include <algorithm>
#include <cmath>
#include <vector>

#include "psf_internal.cuh"

namespace psf {
namespace kry {

constexpr int kBlocks = 256, kThreads = 256, kLevelThreads = 1024;

__global__ void spmv_rows(int n, const int *__restrict__ ip, const int *__restrict__ ix, const double *__restrict__ a,
                          const double *__restrict__ x, double *__restrict__ y) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double v = 0.0;
        for (int k = ip[i]; k < ip[i + 1]; k++) v += a[k] * x[ix[k]];
        y[i] = v;
    }
}

// out = c0 v0 + c1 v1 + c2 v2 + c3 v3, left to right (terms with a null vector are absent)
__global__ void comb(int n, double *out, double c0, const double *v0, double c1, const double *v1, double c2,
                     const double *v2, double c3, const double *v3) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double s = c0 * v0[i];
        if (v1) s = s + c1 * v1[i];
        if (v2) s = s + c2 * v2[i];
        if (v3) s = s + c3 * v3[i];
        out[i] = s;
    }
}

// z = a w + b (x - y + c z) (zeawpbxmypcz, CG.h:53-62)
__global__ void comb_wxyz(int n, double a, const double *w, double b, const double *x, const double *y, double c,
                          double *z) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        z[i] = a * w[i] + b * (x[i] - y[i] + c * z[i]);
}

// v = b / D (Scaling, CG.h:408-415)
__global__ void scale_div(int n, const double *b, const double *D, double *v) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) v[i] = b[i] / D[i];
}

// GetDiagonal (CG.h:397-404): CSR::get(i, i), zero when absent
__global__ void diag_of(int n, const int *ip, const int *ix, const double *a, double *D) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        int lo = ip[i], hi = ip[i + 1];
        while (lo < hi) {
            const int mid = lo + (hi - lo) / 2;
            if (ix[mid] < i) lo = mid + 1;
            else hi = mid;
        }
        D[i] = (lo < ip[i + 1] && ix[lo] == i) ? a[lo] : 0.0;
    }
}

// up to 4 dot products a_q . b_q: per-block partials [q][block]
__global__ void __launch_bounds__(kThreads) dots(int n, int k, const double *a0, const double *b0, const double *a1,
                                                 const double *b1, const double *a2, const double *b2,
                                                 const double *a3, const double *b3, double *part) {
    __shared__ double sm[32 * 4];
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    const double *A[4] = {a0, a1, a2, a3}, *B[4] = {b0, b1, b2, b3};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        for (int q = 0; q < k; q++) acc[q] += A[q][i] * B[q][i];
    block_sum<4>(acc, sm);
    if (threadIdx.x == 0)
        for (int q = 0; q < k; q++) part[q * gridDim.x + blockIdx.x] = acc[q];
}
__global__ void dots_finish(const double *part, int nb, int k, double *out) {
    for (int q = 0; q < k; q++) {
        const double v = warp_canonical_sum(part + q * nb, nb);
        if (threadIdx.x == 0) out[q] = v;
    }
}

// position of column col in the sorted columns ix[begin, end), -1 when absent
__device__ __forceinline__ int find_col(const int *ix, int begin, int end, int col) {
    int lo = begin, hi = end;
    while (lo < hi) {
        const int mid = lo + (hi - lo) / 2;
        if (ix[mid] < col) lo = mid + 1;
        else hi = mid;
    }
    return (lo < end && ix[lo] == col) ? lo : -1;
}

// ILU0 (CG.h:257-284) on A's pattern, rows by level; m holds A's values on entry
__global__ void __launch_bounds__(kLevelThreads) ilu0_factor(int nlev, const int *lptr, const int *lrows,
                                                             const int *ip, const int *ix, double *m) {
    for (int lev = 0; lev < nlev; lev++) {
        for (int t = lptr[lev] + threadIdx.x; t < lptr[lev + 1]; t += blockDim.x) {
            const int i = lrows[t];
            for (int e = ip[i]; e < ip[i + 1]; e++) {
                const int j = ix[e];
                double q = m[e];
                const int lim = i <= j ? i : j;
                // q_ij -= q_ik q_kj for the common k < min(i, j), ascending
                for (int kk = ip[i]; kk < ip[i + 1]; kk++) {
                    const int k = ix[kk];
                    if (k >= lim) break;
                    const int p = find_col(ix, ip[k], ip[k + 1], j);
                    if (p >= 0) q = __dsub_rn(q, __dmul_rn(m[kk], m[p]));
                }
                if (i > j) q = __ddiv_rn(q, m[find_col(ix, ip[j], ip[j + 1], j)]);
                m[e] = q;
            }
        }
        __syncthreads();
    }
}

// PreILU0 (CG.h:288-315): v = U^-1 L^-1 b, forward by lower levels, backward by upper levels
__global__ void __launch_bounds__(kLevelThreads) ilu0_apply(int n, int nlo, const int *loptr, const int *lorows,
                                                            int nup, const int *upptr, const int *uprows,
                                                            const int *ip, const int *ix, const double *m,
                                                            const double *b, double *v) {
    for (int i = threadIdx.x; i < n; i += blockDim.x) v[i] = b[i];
    __syncthreads();
    for (int lev = 0; lev < nlo; lev++) {
        for (int t = loptr[lev] + threadIdx.x; t < loptr[lev + 1]; t += blockDim.x) {
            const int i = lorows[t];
            double s = v[i];
            for (int k = ip[i]; k < ip[i + 1]; k++) {
                if (ix[k] < i) s = __dsub_rn(s, __dmul_rn(m[k], v[ix[k]]));
                else break;
            }
            v[i] = s;
        }
        __syncthreads();
    }
    for (int lev = 0; lev < nup; lev++) {
        for (int t = upptr[lev] + threadIdx.x; t < upptr[lev + 1]; t += blockDim.x) {
            const int i = uprows[t];
            double s = v[i];
            for (int k = ip[i + 1] - 1; k >= ip[i]; k--) {
                if (ix[k] > i) s = __dsub_rn(s, __dmul_rn(m[k], v[ix[k]]));
                else break;
            }
            const int d = find_col(ix, ip[i], ip[i + 1], i);
            v[i] = __ddiv_rn(s, d >= 0 ? m[d] : 0.0);
        }
        __syncthreads();
    }
}

// ------------------------------------------------------------------ host
struct Levels {
    std::vector<int> ptr, rows;
};
// rows grouped by dependence depth: lower (k < i in row i) or upper (k > i)
static Levels levels_of(int n, const int *ip, const int *ix, bool lower) {
    std::vector<int> lev(n, 0);
    int nl = 0;
    if (lower) {
        for (int i = 0; i < n; i++) {
            int l = 0;
            for (int k = ip[i]; k < ip[i + 1]; k++)
                if (ix[k] < i) l = std::max(l, lev[ix[k]] + 1);
            lev[i] = l;
            nl = std::max(nl, l + 1);
        }
    } else {
        for (int i = n - 1; i >= 0; i--) {
            int l = 0;
            for (int k = ip[i]; k < ip[i + 1]; k++)
                if (ix[k] > i) l = std::max(l, lev[ix[k]] + 1);
            lev[i] = l;
            nl = std::max(nl, l + 1);
        }
    }
    Levels L;
    L.ptr.assign(nl + 1, 0);
    for (int i = 0; i < n; i++) L.ptr[lev[i] + 1]++;
    for (int l = 0; l < nl; l++) L.ptr[l + 1] += L.ptr[l];
    L.rows.resize(n);
    std::vector<int> fill(L.ptr.begin(), L.ptr.end() - 1);
    for (int i = 0; i < n; i++) L.rows[fill[lev[i]]++] = i;
    return L;
}

struct Engine {
    cudaStream_t s;
    int n;
    double *part, *res;   // partials, device results
    std::vector<void *> allocs;
    psf_status alloc(void **p, size_t bytes) {
        PSF_CUDA(cudaMallocAsync(p, bytes ? bytes : 16, s));
        allocs.push_back(*p);
        return PSF_OK;
    }
    ~Engine() {
        for (void *p : allocs) cudaFreeAsync(p, s);
        cudaStreamSynchronize(s);
    }
    int grid() const { return std::min(kBlocks, std::max(1, (n + kThreads - 1) / kThreads)); }
    psf_status spmv(const int *ip, const int *ix, const double *a, const double *x, double *y) {
        (spmv_rows<<<std::max(1, (n + kThreads - 1) / kThreads), kThreads, 0, s>>>(n, ip, ix, a, x, y), note_launch());
        return cuda_status(cudaGetLastError(), "spmv");
    }
    psf_status lin(double *out, double c0, const double *v0, double c1 = 0, const double *v1 = nullptr,
                   double c2 = 0, const double *v2 = nullptr, double c3 = 0, const double *v3 = nullptr) {
        (comb<<<grid(), kThreads, 0, s>>>(n, out, c0, v0, c1, v1, c2, v2, c3, v3), note_launch());
        return cuda_status(cudaGetLastError(), "comb");
    }
    // k dot products (a_q . b_q) to the host
    psf_status dot(int k, double *out, const double *a0, const double *b0, const double *a1 = nullptr,
                   const double *b1 = nullptr, const double *a2 = nullptr, const double *b2 = nullptr,
                   const double *a3 = nullptr, const double *b3 = nullptr) {
        const int g = grid();
        (dots<<<g, kThreads, 0, s>>>(n, k, a0, b0, a1, b1, a2, b2, a3, b3, part), note_launch());
        (dots_finish<<<1, 32, 0, s>>>(part, g, k, res), note_launch());
        PSF_CUDA(cudaGetLastError());
        PSF_CUDA(cudaMemcpyAsync(out, res, sizeof(double) * k, cudaMemcpyDeviceToHost, s));
        PSF_CUDA(cudaStreamSynchronize(s));
        return PSF_OK;
    }
};

// the ILU(0) factor of A on the device: values on A's pattern, and the level sets of both solves
struct Ilu {
    int *lo_ptr = nullptr, *lo_rows = nullptr, *up_ptr = nullptr, *up_rows = nullptr;
    int nlo = 0, nup = 0;
    double *m = nullptr;
};

static psf_status ilu_setup(Engine &E, int n, const int *h_ip, const int *h_ix, const int *ip, const int *ix,
                            const double *a, const double *m_given, long long nnz, Ilu *F) {
    // every row needs its diagonal in the pattern (the factor divides by it): checked before any launch
    for (int i = 0; i < n; i++)
        if (!std::binary_search(h_ix + h_ip[i], h_ix + h_ip[i + 1], i)) {
            set_error("ILU(0): row " + std::to_string(i) + " has no diagonal entry");
            return PSF_BAD_INPUT;
        }
    const Levels lo = levels_of(n, h_ip, h_ix, true), up = levels_of(n, h_ip, h_ix, false);
    F->nlo = (int)lo.ptr.size() - 1;
    F->nup = (int)up.ptr.size() - 1;
    PSF_CHECK(E.alloc((void **)&F->lo_ptr, sizeof(int) * lo.ptr.size()));
    PSF_CHECK(E.alloc((void **)&F->lo_rows, sizeof(int) * n));
    PSF_CHECK(E.alloc((void **)&F->up_ptr, sizeof(int) * up.ptr.size()));
    PSF_CHECK(E.alloc((void **)&F->up_rows, sizeof(int) * n));
    PSF_CHECK(E.alloc((void **)&F->m, sizeof(double) * nnz));
    PSF_CUDA(cudaMemcpyAsync(F->lo_ptr, lo.ptr.data(), sizeof(int) * lo.ptr.size(), cudaMemcpyHostToDevice, E.s));
    PSF_CUDA(cudaMemcpyAsync(F->lo_rows, lo.rows.data(), sizeof(int) * n, cudaMemcpyHostToDevice, E.s));
    PSF_CUDA(cudaMemcpyAsync(F->up_ptr, up.ptr.data(), sizeof(int) * up.ptr.size(), cudaMemcpyHostToDevice, E.s));
    PSF_CUDA(cudaMemcpyAsync(F->up_rows, up.rows.data(), sizeof(int) * n, cudaMemcpyHostToDevice, E.s));
    if (m_given) {
        PSF_CUDA(cudaMemcpyAsync(F->m, m_given, sizeof(double) * nnz, cudaMemcpyDeviceToDevice, E.s));
    } else {
        PSF_CUDA(cudaMemcpyAsync(F->m, a, sizeof(double) * nnz, cudaMemcpyDeviceToDevice, E.s));
        (ilu0_factor<<<1, kLevelThreads, 0, E.s>>>(F->nlo, F->lo_ptr, F->lo_rows, ip, ix, F->m), note_launch());
        PSF_CUDA(cudaGetLastError());
    }
    // the backward solve divides by the diagonal of the factor (CG.h:311): a zero one is refused
    std::vector<double> hm(nnz);
    PSF_CUDA(cudaMemcpyAsync(hm.data(), F->m, sizeof(double) * nnz, cudaMemcpyDeviceToHost, E.s));
    PSF_CUDA(cudaStreamSynchronize(E.s));
    for (int i = 0; i < n; i++) {
        const int *b = h_ix + h_ip[i], *e = h_ix + h_ip[i + 1];
        const int *p = std::lower_bound(b, e, i);
        if (p == e || *p != i || !(hm[h_ip[i] + (p - b)] != 0.0) || !std::isfinite(hm[h_ip[i] + (p - b)])) {
            set_error("ILU(0): zero or non-finite pivot in row " + std::to_string(i));
            return PSF_BAD_INPUT;
        }
    }
    return PSF_OK;
}

static psf_status ilu_apply(Engine &E, const Ilu &F, const int *ip, const int *ix, const double *b, double *v) {
    (ilu0_apply<<<1, kLevelThreads, 0, E.s>>>(E.n, F.nlo, F.lo_ptr, F.lo_rows, F.nup, F.up_ptr, F.up_rows, ip, ix, F.m,
                                              b, v),
     note_launch());
    return cuda_status(cudaGetLastError(), "ilu0_apply");
}

// The preconditioned BiCGSTAB of ScalingBiCGSTAB (M = D^-1, p0 = M r0, CG.h:457-495) and of
// ILU0BiCGSTAB (M = (LU)^-1, p0 = r0, CG.h:356-391)
static psf_status precond_bicgstab(Engine &E, const int *ip, const int *ix, const double *a, const double *b,
                                   double *x, bool ilu, const double *D, const Ilu *F, int itmax, double eps,
                                   int *iters, double *rrn, double *bbn, int *conv) {
    const int n = E.n;
    double *r, *rd, *p, *Mp, *AMp, *s, *Ms, *AMs;
    for (double **q : {&r, &rd, &p, &Mp, &AMp, &s, &Ms, &AMs}) PSF_CHECK(E.alloc((void **)q, sizeof(double) * n));
    auto M = [&](const double *in, double *out) -> psf_status {
        if (ilu) return ilu_apply(E, *F, ip, ix, in, out);
        (scale_div<<<E.grid(), kThreads, 0, E.s>>>(n, in, D, out), note_launch());
        return cuda_status(cudaGetLastError(), "scale");
    };
    PSF_CUDA(cudaMemsetAsync(x, 0, sizeof(double) * n, E.s));
    PSF_CHECK(E.spmv(ip, ix, a, x, AMp));
    PSF_CHECK(E.lin(r, 1.0, b, -1.0, AMp));   // subtract (CG.h:17-27)
    PSF_CUDA(cudaMemcpyAsync(rd, r, sizeof(double) * n, cudaMemcpyDeviceToDevice, E.s));
    if (ilu) PSF_CUDA(cudaMemcpyAsync(p, r, sizeof(double) * n, cudaMemcpyDeviceToDevice, E.s));
    else PSF_CHECK(M(r, p));
    double h[4];
    PSF_CHECK(E.dot(2, h, rd, r, b, b));
    double rdr = h[0];
    const double bnorm = sqrt(h[1]);
    *bbn = h[1];
    *conv = 0;
    int k = 0;
    double rr = h[0];
    for (; k < itmax; k++) {
        PSF_CHECK(M(p, Mp));
        PSF_CHECK(E.spmv(ip, ix, a, Mp, AMp));
        PSF_CHECK(E.dot(1, h, rd, AMp));
        const double alpha = rdr / h[0];
        PSF_CHECK(E.lin(s, 1.0, r, -alpha, AMp));
        PSF_CHECK(M(s, Ms));
        PSF_CHECK(E.spmv(ip, ix, a, Ms, AMs));
        PSF_CHECK(E.dot(2, h, AMs, s, AMs, AMs));
        const double omega = h[0] / h[1];
        PSF_CHECK(E.lin(x, 1.0, x, alpha, Mp, omega, Ms));
        PSF_CHECK(E.lin(r, 1.0, s, -omega, AMs));
        PSF_CHECK(E.dot(2, h, rd, r, r, r));
        const double beta = alpha / omega * h[0] / rdr;
        PSF_CHECK(E.lin(p, beta, p, 1.0, r, -beta * omega, AMp));
        rdr = h[0];
        rr = h[1];
        if (!std::isfinite(rr)) { k++; break; }
        if (sqrt(rr) < eps * bnorm) { k++; *conv = 1; break; }
    }
    *iters = k;
    *rrn = rr;
    return PSF_OK;
}

// BiCGSTAB2 (CG.h:196-253)
static psf_status bicgstab2(Engine &E, const int *ip, const int *ix, const double *a, const double *b, double *x,
                            int itmax, double eps, int *iters, double *rrn, double *bbn, int *conv) {
    const int n = E.n;
    double *r, *rd, *p, *u, *tkm1, *w, *z, *Ap, *y, *tk, *At;
    for (double **q : {&r, &rd, &p, &u, &tkm1, &w, &z, &Ap, &y, &tk, &At})
        PSF_CHECK(E.alloc((void **)q, sizeof(double) * n));
    for (double *q : {p, u, tkm1, w, z, x}) PSF_CUDA(cudaMemsetAsync(q, 0, sizeof(double) * n, E.s));
    PSF_CHECK(E.spmv(ip, ix, a, x, Ap));
    PSF_CHECK(E.lin(r, 1.0, b, -1.0, Ap));
    PSF_CUDA(cudaMemcpyAsync(rd, r, sizeof(double) * n, cudaMemcpyDeviceToDevice, E.s));
    double h[4];
    PSF_CHECK(E.dot(2, h, rd, r, b, b));
    double rdr = h[0], beta = 0.0, rr = h[0];
    const double bnorm = sqrt(h[1]);
    *bbn = h[1];
    *conv = 0;
    int k = 0;
    for (; k < itmax; k++) {
        PSF_CHECK(E.lin(p, beta, p, 1.0, r, -beta, u));
        PSF_CHECK(E.spmv(ip, ix, a, p, Ap));
        PSF_CHECK(E.dot(1, h, rd, Ap));
        const double alpha = rdr / h[0];
        PSF_CHECK(E.lin(y, 1.0, tkm1, -1.0, r, -alpha, w, alpha, Ap));
        PSF_CHECK(E.lin(tk, 1.0, r, -alpha, Ap));
        PSF_CHECK(E.spmv(ip, ix, a, tk, At));
        double zeta, ita;
        if (k % 2 == 0) {
            PSF_CHECK(E.dot(2, h, At, tk, At, At));
            zeta = h[0] / h[1];
            ita = 0.0;
        } else {
            PSF_CHECK(E.dot(4, h, At, tk, At, At, y, y, y, tk));
            const double Att = h[0], AtAt = h[1], yy = h[2], yt = h[3];
            PSF_CHECK(E.dot(1, h, At, y));
            const double Aty = h[0];
            zeta = (yy * Att - yt * Aty) / (AtAt * yy - Aty * Aty);
            ita = (AtAt * yt - Aty * Att) / (AtAt * yy - Aty * Aty);
        }
        (comb_wxyz<<<E.grid(), kThreads, 0, E.s>>>(n, zeta, Ap, ita, tkm1, r, beta, u), note_launch());
        PSF_CUDA(cudaGetLastError());
        PSF_CHECK(E.lin(z, ita, z, zeta, r, -alpha, u));
        PSF_CHECK(E.lin(x, 1.0, x, alpha, p, 1.0, z));
        PSF_CHECK(E.lin(r, 1.0, tk, -ita, y, -zeta, At));
        PSF_CHECK(E.dot(2, h, rd, r, r, r));
        beta = alpha * h[0] / (zeta * rdr);
        PSF_CHECK(E.lin(w, 1.0, At, beta, Ap));
        rdr = h[0];
        rr = h[1];
        PSF_CUDA(cudaMemcpyAsync(tkm1, tk, sizeof(double) * n, cudaMemcpyDeviceToDevice, E.s));
        if (!std::isfinite(rr)) { k++; break; }
        if (sqrt(rr) < eps * bnorm) { k++; *conv = 1; break; }
    }
    *iters = k;
    *rrn = rr;
    return PSF_OK;
}

// ILU0CG (CG.h:319-352)
static psf_status ilu0_cg(Engine &E, const int *ip, const int *ix, const double *a, const Ilu &F, const double *b,
                          double *x, int itmax, double eps, int *iters, double *rrn, double *bbn, int *conv) {
    const int n = E.n;
    double *r, *p, *Mr, *Ap;
    for (double **q : {&r, &p, &Mr, &Ap}) PSF_CHECK(E.alloc((void **)q, sizeof(double) * n));
    PSF_CUDA(cudaMemsetAsync(x, 0, sizeof(double) * n, E.s));
    PSF_CHECK(E.spmv(ip, ix, a, x, Ap));
    PSF_CHECK(E.lin(r, 1.0, b, -1.0, Ap));
    PSF_CHECK(ilu_apply(E, F, ip, ix, r, p));
    PSF_CUDA(cudaMemcpyAsync(Mr, p, sizeof(double) * n, cudaMemcpyDeviceToDevice, E.s));
    double h[4];
    PSF_CHECK(E.dot(2, h, b, b, Mr, r));
    const double bnorm = sqrt(h[0]);
    *bbn = h[0];
    double Mrr = h[1], rr = 0.0;
    *conv = 0;
    int k = 0;
    for (; k < itmax; k++) {
        PSF_CHECK(E.spmv(ip, ix, a, p, Ap));
        PSF_CHECK(E.dot(1, h, p, Ap));
        const double alpha = Mrr / h[0];
        PSF_CHECK(E.lin(x, 1.0, x, alpha, p));     // xexpay (CG.h:31-38)
        PSF_CHECK(E.lin(r, 1.0, r, -alpha, Ap));
        PSF_CHECK(ilu_apply(E, F, ip, ix, r, Mr));
        PSF_CHECK(E.dot(2, h, Mr, r, r, r));
        const double beta = h[0] / Mrr;
        PSF_CHECK(E.lin(p, beta, p, 1.0, Mr));     // xeaxpy (CG.h:42-49)
        Mrr = h[0];
        rr = h[1];
        if (!std::isfinite(rr)) { k++; break; }
        if (sqrt(rr) < eps * bnorm) { k++; *conv = 1; break; }
    }
    *iters = k;
    *rrn = rr;
    return PSF_OK;
}

}  // namespace kry

// the solvers of this file on device CSR arrays (h_ip / h_ix: the same pattern on the host,
// for the level sets); m_given: an ILU(0) factor on the pattern (NULL = factor A here)
psf_status krylov_csr_solve(Ctx *c, int solver, int n, long long nnz, const int *h_ip, const int *h_ix, const int *ip,
                            const int *ix, const double *a, const double *m_given, const double *b, double *x,
                            int itmax, double eps, int *iters, double *rr, double *bb, int *conv) {
    kry::Engine E;
    E.s = c->stream;
    E.n = n;
    PSF_CHECK(E.alloc((void **)&E.part, sizeof(double) * 4 * kry::kBlocks));
    PSF_CHECK(E.alloc((void **)&E.res, sizeof(double) * 4));
    if (solver == PSF_SOLVE_CSR_BICGSTAB2_F64) return kry::bicgstab2(E, ip, ix, a, b, x, itmax, eps, iters, rr, bb, conv);
    if (solver == PSF_SOLVE_CSR_SCALING_BICGSTAB_F64) {
        double *D;
        PSF_CHECK(E.alloc((void **)&D, sizeof(double) * n));
        (kry::diag_of<<<E.grid(), kry::kThreads, 0, E.s>>>(n, ip, ix, a, D), note_launch());
        PSF_CUDA(cudaGetLastError());
        return kry::precond_bicgstab(E, ip, ix, a, b, x, false, D, nullptr, itmax, eps, iters, rr, bb, conv);
    }
    kry::Ilu F;
    PSF_CHECK(kry::ilu_setup(E, n, h_ip, h_ix, ip, ix, a, m_given, nnz, &F));
    if (solver == PSF_SOLVE_CSR_ILU0_CG_F64) return kry::ilu0_cg(E, ip, ix, a, F, b, x, itmax, eps, iters, rr, bb, conv);
    if (solver == PSF_SOLVE_CSR_ILU0_BICGSTAB_F64)
        return kry::precond_bicgstab(E, ip, ix, a, b, x, true, nullptr, &F, itmax, eps, iters, rr, bb, conv);
    set_error("krylov_csr_solve: unknown solver");
    return PSF_BAD_INPUT;
}

// ILU0 alone (the factor's values) and PreILU0 alone, on device arrays
psf_status krylov_ilu0(Ctx *c, int n, long long nnz, const int *h_ip, const int *h_ix, const int *ip, const int *ix,
                       const double *a, const double *m_given, const double *b, double *m_out, double *v_out) {
    kry::Engine E;
    E.s = c->stream;
    E.n = n;
    kry::Ilu F;
    PSF_CHECK(kry::ilu_setup(E, n, h_ip, h_ix, ip, ix, a, m_given, nnz, &F));
    if (m_out) PSF_CUDA(cudaMemcpyAsync(m_out, F.m, sizeof(double) * nnz, cudaMemcpyDeviceToDevice, E.s));
    if (b && v_out) PSF_CHECK(kry::ilu_apply(E, F, ip, ix, b, v_out));
    PSF_CUDA(cudaStreamSynchronize(E.s));
    return PSF_OK;
}

}  // namespace psf
