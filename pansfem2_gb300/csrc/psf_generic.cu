// psf_generic.cu -- entry points on the reference's general data structures:
// an arbitrary CSR matrix (CSR<T> of CSR.h) and explicit neighbour lists
// (DensityFilter of DensityFilter.h).  They run on a process-wide internal
// context (stream, grid-sync slot) created on first use on the current device.
#include <cmath>
#include <mutex>

#include "psf_internal.cuh"

namespace psf {
psf_status pcg_csr_any(Ctx *c, long long rows, const int *indptr, const int *indices, const int *diag,
                       const double *data, const double *b, double *x, double *w, int jacobi, int itmax, double eps,
                       int *iters, double *rr, double *bb, int *conv);  // psf_solve.cu
psf_status krylov_csr_solve(Ctx *c, int solver, int n, long long nnz, const int *h_ip, const int *h_ix, const int *ip,
                            const int *ix, const double *a, const double *m_given, const double *b, double *x,
                            int itmax, double eps, int *iters, double *rr, double *bb, int *conv);   // psf_krylov.cu
psf_status krylov_ilu0(Ctx *c, int n, long long nnz, const int *h_ip, const int *h_ix, const int *ip, const int *ix,
                       const double *a, const double *m_given, const double *b, double *m_out, double *v_out);

namespace {
// position of (i, i) in row i (binary search over the sorted columns), -1 when absent
__global__ void diag_positions(int n, const int *indptr, const int *indices, int *diag) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        int lo = indptr[i], hi = indptr[i + 1];
        while (lo < hi) {
            const int mid = lo + (hi - lo) / 2;
            if (indices[mid] < i) lo = mid + 1;
            else hi = mid;
        }
        diag[i] = (lo < indptr[i + 1] && indices[lo] == i) ? lo : -1;
    }
}

// CSR::operator*: each row summed in column order (one thread per row)
__global__ void spmv_rows(int n, const int *indptr, const int *indices, const double *data, const double *x, double *y) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double v = 0.0;
        for (int q = indptr[i]; q < indptr[i + 1]; q++) v += data[q] * x[indices[q]];
        y[i] = v;
    }
}

__global__ void list_filter_kernel(int n, const int *ptr, const int *idx, const double *w, const double *in, double *out) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double acc = 0.0, ws = 0.0;
        for (int k = ptr[i]; k < ptr[i + 1]; k++) {
            acc += w[k] * in[idx[k]];
            ws += w[k];
        }
        out[i] = acc / ws;
    }
}
}  // namespace

static std::mutex g_mu;
static psf_ctx *g_ctx = nullptr;
static int g_dev = -1;

static psf_status generic_ctx(Ctx **out) {
    int dev = 0;
    PSF_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_ctx || g_dev != dev) {
        psf_ctx *h = nullptr;
        PSF_CHECK(psf_create(&h, PSF_Q4_HEAT, 1, 1, 0, 1.0, 1.0, 0.0, 0.3, 1.0));
        g_ctx = h;
        g_dev = dev;
    }
    *out = &g_ctx->c;
    return PSF_OK;
}

// the same internal context for other translation units (explicit meshes, psf_fem.cu)
psf_status generic_context(Ctx **out) { return generic_ctx(out); }

static bool csr_ok(int n, const int32_t *indptr, const int32_t *indices, const double *data) {
    if (n < 0 || !indptr || (n > 0 && (!indices || !data))) return false;
    if (indptr[0] != 0) return false;
    for (int i = 0; i < n; i++)
        if (indptr[i + 1] < indptr[i]) return false;
    for (long long q = 0; q < indptr[n]; q++)
        if (indices[q] < 0 || indices[q] >= n) return false;
    return true;
}

}  // namespace psf

using namespace psf;

extern "C" {

psf_status psf_csr_spmv(int n, const int32_t *indptr, const int32_t *indices, const double *data, const double *x,
                        double *y) {
    if (!csr_ok(n, indptr, indices, data) || !x || !y) { set_error("psf_csr_spmv: invalid CSR arrays"); return PSF_BAD_INPUT; }
    Ctx *c;
    PSF_CHECK(generic_ctx(&c));
    const long long nnz = indptr[n];
    int *dp = nullptr, *di = nullptr;
    double *dd = nullptr, *dx = nullptr, *dy = nullptr;
    cudaStream_t s = c->stream;
    PSF_CUDA(cudaMallocAsync((void **)&dp, sizeof(int) * (n + 1), s));
    PSF_CUDA(cudaMallocAsync((void **)&di, sizeof(int) * (nnz + 1), s));
    PSF_CUDA(cudaMallocAsync((void **)&dd, sizeof(double) * (nnz + 1), s));
    PSF_CUDA(cudaMallocAsync((void **)&dx, sizeof(double) * (n + 1), s));
    PSF_CUDA(cudaMallocAsync((void **)&dy, sizeof(double) * (n + 1), s));
    PSF_CUDA(cudaMemcpyAsync(dp, indptr, sizeof(int) * (n + 1), cudaMemcpyHostToDevice, s));
    PSF_CUDA(cudaMemcpyAsync(di, indices, sizeof(int) * nnz, cudaMemcpyHostToDevice, s));
    PSF_CUDA(cudaMemcpyAsync(dd, data, sizeof(double) * nnz, cudaMemcpyHostToDevice, s));
    PSF_CUDA(cudaMemcpyAsync(dx, x, sizeof(double) * n, cudaMemcpyHostToDevice, s));
    (spmv_rows<<<grid_for(n, 256, 65536), 256, 0, s>>>(n, dp, di, dd, dx, dy), ::psf::note_launch());
    PSF_CUDA(cudaGetLastError());
    PSF_CUDA(cudaMemcpyAsync(y, dy, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
    for (void *p : {(void *)dp, (void *)di, (void *)dd, (void *)dx, (void *)dy}) PSF_CUDA(cudaFreeAsync(p, s));
    PSF_CUDA(cudaStreamSynchronize(s));
    return PSF_OK;
}

static bool krylov_solver(int solver) {
    return solver == PSF_SOLVE_CSR_SCALING_BICGSTAB_F64 || solver == PSF_SOLVE_CSR_BICGSTAB2_F64 ||
           solver == PSF_SOLVE_CSR_ILU0_CG_F64 || solver == PSF_SOLVE_CSR_ILU0_BICGSTAB_F64;
}

// the solvers of psf_krylov.cu on host CSR arrays (m: a given ILU(0) factor or NULL)
static psf_status krylov_host(int n, const int32_t *indptr, const int32_t *indices, const double *data,
                              const double *m, const double *b, int solver, int itmax, double eps, double *x,
                              psf_solve_info *info) {
    Ctx *c;
    PSF_CHECK(generic_ctx(&c));
    const long long nnz = indptr[n];
    int *dp = nullptr, *di = nullptr;
    double *dd = nullptr, *dm = nullptr, *db = nullptr, *dx = nullptr;
    cudaStream_t s = c->stream;
    PSF_CUDA(cudaMallocAsync((void **)&dp, sizeof(int) * (n + 1), s));
    PSF_CUDA(cudaMallocAsync((void **)&di, sizeof(int) * (nnz + 1), s));
    PSF_CUDA(cudaMallocAsync((void **)&dd, sizeof(double) * (nnz + 1), s));
    PSF_CUDA(cudaMallocAsync((void **)&dm, sizeof(double) * (nnz + 1), s));
    PSF_CUDA(cudaMallocAsync((void **)&db, sizeof(double) * (n + 1), s));
    PSF_CUDA(cudaMallocAsync((void **)&dx, sizeof(double) * (n + 1), s));
    PSF_CUDA(cudaMemcpyAsync(dp, indptr, sizeof(int) * (n + 1), cudaMemcpyHostToDevice, s));
    PSF_CUDA(cudaMemcpyAsync(di, indices, sizeof(int) * nnz, cudaMemcpyHostToDevice, s));
    PSF_CUDA(cudaMemcpyAsync(dd, data, sizeof(double) * nnz, cudaMemcpyHostToDevice, s));
    if (m) PSF_CUDA(cudaMemcpyAsync(dm, m, sizeof(double) * nnz, cudaMemcpyHostToDevice, s));
    PSF_CUDA(cudaMemcpyAsync(db, b, sizeof(double) * n, cudaMemcpyHostToDevice, s));
    int it = 0, conv = 0;
    double rr = 0, bb = 0;
    psf_status st = krylov_csr_solve(c, solver, n, nnz, indptr, indices, dp, di, dd, m ? dm : nullptr, db, dx, itmax,
                                     eps, &it, &rr, &bb, &conv);
    if (st == PSF_OK) st = cuda_status(cudaMemcpyAsync(x, dx, sizeof(double) * n, cudaMemcpyDeviceToHost, s), "copy");
    for (void *p : {(void *)dp, (void *)di, (void *)dd, (void *)dm, (void *)db, (void *)dx}) cudaFreeAsync(p, s);
    PSF_CUDA(cudaStreamSynchronize(s));
    if (st != PSF_OK) return st;
    if (!std::isfinite(rr) || !std::isfinite(bb)) {
        set_error("non-finite residual (non-finite matrix or right-hand side entries)");
        return PSF_NOT_FINITE;
    }
    if (info) {
        psf_solve_info inf{};
        inf.iterations = it;
        inf.outer_iterations = 1;
        inf.rel_residual_recurrence = bb > 0 ? sqrt(rr / bb) : 0.0;
        inf.rel_residual = -1.0;   // not computed on this path
        *info = inf;
    }
    return conv ? PSF_OK : PSF_NOT_CONVERGED;
}

psf_status psf_csr_solve(int n, const int32_t *indptr, const int32_t *indices, const double *data, const double *b,
                         int solver, int itmax, double eps, double *x, psf_solve_info *info) {
    if (!csr_ok(n, indptr, indices, data) || !b || !x) { set_error("psf_csr_solve: invalid CSR arrays"); return PSF_BAD_INPUT; }
    if (itmax < 1 || !(eps > 0)) { set_error("psf_csr_solve: itmax >= 1 and eps > 0 required"); return PSF_BAD_INPUT; }
    if (krylov_solver(solver)) return krylov_host(n, indptr, indices, data, nullptr, b, solver, itmax, eps, x, info);
    if (solver != PSF_SOLVE_CSR_JACOBI_F64 && solver != PSF_SOLVE_CSR_CG_F64 && solver != PSF_SOLVE_CSR_BICGSTAB_F64) {
        set_error("psf_csr_solve: solver must be one of the PSF_SOLVE_CSR_* kinds");
        return PSF_BAD_INPUT;
    }
    if (itmax < 1 || !(eps > 0)) { set_error("psf_csr_solve: itmax >= 1 and eps > 0 required"); return PSF_BAD_INPUT; }
    Ctx *c;
    PSF_CHECK(generic_ctx(&c));
    const long long nnz = indptr[n];
    int *dp = nullptr, *di = nullptr, *dg = nullptr;
    double *dd = nullptr, *db = nullptr, *dx = nullptr, *w = nullptr;
    cudaStream_t s = c->stream;
    PSF_CUDA(cudaMallocAsync((void **)&dp, sizeof(int) * (n + 1), s));
    PSF_CUDA(cudaMallocAsync((void **)&di, sizeof(int) * (nnz + 1), s));
    PSF_CUDA(cudaMallocAsync((void **)&dg, sizeof(int) * (n + 1), s));
    PSF_CUDA(cudaMallocAsync((void **)&dd, sizeof(double) * (nnz + 1), s));
    PSF_CUDA(cudaMallocAsync((void **)&db, sizeof(double) * (n + 1), s));
    PSF_CUDA(cudaMallocAsync((void **)&dx, sizeof(double) * (n + 1), s));
    PSF_CUDA(cudaMallocAsync((void **)&w, sizeof(double) * 7 * (n + 1), s));
    PSF_CUDA(cudaMemcpyAsync(dp, indptr, sizeof(int) * (n + 1), cudaMemcpyHostToDevice, s));
    PSF_CUDA(cudaMemcpyAsync(di, indices, sizeof(int) * nnz, cudaMemcpyHostToDevice, s));
    PSF_CUDA(cudaMemcpyAsync(dd, data, sizeof(double) * nnz, cudaMemcpyHostToDevice, s));
    PSF_CUDA(cudaMemcpyAsync(db, b, sizeof(double) * n, cudaMemcpyHostToDevice, s));
    (diag_positions<<<grid_for(n, 256, 65536), 256, 0, s>>>(n, dp, di, dg), ::psf::note_launch());
    PSF_CUDA(cudaGetLastError());
    c->ksec = 0.0;
    c->klaunch = 0;
    int it = 0, conv = 0;
    double rr = 0, bb = 0;
    psf_status st;
    if (solver == PSF_SOLVE_CSR_BICGSTAB_F64) {
        double *const v[6] = {w, w + (n + 1), w + 2 * (n + 1), w + 3 * (n + 1), w + 4 * (n + 1), w + 5 * (n + 1)};
        st = bicgstab_csr_any(c, n, dp, di, dd, db, dx, v, itmax, eps, &it, &rr, &bb, &conv);
    } else {
        st = pcg_csr_any(c, n, dp, di, dg, dd, db, dx, w, solver == PSF_SOLVE_CSR_JACOBI_F64 ? 1 : 0, itmax, eps, &it,
                         &rr, &bb, &conv);
    }
    if (st == PSF_OK) {
        PSF_CUDA(cudaMemcpyAsync(x, dx, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
    }
    for (void *p : {(void *)dp, (void *)di, (void *)dg, (void *)dd, (void *)db, (void *)dx, (void *)w})
        cudaFreeAsync(p, s);
    PSF_CUDA(cudaStreamSynchronize(s));
    if (st != PSF_OK) return st;
    if (info) {
        psf_solve_info inf{};
        inf.iterations = it;
        inf.outer_iterations = 1;
        inf.rel_residual_recurrence = bb > 0 ? sqrt(rr / bb) : 0.0;
        inf.rel_residual = -1.0;   // not computed on this path
        inf.kernel_seconds = c->ksec;
        inf.kernel_launches = c->klaunch;
        *info = inf;
    }
    return conv ? PSF_OK : PSF_NOT_CONVERGED;
}

psf_status psf_csr_solve_ilu0(int n, const int32_t *indptr, const int32_t *indices, const double *data,
                              const double *m, const double *b, int solver, int itmax, double eps, double *x,
                              psf_solve_info *info) {
    if (!csr_ok(n, indptr, indices, data) || !b || !x) {
        set_error("psf_csr_solve_ilu0: invalid CSR arrays");
        return PSF_BAD_INPUT;
    }
    if (solver != PSF_SOLVE_CSR_ILU0_CG_F64 && solver != PSF_SOLVE_CSR_ILU0_BICGSTAB_F64) {
        set_error("psf_csr_solve_ilu0: solver must be PSF_SOLVE_CSR_ILU0_CG_F64 or PSF_SOLVE_CSR_ILU0_BICGSTAB_F64");
        return PSF_BAD_INPUT;
    }
    if (itmax < 1 || !(eps > 0)) { set_error("psf_csr_solve_ilu0: itmax >= 1 and eps > 0 required"); return PSF_BAD_INPUT; }
    return krylov_host(n, indptr, indices, data, m, b, solver, itmax, eps, x, info);
}

psf_status psf_csr_ilu0(int n, const int32_t *indptr, const int32_t *indices, const double *data,
                        const double *m_in, const double *b, double *m_out, double *v_out) {
    if (!csr_ok(n, indptr, indices, data) || (!m_out && !(b && v_out))) {
        set_error("psf_csr_ilu0: invalid arrays");
        return PSF_BAD_INPUT;
    }
    Ctx *c;
    PSF_CHECK(generic_ctx(&c));
    const long long nnz = indptr[n];
    int *dp = nullptr, *di = nullptr;
    double *dd = nullptr, *dmi = nullptr, *dmo = nullptr, *db = nullptr, *dv = nullptr;
    cudaStream_t s = c->stream;
    PSF_CUDA(cudaMallocAsync((void **)&dp, sizeof(int) * (n + 1), s));
    PSF_CUDA(cudaMallocAsync((void **)&di, sizeof(int) * (nnz + 1), s));
    PSF_CUDA(cudaMallocAsync((void **)&dd, sizeof(double) * (nnz + 1), s));
    PSF_CUDA(cudaMallocAsync((void **)&dmi, sizeof(double) * (nnz + 1), s));
    PSF_CUDA(cudaMallocAsync((void **)&dmo, sizeof(double) * (nnz + 1), s));
    PSF_CUDA(cudaMallocAsync((void **)&db, sizeof(double) * (n + 1), s));
    PSF_CUDA(cudaMallocAsync((void **)&dv, sizeof(double) * (n + 1), s));
    PSF_CUDA(cudaMemcpyAsync(dp, indptr, sizeof(int) * (n + 1), cudaMemcpyHostToDevice, s));
    PSF_CUDA(cudaMemcpyAsync(di, indices, sizeof(int) * nnz, cudaMemcpyHostToDevice, s));
    PSF_CUDA(cudaMemcpyAsync(dd, data, sizeof(double) * nnz, cudaMemcpyHostToDevice, s));
    if (m_in) PSF_CUDA(cudaMemcpyAsync(dmi, m_in, sizeof(double) * nnz, cudaMemcpyHostToDevice, s));
    if (b) PSF_CUDA(cudaMemcpyAsync(db, b, sizeof(double) * n, cudaMemcpyHostToDevice, s));
    psf_status st = krylov_ilu0(c, n, nnz, indptr, indices, dp, di, dd, m_in ? dmi : nullptr, b ? db : nullptr, dmo,
                                (b && v_out) ? dv : nullptr);
    if (st == PSF_OK && m_out)
        st = cuda_status(cudaMemcpyAsync(m_out, dmo, sizeof(double) * nnz, cudaMemcpyDeviceToHost, s), "copy");
    if (st == PSF_OK && b && v_out)
        st = cuda_status(cudaMemcpyAsync(v_out, dv, sizeof(double) * n, cudaMemcpyDeviceToHost, s), "copy");
    for (void *p : {(void *)dp, (void *)di, (void *)dd, (void *)dmi, (void *)dmo, (void *)db, (void *)dv})
        cudaFreeAsync(p, s);
    PSF_CUDA(cudaStreamSynchronize(s));
    return st;
}

psf_status psf_list_filter(int n, const int32_t *ptr, const int32_t *idx, const double *w, const double *in,
                           double *out) {
    if (n < 0 || !ptr || !in || !out || (n > 0 && ptr[n] > 0 && (!idx || !w))) {
        set_error("psf_list_filter: invalid arrays");
        return PSF_BAD_INPUT;
    }
    for (int i = 0; i < n; i++)
        if (ptr[i + 1] < ptr[i]) { set_error("psf_list_filter: ptr not monotone"); return PSF_BAD_INPUT; }
    const long long m = ptr[n];
    for (long long k = 0; k < m; k++)
        if (idx[k] < 0 || idx[k] >= n) { set_error("psf_list_filter: neighbour index out of range"); return PSF_BAD_INPUT; }
    Ctx *c;
    PSF_CHECK(generic_ctx(&c));
    cudaStream_t s = c->stream;
    int *dp = nullptr, *di = nullptr;
    double *dw = nullptr, *dinp = nullptr, *dout = nullptr;
    PSF_CUDA(cudaMallocAsync((void **)&dp, sizeof(int) * (n + 1), s));
    PSF_CUDA(cudaMallocAsync((void **)&di, sizeof(int) * (m + 1), s));
    PSF_CUDA(cudaMallocAsync((void **)&dw, sizeof(double) * (m + 1), s));
    PSF_CUDA(cudaMallocAsync((void **)&dinp, sizeof(double) * (n + 1), s));
    PSF_CUDA(cudaMallocAsync((void **)&dout, sizeof(double) * (n + 1), s));
    PSF_CUDA(cudaMemcpyAsync(dp, ptr, sizeof(int) * (n + 1), cudaMemcpyHostToDevice, s));
    PSF_CUDA(cudaMemcpyAsync(di, idx, sizeof(int) * m, cudaMemcpyHostToDevice, s));
    PSF_CUDA(cudaMemcpyAsync(dw, w, sizeof(double) * m, cudaMemcpyHostToDevice, s));
    PSF_CUDA(cudaMemcpyAsync(dinp, in, sizeof(double) * n, cudaMemcpyHostToDevice, s));
    (list_filter_kernel<<<grid_for(n, 256, 65536), 256, 0, s>>>(n, dp, di, dw, dinp, dout), ::psf::note_launch());
    PSF_CUDA(cudaGetLastError());
    PSF_CUDA(cudaMemcpyAsync(out, dout, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
    for (void *p : {(void *)dp, (void *)di, (void *)dw, (void *)dinp, (void *)dout}) PSF_CUDA(cudaFreeAsync(p, s));
    PSF_CUDA(cudaStreamSynchronize(s));
    return PSF_OK;
}

}  // extern "C"
