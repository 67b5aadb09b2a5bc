// psf_generic.cu -- entry points on the reference's general data structures:
// an arbitrary CSR matrix (CSR<T> of CSR.h) and explicit neighbour lists
// (DensityFilter of DensityFilter.h).  They run on a process-wide internal
// context (stream, grid-sync slot) created on first use on the current device.
#include <mutex>

#include "psf_internal.cuh"

namespace psf {
psf_status pcg_csr_any(Ctx *c, long long rows, const int *indptr, const int *indices, const int *diag,
                       const double *data, const double *b, double *x, double *w, int jacobi, int itmax, double eps,
                       int *iters, double *rr, double *bb, int *conv);  // psf_solve.cu

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

psf_status psf_csr_solve(int n, const int32_t *indptr, const int32_t *indices, const double *data, const double *b,
                         int solver, int itmax, double eps, double *x, psf_solve_info *info) {
    if (!csr_ok(n, indptr, indices, data) || !b || !x) { set_error("psf_csr_solve: invalid CSR arrays"); return PSF_BAD_INPUT; }
    if (solver != PSF_SOLVE_CSR_JACOBI_F64 && solver != PSF_SOLVE_CSR_CG_F64 && solver != PSF_SOLVE_CSR_BICGSTAB_F64) {
        set_error("psf_csr_solve: solver must be PSF_SOLVE_CSR_JACOBI_F64, PSF_SOLVE_CSR_CG_F64 or "
                  "PSF_SOLVE_CSR_BICGSTAB_F64");
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
