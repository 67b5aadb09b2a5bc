// psf_noalloc.cu -- ScalingCG on a device-resident CSR matrix without any
// device allocation (psf_csr_solve_noalloc).
//
// Some callers of this library cannot allocate device memory at the point
// where they need a solve: a host that hands the whole device heap to its own
// pool allocator before any solver runs, a real-time or embedded loop that
// forbids allocation (and the synchronisation cudaMalloc/cudaFree can imply)
// after start-up, or a host whose allocator belongs to another framework and
// must not be bypassed.  For them this entry point takes inputs and outputs
// already in device memory and keeps its scratch (Krylov vectors, diagonal
// positions, reduction slots) in one fixed file-scope device array,
// g_noalloc_scratch, sized for kNoallocMaxRows rows.  The array is part of the
// loaded module: every GPU that loads the library holds its ~11.6 MB until the
// process exits.
#include <mutex>

#include "psf_internal.cuh"

namespace psf {

psf_status pcg_csr_launch_raw(cudaStream_t s, long long rows, const int *indptr, const int *indices, const int *diag,
                              const double *data, const double *b, double *x, double *w, int itmax, double eps,
                              GridSync *gs, double *partials, int max_blocks, double *out);   // psf_solve.cu

constexpr long long kNoallocMaxRows = 262144;   // PSF_NOALLOC_MAX_ROWS
constexpr int kNoallocMaxBlocks = 1024;

// scratch layout (bytes, each part 256-byte aligned)
constexpr size_t kOffW = 0;                                                        // 5 * rows doubles
constexpr size_t kOffDiag = kOffW + 5 * kNoallocMaxRows * sizeof(double);          // rows ints
constexpr size_t kOffPart = kOffDiag + kNoallocMaxRows * sizeof(int);              // partial sums
constexpr size_t kOffSync = kOffPart + (size_t)(kMaxRed + 2) * kNoallocMaxBlocks * sizeof(double);
constexpr size_t kOffOut = kOffSync + 256;                                         // 8 doubles
constexpr size_t kScratchBytes = kOffOut + 256;
static_assert(sizeof(GridSync) <= 256, "grid sync slot exceeds its scratch part");
static_assert(kOffDiag % 256 == 0 && kOffPart % 256 == 0 && kOffSync % 256 == 0, "scratch parts misaligned");

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

namespace {
// position of (i, i) in row i, -1 when absent (the reference's get(i, i) returns 0 there)
__global__ void noalloc_diag(int n, const int *indptr, const int *indices, int *diag) {
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
}  // namespace

// Device address of the scratch array on the current device.  The array's name
// in host code is only a host-side stand-in, so the address is looked up once
// per device with that device current and cached.
static psf_status scratch_address(unsigned char **out) {
    static std::mutex mu;
    static unsigned char *addr[64] = {nullptr};
    int dev = 0;
    PSF_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) { set_error("psf_csr_solve_noalloc: device index out of range"); return PSF_BAD_INPUT; }
    std::lock_guard<std::mutex> lk(mu);
    if (!addr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return cuda_status(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
        addr[dev] = (unsigned char *)p;
    }
    *out = addr[dev];
    return PSF_OK;
}

}  // namespace psf

using namespace psf;

extern "C" psf_status psf_csr_solve_noalloc(int n, const int32_t *d_indptr, const int32_t *d_indices,
                                            const double *d_data, const double *d_b, double *d_x, int itmax,
                                            double eps, void *stream, psf_solve_info *info) {
    if (n < 1 || n > kNoallocMaxRows) {
        set_error("psf_csr_solve_noalloc: n must be in [1, " + std::to_string(kNoallocMaxRows) +
                  "] (the fixed scratch array holds that many rows)");
        return PSF_BAD_INPUT;
    }
    if (!d_indptr || !d_indices || !d_data || !d_b || !d_x) {
        set_error("psf_csr_solve_noalloc: null device pointer");
        return PSF_BAD_INPUT;
    }
    if (itmax < 1 || !(eps > 0)) { set_error("psf_csr_solve_noalloc: itmax >= 1 and eps > 0 required"); return PSF_BAD_INPUT; }
    unsigned char *base = nullptr;
    PSF_CHECK(scratch_address(&base));
    cudaStream_t s = (cudaStream_t)stream;
    double *w = (double *)(base + kOffW);
    int *diag = (int *)(base + kOffDiag);
    double *partials = (double *)(base + kOffPart);
    GridSync *gs = (GridSync *)(base + kOffSync);
    double *out = (double *)(base + kOffOut);
    (noalloc_diag<<<grid_for(n, 256, 4096), 256, 0, s>>>(n, d_indptr, d_indices, diag), ::psf::note_launch());
    PSF_CUDA(cudaGetLastError());
    PSF_CHECK(pcg_csr_launch_raw(s, n, d_indptr, d_indices, diag, d_data, d_b, d_x, w, itmax, eps, gs, partials,
                                 kNoallocMaxBlocks, out));
    double h[4] = {0, 0, 0, 0};
    int st = 0;
    PSF_CUDA(cudaMemcpyAsync(h, out, sizeof h, cudaMemcpyDeviceToHost, s));
    PSF_CUDA(cudaMemcpyAsync(&st, &gs->status, sizeof(int), cudaMemcpyDeviceToHost, s));
    PSF_CUDA(cudaStreamSynchronize(s));
    if (st != 0) { set_error("device-side grid barrier wait exceeded its limit"); return (psf_status)st; }
    if (info) {
        psf_solve_info inf{};
        inf.iterations = (int)h[0];
        inf.outer_iterations = 1;
        inf.rel_residual_recurrence = h[2] > 0 ? sqrt(h[1] / h[2]) : 0.0;
        inf.rel_residual = -1.0;   // not computed on this path
        *info = inf;
    }
    return h[3] != 0.0 ? PSF_OK : PSF_NOT_CONVERGED;
}
