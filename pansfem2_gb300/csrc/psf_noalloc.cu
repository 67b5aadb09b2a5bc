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
// positions, reduction slots, the validation flag) in one fixed file-scope
// device array, g_noalloc_scratch, sized for kNoallocMaxRows rows (~16.1 MB).
//
// The driver allocates that array, and the code of the kernels the solve
// launches, when it loads their modules.  With lazy module loading (the CUDA
// default) that happens at the first use on each device, so a call with n == 0
// exists to do it at start-up: it loads the modules of every kernel the solve
// launches and looks up the array's address, and allocates nothing afterwards.
// Every GPU that loads the modules holds the array until the process exits.
#include <cmath>
#include <string>

#include "psf_internal.cuh"

namespace psf {

psf_status pcg_csr_launch_raw(cudaStream_t s, long long rows, const int *indptr, const int *indices, const int *diag,
                              const double *data, const double *b, double *x, double *w, int itmax, double eps,
                              GridSync *gs, double *partials, int max_blocks, double *out);   // psf_solve.cu
psf_status pcg_csr_load_module();                                                             // psf_solve.cu

constexpr long long kNoallocMaxRows = 262144;   // PSF_NOALLOC_MAX_ROWS
constexpr int kNoallocMaxBlocks = 1024;

// scratch layout (bytes, each part 256-byte aligned)
constexpr size_t kOffW = 0;                                                        // 7 * rows doubles
constexpr size_t kOffDiag = kOffW + 7 * kNoallocMaxRows * sizeof(double);          // rows ints
constexpr size_t kOffPart = kOffDiag + kNoallocMaxRows * sizeof(int);              // partial sums
constexpr size_t kOffSync = kOffPart + (size_t)kPartialSlots * kNoallocMaxBlocks * sizeof(double);
constexpr size_t kOffOut = kOffSync + 256;   // out[0..3] solver results, [4..5] true residual sums
constexpr size_t kOffFlag = kOffOut + 128;   // CSR validation flag (int)
constexpr size_t kScratchBytes = kOffOut + 256;
static_assert(sizeof(GridSync) <= 256, "grid sync slot exceeds its scratch part");
static_assert(kOffDiag % 256 == 0 && kOffPart % 256 == 0 && kOffSync % 256 == 0, "scratch parts misaligned");
constexpr int kResBlocks = 512;   // blocks of the true-residual pass (partials fit the partials part)
static_assert(2 * kResBlocks <= kPartialSlots * kNoallocMaxBlocks, "residual partials exceed their part");

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

namespace {
// CSR checks on the flat arrays only (no address is formed from their contents):
// indptr[0] == 0, indptr non-decreasing, indptr[n] == nnz, every column index in [0, n).
// A violation sets *flag; the host reads it before any kernel indexes through indptr.
__global__ void noalloc_validate(int n, long long nnz, const int *indptr, const int *indices, int *flag) {
    const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long stride = (long long)gridDim.x * blockDim.x;
    int bad = 0;
    for (long long i = tid; i <= n; i += stride) {
        const int v = indptr[i];
        if (i == 0 && v != 0) bad = 1;
        if (i == n && (long long)v != nnz) bad = 1;
        if (i < n && indptr[i + 1] < v) bad = 1;
    }
    for (long long k = tid; k < nnz; k += stride) {
        const int c = indices[k];
        if (c < 0 || c >= n) bad = 1;
    }
    if (bad) atomicOr(flag, 1);
}

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

// FP64 true residual of the result: per-block partial sums of |b - A x|^2 and |b|^2 (rows summed
// in column order within a row, blocks in a fixed tree), then one warp adds the partials in order
__global__ void __launch_bounds__(256) noalloc_residual(int n, const int *indptr, const int *indices,
                                                        const double *data, const double *b, const double *x,
                                                        double *partials) {
    __shared__ double sm[32 * 2];
    double acc[2] = {0.0, 0.0};
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        double ax = 0.0;
        for (int k = indptr[i]; k < indptr[i + 1]; k++) ax += data[k] * x[indices[k]];
        const double r = b[i] - ax;
        acc[0] += r * r;
        acc[1] += b[i] * b[i];
    }
    block_sum<2>(acc, sm);
    if (threadIdx.x == 0) {
        partials[blockIdx.x] = acc[0];
        partials[gridDim.x + blockIdx.x] = acc[1];
    }
}
__global__ void noalloc_residual_finish(int nb, const double *partials, double *out) {
    const double rr = warp_canonical_sum(partials, nb);
    const double bb = warp_canonical_sum(partials + nb, nb);
    if (threadIdx.x == 0) {
        out[4] = rr;
        out[5] = bb;
    }
}
}  // namespace

// Device address of the scratch array on the current device.  The array's name in host code
// is only a host-side stand-in, so the address is looked up with the device current, on
// every call (cheap once the module is loaded; no cached pointer can outlive a context).
static psf_status scratch_address(unsigned char **out) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_status(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
    *out = (unsigned char *)p;
    return PSF_OK;
}

// Loads the modules of every kernel a solve launches (the driver allocates their code and
// static data, this array included, when it loads them) and looks up the array's address.
static psf_status noalloc_setup(unsigned char **base) {
    cudaFuncAttributes fa;
    PSF_CUDA(cudaFuncGetAttributes(&fa, noalloc_validate));
    PSF_CUDA(cudaFuncGetAttributes(&fa, noalloc_diag));
    PSF_CUDA(cudaFuncGetAttributes(&fa, noalloc_residual));
    PSF_CUDA(cudaFuncGetAttributes(&fa, noalloc_residual_finish));
    PSF_CHECK(pcg_csr_load_module());
    return scratch_address(base);
}

}  // namespace psf

using namespace psf;

extern "C" psf_status psf_csr_solve_noalloc(int n, int64_t nnz, const int32_t *d_indptr, const int32_t *d_indices,
                                            const double *d_data, const double *d_b, double *d_x, int itmax,
                                            double eps, void *stream, psf_solve_info *info) {
    if (n == 0) {   // set-up only (see the header)
        unsigned char *base = nullptr;
        return noalloc_setup(&base);
    }
    if (n < 1 || n > kNoallocMaxRows) {
        set_error("psf_csr_solve_noalloc: n must be in [1, " + std::to_string(kNoallocMaxRows) +
                  "] (the fixed scratch array holds that many rows)");
        return PSF_BAD_INPUT;
    }
    if (nnz < 0 || nnz > 0x7fffffffLL) { set_error("psf_csr_solve_noalloc: nnz must be in [0, 2^31)"); return PSF_BAD_INPUT; }
    if (!d_indptr || (nnz > 0 && (!d_indices || !d_data)) || !d_b || !d_x) {
        set_error("psf_csr_solve_noalloc: null device pointer");
        return PSF_BAD_INPUT;
    }
    if (itmax < 1 || !(eps > 0)) { set_error("psf_csr_solve_noalloc: itmax >= 1 and eps > 0 required"); return PSF_BAD_INPUT; }
    unsigned char *base = nullptr;
    PSF_CHECK(noalloc_setup(&base));
    cudaStream_t s = (cudaStream_t)stream;
    double *w = (double *)(base + kOffW);
    int *diag = (int *)(base + kOffDiag);
    double *partials = (double *)(base + kOffPart);
    GridSync *gs = (GridSync *)(base + kOffSync);
    double *out = (double *)(base + kOffOut);
    int *flag = (int *)(base + kOffFlag);
    // the matrix is checked before any kernel forms an address from indptr or indices
    int bad = 0;
    PSF_CUDA(cudaMemsetAsync(flag, 0, sizeof(int), s));
    (noalloc_validate<<<grid_for((long long)n + 1 > nnz ? (long long)n + 1 : nnz, 256, 4096), 256, 0, s>>>(
         n, (long long)nnz, d_indptr, d_indices, flag),
     ::psf::note_launch());
    PSF_CUDA(cudaGetLastError());
    PSF_CUDA(cudaMemcpyAsync(&bad, flag, sizeof(int), cudaMemcpyDeviceToHost, s));
    PSF_CUDA(cudaStreamSynchronize(s));
    if (bad) {
        set_error("psf_csr_solve_noalloc: malformed CSR (need indptr[0] == 0, non-decreasing indptr, "
                  "indptr[n] == nnz and column indices in [0, n))");
        return PSF_BAD_INPUT;
    }
    (noalloc_diag<<<grid_for(n, 256, 4096), 256, 0, s>>>(n, d_indptr, d_indices, diag), ::psf::note_launch());
    PSF_CUDA(cudaGetLastError());
    PSF_CHECK(pcg_csr_launch_raw(s, n, d_indptr, d_indices, diag, d_data, d_b, d_x, w, itmax, eps, gs, partials,
                                 kNoallocMaxBlocks, out));
    const int rb = grid_for(n, 256, kResBlocks);
    (noalloc_residual<<<rb, 256, 0, s>>>(n, d_indptr, d_indices, d_data, d_b, d_x, partials), ::psf::note_launch());
    (noalloc_residual_finish<<<1, 32, 0, s>>>(rb, partials, out), ::psf::note_launch());
    PSF_CUDA(cudaGetLastError());
    double h[6] = {0, 0, 0, 0, 0, 0};
    int st = 0;
    PSF_CUDA(cudaMemcpyAsync(h, out, sizeof h, cudaMemcpyDeviceToHost, s));
    PSF_CUDA(cudaMemcpyAsync(&st, &gs->status, sizeof(int), cudaMemcpyDeviceToHost, s));
    PSF_CUDA(cudaStreamSynchronize(s));
    if (st != 0) {
        set_error(st == PSF_TIMEOUT ? "device-side grid barrier wait exceeded its limit"
                                    : "zero or non-finite diagonal entry (the Jacobi scaling divides by it)");
        return (psf_status)st;
    }
    if (info) {
        psf_solve_info inf{};
        inf.iterations = (int)h[0];
        inf.outer_iterations = 1;
        inf.rel_residual_recurrence = h[2] > 0 ? sqrt(h[1] / h[2]) : 0.0;
        inf.rel_residual = h[5] > 0 ? sqrt(h[4] / h[5]) : 0.0;
        *info = inf;
    }
    if (!std::isfinite(h[1]) || !std::isfinite(h[2])) {
        set_error("non-finite residual (non-finite matrix or right-hand side entries)");
        return PSF_NOT_FINITE;
    }
    return h[3] != 0.0 ? PSF_OK : PSF_NOT_CONVERGED;
}
