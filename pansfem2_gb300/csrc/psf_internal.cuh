// psf_internal.cuh -- the context and the launchers shared by the library's
// translation units.  Host code only sees psf_ctx through pansfem2_gpu.h.
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "psf_common.cuh"

namespace psf {

// Device-resident state of one structured-grid problem.  Layouts in HBM:
//   nodal vectors: node-major, dof-minor (node id (ny+1)*i + j, or
//                  ((ny+1)*i + j)*(nz+1) + k in 3D), nnodes*ndof entries,
//                  fixed dofs held at zero.  This is the order of the
//                  reference's global numbering, so reduced (free) vectors are
//                  the nodal vector with the fixed entries squeezed out.
//   element fields: element id ny*i + j (3D: (ny*i + j)*nz + k), ne entries.
//   CSR (free x free): int32 indptr/indices, FP64 values (FP32 copy for the
//                  mixed-precision path), the diagonal position per row.
// default launch shape of the CSR PCG kernel: lanes per row, threads per block, blocks per SM
// (the allocation-free entry point, which reads the CSR as it is); a context's solves default
// to one lane per row on the sliced copy of the CSR (kPcgSliced)
constexpr int kPcgDefaultLanes = 4, kPcgDefaultThreads = 1024, kPcgDefaultBlocksPerSm = 1;
constexpr int kPcgSliced = 1;

template <class T>
struct DevBuf {
    T *p = nullptr;
    size_t n = 0;
};

struct Ctx {
    int kind = 0, nx = 0, ny = 0, nz = 0;
    int nen = 4, ndof = 2, dim = 2;
    long long ne = 0, nnodes = 0, ndofs = 0;   // ndofs = nnodes*ndof
    long long nfree = 0, nnz = 0;
    double lx = 0, ly = 0, lz = 0, V = 0.3, t = 1.0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    cudaEvent_t evk0 = nullptr, evk1 = nullptr;   // around each Krylov kernel launch
    double ksec = 0.0;                            // accumulated Krylov kernel time of the current solve
    int klaunch = 0;

    // numbering
    int *n2g = nullptr;          // ndofs, -1 fixed
    int *g2n = nullptr;          // nfree -> nodal dof index
    unsigned char *fixed = nullptr;
    double *ufixed = nullptr;    // prescribed values (nodal)
    bool have_bc = false, nonzero_ufixed = false;
    std::vector<int> load_node, load_dof;
    std::vector<double> load_val;

    // element matrix of element 0 with E = 1 (Ke0) in FP64 and FP32
    double *Ke0 = nullptr;
    float *Ke0f = nullptr;
    std::vector<double> Ke0_host;

    // CSR
    int *indptr = nullptr, *indices = nullptr, *diag = nullptr;
    double *data = nullptr;
    bool have_csr = false, have_values = false;

    // right-hand side (reduced and nodal) and solution
    double *F = nullptr;         // nfree
    double *Fn = nullptr;        // nodal load vector (fixed entries zero)
    double *u = nullptr;         // nfree (reduced solution)
    double *un = nullptr;        // nodal solution
    double *E = nullptr;         // ne element moduli
    float *Ef = nullptr;         // FP32 copy
    double *Epad = nullptr;      // (nx+2)(ny+2)[(nz+2)] zero-padded moduli for the matrix-free kernels
    float *Epadf = nullptr;
    double *Dn = nullptr;        // nodal diagonal of K (1 on fixed dofs)
    float *Dnf = nullptr;
    float *Dl1f = nullptr;       // nodal l1 row sums sum_j |K_ij| (the multigrid smoother's diagonal)

    // Krylov work vectors (nodal length, FP64 and FP32)
    double *w64[8] = {nullptr};
    float *w32[8] = {nullptr};
    // grid sync + partials for the persistent kernels
    GridSync *gs = nullptr;
    double *partials = nullptr;
    int coop_blocks = 0;         // resident blocks for the persistent kernels
    // launch shapes (psf_set_launch_shape; the autotuner picks them per workload)
    int pcg_lanes = kPcgSliced, pcg_threads = kPcgDefaultThreads, pcg_blocks_per_sm = kPcgDefaultBlocksPerSm;
    // sliced copy of the CSR for the one-lane-per-row PCG (grown on demand, refilled per solve):
    // slices of 32 rows, slice s holds its rows' entries column-major from slot sell_ptr[s]
    int *sell_ptr = nullptr;     // slices + 1 slot offsets, then the slot total
    long long sell_ptr_cap = 0;
    int *sell_col = nullptr;
    double *sell_val = nullptr;
    long long sell_cap = 0;
    int opt_blocks_per_sm = 2;   // OC / MMA / CONLIN persistent kernels (256 threads)

    // filter (structured stencil)
    int filt_r = 0;              // stencil half width in elements
    int filt_n = 0;              // stencil entries
    int *filt_off = nullptr;     // offsets (di, dj, dk) x filt_n
    double *filt_w = nullptr;    // weights
    double *filt_wsum = nullptr; // per-element weight sum (in-bounds entries)
    double *filt_vw = nullptr;   // per-element volume weight sum over e in N(j) of w_ej / wsum_e (OC)
    double *oc_bp = nullptr;     // OC: x (-dfdx / dgdx)^iota per element
    double *oc_cs = nullptr;     // OC: two sets of canonical chunk sums
    double R = 0;

    // SIMP state
    double *s = nullptr, *rho = nullptr, *dfdrho = nullptr, *dgdrho = nullptr, *dfds = nullptr,
           *dgds = nullptr, *snew = nullptr;
    double *scal = nullptr;      // device scalars (f, g, ...), 16 doubles
    int heav = 0;                // Heaviside projection after the density filter
    double beta = 1.0;           // its current beta
    double *dH = nullptr, *tmp_ne = nullptr;   // d rho / d rho~ per element; scratch
    psf_simp_params prm{};
    bool simp_ready = false;
    double oc_prev = 0.0;
    int iter = 0;

    // MMA state (m = 1)
    double *mma_L = nullptr, *mma_U = nullptr, *mma_xkm1 = nullptr, *mma_xkm2 = nullptr;
    double *mma_work = nullptr;  // 21*ne scratch (MMA and CONLIN; the double-word kernel uses all of it)
    int opt_fp64_fallbacks = 0;  // double-word updates rerun in FP64 (data outside the FP32 pair range)
    int mma_k = 0;
    double mma_prev = 0.0, mma_epsvalue = 1e-5;
    double mma_a0 = 1, mma_a = 0, mma_c = 1e4, mma_d = 0, mma_xmin = 0.01, mma_xmax = 1.0;
    double mma_raa0 = 1e-5, mma_albefa = 0.1, mma_move = 0.5, mma_asyinit = 0.5, mma_asydecr = 0.7,
           mma_asyincr = 1.2;
    bool mma_ready = false;
    // CONLIN (CONLIN.h:17-52): parameters and outer state; work space shared with MMA (mma_work)
    double cl_a0 = 1, cl_a = 0, cl_c = 1e4, cl_d = 0, cl_xmin = 0.01, cl_xmax = 1.0, cl_move = 0.5;
    double cl_prev = 0.0, cl_epsvalue = 1e-5;
    int cl_k = 0;
    bool cl_ready = false;

    // multigrid hierarchy (mixed-precision preconditioner)
    void *mg = nullptr;
    // learned preconditioner
    void *learned = nullptr;
    // VTK export (pinned buffers, writer thread)
    void *vtk = nullptr;

    std::vector<void *> allocs;
};

// allocation tracked by the context (freed in psf_destroy)
template <class T>
psf_status dalloc(Ctx *c, T **p, size_t n) {
    void *q = nullptr;
    cudaError_t e = cudaMalloc(&q, (n ? n : 1) * sizeof(T));
    if (e != cudaSuccess) return cuda_status(e, "cudaMalloc");
    c->allocs.push_back(q);
    *p = (T *)q;
    return PSF_OK;
}
template <class T>
psf_status dzalloc(Ctx *c, T **p, size_t n) {
    PSF_CHECK(dalloc(c, p, n));
    cudaError_t e = cudaMemsetAsync(*p, 0, (n ? n : 1) * sizeof(T), c->stream);
    if (e != cudaSuccess) return cuda_status(e, "cudaMemsetAsync");
    return PSF_OK;
}

inline int grid_for(long long n, int block, int max_blocks = 1 << 20) {
    long long g = (n + block - 1) / block;
    if (g < 1) g = 1;
    if (g > max_blocks) g = max_blocks;
    return (int)g;
}

// launches a persistent kernel cooperatively over c->coop_blocks blocks
psf_status launch_coop(Ctx *c, const void *fn, int blocks, int threads, void **args, size_t smem = 0);
psf_status reset_sync(Ctx *c);
psf_status add_kernel_time(Ctx *c);   // accumulates evk0..evk1 into ksec / klaunch
psf_status read_sync_status(Ctx *c);

// ------------------------------------------------------------------ cross-file entry points
psf_status ke_element0(Ctx *c, double E, double *Ke_dev);       // psf_mesh.cu
psf_status build_pattern(Ctx *c);                               // psf_mesh.cu
psf_status assemble_values(Ctx *c, const double *E_dev);        // psf_mesh.cu
psf_status build_rhs(Ctx *c);                                   // psf_mesh.cu (nodal/reduced F with lift)
psf_status set_moduli(Ctx *c, const double *E_dev);             // psf_mesh.cu (E, Ef, Epad, diag)
psf_status spmv_csr64(Ctx *c, const double *x, double *y);      // psf_mesh.cu
psf_status ebe_apply64(Ctx *c, const double *xn, double *yn);   // psf_solve.cu (nodal)
psf_status ebe_apply32(Ctx *c, const float *xn, float *yn);     // psf_solve.cu (nodal)
psf_status scatter_reduced(Ctx *c, const double *red, double *nodal);  // psf_mesh.cu
psf_status gather_reduced(Ctx *c, const double *nodal, double *red);   // psf_mesh.cu
psf_status solve(Ctx *c, int solver, int itmax, double eps, bool warm, psf_solve_info *info);  // psf_solve.cu
psf_status filter_apply(Ctx *c, const double *in, double *out, bool backward);               // psf_opt.cu
psf_status heaviside_forward(Ctx *c, double beta, const double *s, double *rho);
psf_status generic_context(Ctx **out);   // psf_generic.cu: the process-wide internal context
psf_status fem_body_forces(cudaStream_t s, int kind, long long ne, int nen, const int *conn, const double *coords,
                           double fx, double fy, double t, double *Fe);   // psf_element.cu
psf_status fem_edge_forces(cudaStream_t s, int nedge, const int *edges, const double *coords, double tx, double ty,
                           double t, double *Fe);                          // psf_element.cu
psf_status fem_element_matrices(cudaStream_t s, int kind, long long ne, int nen, const int *conn, const double *coords,
                                const double *E, double V, double t, double *Ke);   // psf_element.cu
psf_status heaviside_back(Ctx *c, const double *d, double *out);                            // psf_opt.cu
psf_status sensitivity_filter(Ctx *c, const double *s, const double *d, int mode, double *out);  // psf_opt.cu
psf_status compliance_sens(Ctx *c, const double *rho, double E1, double E0, double p, double scale0,
                           double *f_dev, double *dfdrho);                                 // psf_opt.cu
psf_status oc_update(Ctx *c, double *x, const double *dfdx, const double *dgdx, double iota, double lmin,
                     double lmax, double leps, double move, double vf, double scale1, double *lambda);
psf_status mma_update(Ctx *c, double *x, double f, const double *dfdx, double g, const double *dgdx,
                      int *newton);
psf_status conlin_update(Ctx *c, double *x, double f, const double *dfdx, double g, const double *dgdx,
                         int *newton);
psf_status mma_dw_update(Ctx *c, bool conlin, double *x, const double *dfdx, double g, const double *dgdx,
                         int *newton, bool *capped, bool *done);
psf_status moduli_from_rho(Ctx *c, const double *rho, double E1, double E0, double p, double *E_dev);
psf_status mg_free(Ctx *c);
psf_status mg_precondition(Ctx *c, const double *r, double *z);   // psf_mg.cu
psf_status learned_free(Ctx *c);                                                       // psf_learned.cu
void vtk_free(Ctx *c);                                                                 // psf_vtk.cu
psf_status learned_solve(Ctx *c, int itmax, double eps, bool warm, psf_solve_info *info);  // psf_learned.cu
psf_status residual64_pub(Ctx *c, const double *b, const double *x, double *r, double *rnorm, double *bnorm);  // psf_solve.cu
psf_status diag_barrier_timeout(Ctx *c, int blocks, long long spin_limit);                                   // psf_solve.cu
psf_status bicgstab_csr_any(Ctx *c, long long rows, const int *indptr, const int *indices, const double *data,
                            const double *b, double *x, double *const v[6], int itmax, double eps, int *iters,
                            double *rr, double *bb, int *conv);                                           // psf_solve.cu

}  // namespace psf

struct psf_ctx {
    psf::Ctx c;
};
