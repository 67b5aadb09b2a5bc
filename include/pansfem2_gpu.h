/*
 * pansfem2_gpu.h -- C ABI of the GB300 (sm_103a) SIMP topology-optimisation library.
 *
 * The library replaces the hot path of PANSFEM2's density-based topology
 * optimisation (the sample drivers sample/optimize/sample_optimize_density_oc.cpp
 * and sample_optimize_density_mma.cpp) on structured Q4 / H8 grids.  Every
 * entry point takes plain pointers and sizes, returns a psf_status, and runs on
 * one GPU.  Host pointers are borrowed for the duration of the call (copied in
 * or out); device memory is owned by the context.  A context is not
 * thread-safe: one host thread drives it; its device work is ordered on the
 * context's stream.
 *
 * Citations name the PANSFEM2 routine each entry point replaces.
 */
#ifndef PANSFEM2_GPU_H
#define PANSFEM2_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    PSF_OK = 0,
    PSF_NOT_CONVERGED = 1,   /* solver hit its iteration cap; the last iterate is returned,
                                as CG.h:451-452 does after printing "Convergence:faild" */
    PSF_FELL_BACK = 2,       /* a preconditioner stalled and the solve finished with Jacobi PCG */
    PSF_BAD_INPUT = 3,       /* invalid argument, size or state */
    PSF_CUDA_ERROR = 4,      /* a CUDA runtime error (message via psf_last_error) */
    PSF_TIMEOUT = 5,         /* a device-side wait ran past its limit; the context stays usable */
    PSF_NOT_FINITE = 6       /* NaN/Inf in a scalar recurrence (e.g. pow of a negative base in OC) */
} psf_status;

typedef enum {
    PSF_Q4_PLANE_STRAIN = 0, /* PlaneStrainStiffness<ShapeFunction4Square, Gauss4Square> (PlaneStrain.h:20-58) */
    PSF_Q4_HEAT = 1,         /* HeatTransfer<ShapeFunction4Square, Gauss4Square> (HeatTransfer.h:19-43) */
    PSF_H8_SOLID = 2,        /* SolidLinearIsotropicElastic<ShapeFunction8Cubic, Gauss8Cubic> (Solid.h:20-64) */
    PSF_T3_PLANE_STRAIN = 3  /* PlaneStrainStiffness<ShapeFunction3Triangle, Gauss1Triangle> (explicit meshes only) */
} psf_element_kind;

typedef enum {
    PSF_SOLVE_CSR_JACOBI_F64 = 0, /* ScalingCG on the assembled CSR (CG.h:419-453), all FP64 */
    PSF_SOLVE_EBE_JACOBI_F64 = 1, /* same iteration, matrix-free element-by-element K.u, FP64 */
    PSF_SOLVE_IR_JACOBI_F32 = 2,  /* FP32 matrix-free Jacobi PCG inside FP64 iterative refinement */
    PSF_SOLVE_IR_MG_F32 = 3,      /* FP32 multigrid-preconditioned flexible CG inside FP64 refinement */
    PSF_SOLVE_CSR_CG_F64 = 4,     /* CG (CG.h:123-154) on the CSR */
    PSF_SOLVE_CSR_BICGSTAB_F64 = 5, /* BiCGSTAB (CG.h:158-193) on the CSR */
    PSF_SOLVE_IR_LEARNED_F32 = 6, /* FP32 FCG preconditioned by the learned grid U-Net inside FP64 refinement */
    PSF_SOLVE_CSR_SCALING_BICGSTAB_F64 = 7, /* ScalingBiCGSTAB (CG.h:457-495), psf_csr_solve */
    PSF_SOLVE_CSR_BICGSTAB2_F64 = 8,        /* BiCGSTAB2 (CG.h:196-253), psf_csr_solve */
    PSF_SOLVE_CSR_ILU0_CG_F64 = 9,          /* ILU0 + ILU0CG (CG.h:257-284, :319-352), psf_csr_solve(_ilu0) */
    PSF_SOLVE_CSR_ILU0_BICGSTAB_F64 = 10    /* ILU0 + ILU0BiCGSTAB (CG.h:356-391), psf_csr_solve(_ilu0) */
} psf_solver;

typedef struct psf_ctx psf_ctx;

typedef struct {
    int iterations;          /* Krylov iterations (inner iterations summed for IR) */
    int outer_iterations;    /* refinement steps (1 for the plain FP64 solvers) */
    int fell_back;           /* 1 if the solve fell back to Jacobi PCG */
    double rel_residual;     /* FP64 true residual ||b - K u|| / ||b|| of the returned u */
    double rel_residual_recurrence; /* the recurrence residual the stopping test used */
    double seconds;          /* device time of the solve (CUDA events) */
    double kernel_seconds;   /* device time inside the Krylov kernel launches alone */
    int kernel_launches;     /* Krylov kernel launches (persistent: one per (inner) solve) */
    int pad_;
} psf_solve_info;

/* ---------------- context / mesh ---------------- */
/* SquareMesh(lx, ly, nx, ny) nodes/elements (SquareMesh.h:61-106) or the H8
 * analogue (node ((ny+1)*i+j)*(nz+1)+k), material V (Poisson) and t
 * (thickness; unused for H8).  nz is ignored for the Q4 kinds. */
psf_status psf_create(psf_ctx **ctx, int kind, int nx, int ny, int nz, double lx, double ly,
                      double lz, double V, double t);
psf_status psf_destroy(psf_ctx *ctx);
const char *psf_last_error(void);
/* kernel launches this host thread has made through the library so far (graph replays count
 * their kernel nodes); the difference over a call sequence is its launch count */
psf_status psf_kernel_launches(long long *n);
/* Launch shape of a persistent kernel family of this context (no counterpart in the
 * reference; the autotuner pansfem2_gb300/autotune.py times candidates on the workload and
 * sets the fastest).  kernel = PSF_KERNEL_PCG_CSR: a = lanes per CSR row (4, 8, 16), or 1
 * for one lane per row on a sliced copy of the CSR that the context builds before each solve
 * (slices of 32 rows stored column by column, about 12 bytes per stored entry; the default),
 * b = threads per block (256, 512, 1024), c = blocks per SM (1-8).  kernel = PSF_KERNEL_OPT
 * (the OC / MMA / CONLIN kernels, 256 threads): c = blocks per SM (1-8), a and b ignored.
 * Blocks per SM are capped by what fits.  Results agree to rounding across shapes. */
#define PSF_KERNEL_PCG_CSR 0
#define PSF_KERNEL_OPT 1
psf_status psf_set_launch_shape(psf_ctx *ctx, int kernel, int a, int b, int c);
psf_status psf_get_launch_shape(const psf_ctx *ctx, int kernel, int *a, int *b, int *c);
/* Diagnostic of the bounded device waits (no counterpart in the reference): a cooperative
 * launch of `blocks` blocks in which the last block never arrives at a grid barrier (the
 * arrival is a flag nothing sets); the others poll at most spin_limit times (1 .. 2^23; the
 * solvers use 2^23, about a second), record PSF_TIMEOUT and return.  Returns the status the
 * host read back (PSF_TIMEOUT) and leaves the context usable.  Nothing faults or hangs. */
psf_status psf_diag_barrier_timeout(psf_ctx *ctx, int blocks, int64_t spin_limit);
/* sizes: elements, nodes, dofs per node, free dofs (after psf_set_dirichlet), CSR nnz (after psf_build_csr) */
psf_status psf_sizes(const psf_ctx *ctx, int64_t *ne, int64_t *nnodes, int *ndof, int64_t *nfree,
                     int64_t *nnz);

/* SetDirichlet + Renumbering (BoundaryCondition.h:19-25, Assembling.h:175-186):
 * marks (node, dof) pairs fixed with prescribed values (NULL = zeros) and numbers
 * the free dofs node-major / dof-minor on the device.  n2g_out (nnodes*ndof,
 * optional) receives the numbering with -1 for fixed dofs. */
psf_status psf_set_dirichlet(psf_ctx *ctx, int n, const int *node, const int *dof,
                             const double *value, int32_t *n2g_out);
/* Assembling(F, qfixed, nodetoglobal) (Assembling.h:151-158): point loads on free dofs. */
psf_status psf_set_loads(psf_ctx *ctx, int n, const int *node, const int *dof, const double *value);

/* Element matrix of element 0 for modulus E (conductivity for heat): the
 * reference element routine evaluated on the device in its operation order.
 * Ke_out is (nen*ndof)^2 row-major. */
psf_status psf_element_matrix(psf_ctx *ctx, double E, double *Ke_out);

/* LILCSR -> CSR (CSR.h:92-105) pattern on the device: every free-free dof pair
 * sharing an element, columns ascending.  indptr_out (nfree+1) / indices_out
 * (nnz) are optional host copies; call psf_sizes for nnz. */
psf_status psf_build_csr(psf_ctx *ctx, int32_t *indptr_out, int32_t *indices_out);

/* Assembling(LILCSR&, F, u, Ke, ...) (Assembling.h:46-66) for every element with
 * modulus E_e (ne values): CSR values summed in ascending element order plus the
 * Dirichlet lift into F, then the point loads.  data_out (nnz) and F_out (nfree)
 * are optional host copies. */
psf_status psf_assemble(psf_ctx *ctx, const double *E_e, double *data_out, double *F_out);

/* y = K x with the assembled CSR (CSR::operator*, CSR.h:108-122). Host vectors of length nfree. */
psf_status psf_spmv(psf_ctx *ctx, const double *x, double *y);
/* y = K x matrix-free (element-by-element with Ke(E=1) scaled by E_e), same K. */
psf_status psf_ebe_matvec(psf_ctx *ctx, const double *x, double *y);
/* z = M^-1 r with M^-1 one V(2,2)-cycle of the geometric multigrid that preconditions
 * PSF_SOLVE_IR_MG_F32 (no counterpart in the reference; the hierarchy is built for the
 * current moduli): z = |r| V(r / |r|) in FP32, returned in FP64.  Host vectors of length
 * nfree. */
psf_status psf_mg_precondition(psf_ctx *ctx, const double *r, double *z);

/* Solve K u = F for the current E_e / loads (ScalingCG signature: itmax, eps;
 * CG.h:420).  u_out (nfree) is the reduced solution, optional.  For the
 * refinement solvers eps is the FP64 true-residual target. */
psf_status psf_solve(psf_ctx *ctx, int solver, int itmax, double eps, double *u_out,
                     psf_solve_info *info);

/* ---------------- SIMP pieces ---------------- */
/* DensityFilter / HeavisideFilter neighbour lists (DensityFilter.h:16-30): the
 * lists of the samples (sample_optimize_density_oc.cpp:50-60), every element j
 * whose centroid lies within R, weight (R - d)/R, built on the device. */
psf_status psf_filter_setup(psf_ctx *ctx, double R);
/* GetFilteredVariables (DensityFilter.h:44-56): rho = W s / wsum; host arrays of ne. */
psf_status psf_filter_forward(psf_ctx *ctx, const double *s, double *rho);
/* GetFilteredSensitivitis (DensityFilter.h:59-71): dfds_i = sum_j w_ij dfdrho_j / wsum_i. */
psf_status psf_filter_backward(psf_ctx *ctx, const double *dfdrho, double *dfds);
/* SensitivityFilter::GetFilteredSensitivitis (Sigmund's scheme, SensitivityFilter.h:38-50) for
 * mode 0, SensitivityFilter2 (Borrvall's scheme, :78-90) for mode 1, on the filter of
 * psf_filter_setup: out_i = sum_j w_ij s_j d_j / (wsum_i s_i), resp. / sum_j w_ij s_j (host arrays) */
psf_status psf_sensitivity_filter(psf_ctx *ctx, int mode, const double *s, const double *dfds_in, double *dfds_out);

/* HeavisideFilter (HeavisideFilter.h:16-98) on the filter of psf_filter_setup, host arrays:
 * GetFilteredVariables: rho_i = H_beta(sum_j w_ij s_j / wsum_i) (HeavisideFilter.h:61-74);
 * GetFilteredSensitivitis: dfds_i = sum_j w_ij dfdrho_j H'_beta(rt_j) / wsum_i (:77-97),
 * with H_beta(r) = (tanh(beta/2) + tanh(beta (r - 1/2))) / (2 tanh(beta/2)).  beta is the
 * value UpdateBeta (:55-57) last set. */
psf_status psf_heaviside_forward(psf_ctx *ctx, double beta, const double *s, double *rho);
psf_status psf_heaviside_backward(psf_ctx *ctx, double beta, const double *s, const double *dfdrho,
                                  double *dfds);

/* Compliance and sensitivities of sample_optimize_density_oc.cpp:136-162 for the
 * solved u: f = scale0 * u.K u and dfdrho_e = -scale0*p*(E1 - E0)*rho_e^(p-1) u_e.Ke(1) u_e.
 * rho (ne) in, dfdrho (ne) out. */
psf_status psf_compliance_sensitivity(psf_ctx *ctx, const double *rho, double E1, double E0,
                                      double p, double scale0, double *f, double *dfdrho);

/* OC::UpdateVariables (OC.h:76-107) with the samples' volume callback
 * (filtered volume fraction vf, scale1): x (ne) updated in place. */
psf_status psf_oc_update(psf_ctx *ctx, double *x, const double *dfdx, const double *dgdx,
                         double iota, double lmin, double lmax, double leps, double move,
                         double vf, double scale1, double *lambda_out);

/* MMA (MMA.h:18-509) for m = 1 with state (asymptotes, history) kept on the device. */
psf_status psf_mma_init(psf_ctx *ctx, double a0, double a, double c, double d, double xmin,
                        double xmax, double raa0, double albefa, double move, double asyinit,
                        double asydecr, double asyincr, double epsvalue);
psf_status psf_mma_update(psf_ctx *ctx, double *x, double f, const double *dfdx, double g,
                          const double *dgdx, int *newton_steps);

/* MMA<T> (MMA.h:18-509) as a standalone object for any n and 1 <= m <= 4
 * constraints, with per-variable bounds: MMA(n, m, a0, a, c, d, xmin, xmax)
 * (MMA.h:64-90; a, c, d have m entries, xmin and xmax n), SetParameters (MMA.h:92-100),
 * UpdateVariables (MMA.h:116-419) on host arrays: x (n, in / out), dfdx (n), g (m), dgdx
 * (m x n, row i = constraint i).  The state (asymptotes, history) stays on the device.
 * n > m: the (m+1) Newton system, one persistent launch; n <= m: the (n+1) system, one
 * thread.  IsConvergence (MMA.h:107-113) is the caller's comparison of f values. */
typedef struct psf_mma psf_mma;
psf_status psf_mma_create(int n, int m, double a0, const double *a, const double *c, const double *d,
                          const double *xmin, const double *xmax, psf_mma **out);
psf_status psf_mma_set_parameters(psf_mma *mma, double raa0, double albefa, double move, double asyinit,
                                  double asydecr, double asyincr, double epsvalue);
psf_status psf_mma_update_host(psf_mma *mma, double *x, double f, const double *dfdx, const double *g,
                               const double *dgdx, int *newton_steps);
psf_status psf_mma_destroy(psf_mma *mma);

/* CONLIN (CONLIN.h:17-455) for m = 1: the constructor's a0, a, c, d, xmin, xmax
 * (CONLIN.h:55-67) and SetParameters(move, epsvalue) (CONLIN.h:71-74).  The
 * approximation has q_j / x_j terms, so 0 < xmin < xmax is required. */
psf_status psf_conlin_init(psf_ctx *ctx, double a0, double a, double c, double d, double xmin,
                           double xmax, double move, double epsvalue);
/* CONLIN::UpdateVariables (CONLIN.h:91-365): x (ne) updated in place; returns the
 * interior-point Newton steps. */
psf_status psf_conlin_update(psf_ctx *ctx, double *x, double f, const double *dfdx, double g,
                             const double *dgdx, int *newton_steps);

/* ---------------- the whole SIMP loop on the device ---------------- */
typedef struct {
    double E1, E0, p;        /* E = E1*rho^p + E0*(1 - rho^p) (sample law) */
    double vf, R, scale0, scale1, rho0;
    int optimizer;           /* 0 = OC, 1 = MMA, 2 = CONLIN (reads mma_a0, mma_c, mma_d, mma_xmin,
                                mma_xmax, mma_move, mma_eps) */
    double oc_iota, oc_lmin, oc_lmax, oc_leps, oc_move;
    double mma_raa0, mma_albefa, mma_move, mma_asyinit, mma_asydecr, mma_asyincr, mma_eps;
    double mma_a0, mma_c, mma_d, mma_xmin, mma_xmax;
    int solver;              /* psf_solver */
    int cg_itmax;
    double cg_eps;           /* recurrence (plain) or FP64 true-residual (refinement) target */
    int warm_start;          /* 1: start each solve from the previous displacement */
    /* HeavisideFilter (HeavisideFilter.h:16-98) in place of DensityFilter, with the
     * samples' beta continuation (sample_optimize_density_oc.cpp:85-88): at every
     * iteration k with k % beta_every == 0, beta *= beta_mult */
    int heaviside;           /* 0: DensityFilter, 1: HeavisideFilter */
    double beta;             /* beta before the first continuation step (the samples: 0.5) */
    int beta_every;          /* continuation period (the samples: 40; 0: never) */
    double beta_mult;        /* continuation factor (the samples: 2) */
} psf_simp_params;

typedef struct {
    double f, g;             /* objective and volume constraint of this iteration */
    double lambda;           /* last OC lambda */
    int newton_steps;        /* MMA / CONLIN interior-point steps */
    int converged;           /* IsConvergence (OC.h:67-73 / MMA.h:107-113 / CONLIN.h:82-87) on f */
    psf_solve_info solve;
    double phase_seconds[6]; /* filter, assemble, solve, sensitivity, filter-back, update */
} psf_iter_info;

/* Uploads the design s0 (ne, NULL = uniform rho0) and sets up filter/optimiser. */
psf_status psf_simp_begin(psf_ctx *ctx, const psf_simp_params *prm, const double *s0);
/* One SIMP iteration on the device (filter, volume, solve, compliance,
 * sensitivities, filtered sensitivities, OC/MMA/CONLIN update). */
psf_status psf_simp_step(psf_ctx *ctx, psf_iter_info *info);
/* The same iteration through host buffers: s_in (ne) is copied to the device
 * first, s_out / rho_out (ne, optional) and u_out (nnodes*ndof, optional) are
 * copied back.  This is the call a host loop replacing the sample driver makes. */
psf_status psf_simp_step_host(psf_ctx *ctx, const double *s_in, double *s_out, double *rho_out,
                              double *u_out, psf_iter_info *info);
/* Host copies of the current device fields (optional pointers). */
psf_status psf_simp_fields(psf_ctx *ctx, double *s, double *rho, double *dfdrho, double *dfds,
                           double *u_nodal);

/* Device pointers of the context's arrays, for callers that keep data resident
 * (name: "s", "rho", "E", "dfdrho", "dfds", "u" (nodal, nnodes*ndof doubles)). */
psf_status psf_device_ptr(psf_ctx *ctx, const char *name, void **ptr);

/* Synchronise the context's stream. */
psf_status psf_sync(psf_ctx *ctx);

/* ---------------- explicit (unstructured) meshes ---------------- */
/* The reference's general assembly path on a mesh given as coordinates + connectivity
 * (ImportFromCSV.h:23-101 meshes; sample/planestrain/sample_planestrain.cpp:20-77), on the
 * device and bit for bit the reference's results:
 *   element matrices  PlaneStrainStiffness<ShapeFunction3Triangle, Gauss1Triangle> (T3),
 *                     <ShapeFunction4Square, Gauss4Square> (Q4), HeatTransfer (Q4),
 *                     SolidLinearIsotropicElastic (H8), each from its element's coordinates;
 *   numbering         SetDirichlet + Renumbering (BoundaryCondition.h:19-25, Assembling.h:175-186);
 *   system            Assembling into LILCSR + CSR(LILCSR&) (Assembling.h:46-66, CSR.h:92-105):
 *                     pattern incl. exact zeros, columns ascending, each entry summed in
 *                     ascending element order; F -= Ke u_fixed likewise, then the point loads
 *                     (Assembling.h:151-158);
 *   solve             ScalingCG (CG.h:419-453) or CG (CG.h:123-154) on that CSR;
 *   reaction          r = sum_e Ke_e u_e over all dofs (sample_planestrain.cpp:66-77).
 * coords: nnodes x 2 (3 for H8); conn: nelem x nen (3 T3, 4 Q4, 8 H8), node ids in [0, nnodes).
 * Loads: point loads, prescribed values, uniform body forces and uniform edge tractions. */
typedef struct psf_fem psf_fem;
psf_status psf_fem_create(int kind, long long nnodes, const double *coords, long long nelem, int nen,
                          const int32_t *conn, psf_fem **out);
psf_status psf_fem_destroy(psf_fem *fem);
/* Dirichlet dofs (node, dof) with prescribed values (NULL = 0); *nfree = free dofs. */
psf_status psf_fem_set_dirichlet(psf_fem *fem, int n, const int32_t *node, const int32_t *dof,
                                 const double *value, int *nfree);
/* point loads, added to F after the element terms, in list order */
psf_status psf_fem_set_loads(psf_fem *fem, int n, const int32_t *node, const int32_t *dof, const double *value);
/* plane strain: a uniform body force (PlaneStrainBodyForce, PlaneStrain.h:503-534) on every element,
 * assembled with each element's terms; uniform tractions on 2-node edges (PlaneStrainSurfaceForce
 * <ShapeFunction2Line, Gauss1Line>, PlaneStrain.h:421-452), assembled after the point loads, in
 * edge order (sample_planestrain.cpp:42-60) */
psf_status psf_fem_set_body_force(psf_fem *fem, double fx, double fy);
psf_status psf_fem_set_edge_loads(psf_fem *fem, int nedge, const int32_t *edges, double tx, double ty);
/* element matrices (modulus / conductivity E[e], Poisson ratio V, thickness t) and the CSR system */
psf_status psf_fem_assemble(psf_fem *fem, const double *E, double V, double t, long long *nnz);
/* device time of the last psf_fem_assemble, in ms (optional pointers): the element matrices, the
 * CSR pattern (0 when the pattern of an earlier call was reused), the values and loads */
psf_status psf_fem_timings(psf_fem *fem, double *element_ms, double *pattern_ms, double *values_ms);
/* host copies (optional pointers): n2g (nnodes x ndof, -1 fixed), indptr (nfree + 1), indices and
 * data (nnz), F (nfree) */
psf_status psf_fem_get_system(psf_fem *fem, int32_t *n2g, int32_t *indptr, int32_t *indices, double *data,
                              double *F);
/* solver: PSF_SOLVE_CSR_JACOBI_F64 (ScalingCG) or PSF_SOLVE_CSR_CG_F64 (CG); u_nodal (nnodes x ndof)
 * receives the free values and the prescribed ones */
psf_status psf_fem_solve(psf_fem *fem, int solver, int itmax, double eps, double *u_nodal, psf_solve_info *info);
psf_status psf_fem_reaction(psf_fem *fem, const double *u_nodal, double *r_nodal);

/* ---------------- entry points on the reference's general data structures ---------------- */
/* CSR<T>::operator* (CSR.h:108-122) on host CSR arrays: indptr (n+1), indices and
 * data (indptr[n] entries, columns ascending per row). */
psf_status psf_csr_spmv(int n, const int32_t *indptr, const int32_t *indices, const double *data,
                        const double *x, double *y);
/* ScalingCG (CG.h:419-453; solver PSF_SOLVE_CSR_JACOBI_F64) or CG (CG.h:123-154;
 * PSF_SOLVE_CSR_CG_F64) on host CSR arrays: x0 = 0, stop when the recurrence
 * residual drops below eps*||b||, last iterate returned with PSF_NOT_CONVERGED
 * after itmax iterations.  x has n entries.  Also the solvers 7-10 (ScalingBiCGSTAB,
 * BiCGSTAB2, ILU0CG, ILU0BiCGSTAB).  Where the reference divides by a zero
 * diagonal and lets inf / NaN run, ScalingCG returns PSF_BAD_INPUT; a non-finite
 * residual (non-finite entries) returns PSF_NOT_FINITE. */
psf_status psf_csr_solve(int n, const int32_t *indptr, const int32_t *indices, const double *data,
                         const double *b, int solver, int itmax, double eps, double *x,
                         psf_solve_info *info);
/* The solvers PSF_SOLVE_CSR_ILU0_CG_F64 / _ILU0_BICGSTAB_F64 with a given ILU(0)
 * factor m on the matrix's pattern (ILU0CG(A, M, b, ...), CG.h:319; ILU0BiCGSTAB,
 * CG.h:356), m = NULL factoring A here.  The triangular solves run level by level. */
psf_status psf_csr_solve_ilu0(int n, const int32_t *indptr, const int32_t *indices, const double *data,
                              const double *m, const double *b, int solver, int itmax, double eps, double *x,
                              psf_solve_info *info);
/* ILU0 (CG.h:257-284) of a CSR matrix on its own pattern: m_out (nnz values, optional)
 * receives the factor (m_in given: used as the factor instead); with b and v_out,
 * PreILU0 (CG.h:288-315) v = U^-1 L^-1 b.  Level-scheduled on the device, each row's
 * sums in the reference's order (bit-exact). */
psf_status psf_csr_ilu0(int n, const int32_t *indptr, const int32_t *indices, const double *data,
                        const double *m_in, const double *b, double *m_out, double *v_out);
/* DensityFilter::GetFilteredVariables / GetFilteredSensitivitis (DensityFilter.h:44-71)
 * with explicit neighbour lists: out_i = sum_k w[k]*in[idx[k]] / sum_k w[k] over
 * k in [ptr[i], ptr[i+1]), summed in list order. */
psf_status psf_list_filter(int n, const int32_t *ptr, const int32_t *idx, const double *w,
                           const double *in, double *out);

/* ---------------- allocation-free solve ---------------- */
/* No counterpart in the reference.  The ScalingCG iteration of psf_csr_solve
 * (PSF_SOLVE_CSR_JACOBI_F64) for callers that cannot allocate device memory
 * when they solve: a host whose pool allocator owns the device heap, a
 * real-time or embedded loop that forbids allocation after start-up, a host
 * whose allocator belongs to another framework.  Inputs and outputs are DEVICE
 * pointers (CSR arrays of n rows and nnz stored entries, b, x); the call makes
 * no cudaMalloc / cudaFree and calls no allocating library routine.  Its
 * scratch lives in one fixed file-scope device array sized for
 * PSF_NOALLOC_MAX_ROWS rows (about 16.1 MB); larger n is rejected with
 * PSF_BAD_INPUT.
 *
 * Set-up: the driver allocates that array, and the code of the kernels the
 * solve launches, when it loads their modules, which with lazy module loading
 * (the CUDA default) happens at their first use on a device.  A call with
 * n == 0 (all pointers may be NULL) does only that set-up on the current device
 * and returns PSF_OK: make it once per device at start-up, before the host's
 * pool claims the device heap and before any stream capture.  Without it the
 * first solve on a device does the set-up itself.  Every GPU that loads the
 * library's modules holds the array until the process exits.
 *
 * The matrix is checked on the device before any kernel indexes through it:
 * indptr[0] == 0, indptr non-decreasing, indptr[n] == nnz, column indices in
 * [0, n); a malformed matrix returns PSF_BAD_INPUT.  Every call reuses the same
 * array, so calls that overlap on the GPU (other streams, other host threads)
 * race: order them on one stream or synchronise between them.  stream may be
 * NULL (the default stream).  The call returns after its work is done.
 * info->rel_residual is the FP64 true residual |b - A x| / |b| of the result,
 * info->rel_residual_recurrence the CG recurrence's.  Returns
 * PSF_NOT_CONVERGED with the last iterate after itmax iterations. */
#define PSF_NOALLOC_MAX_ROWS 262144
psf_status psf_csr_solve_noalloc(int n, int64_t nnz, const int32_t *d_indptr, const int32_t *d_indices,
                                 const double *d_data, const double *d_b, double *d_x, int itmax,
                                 double eps, void *stream, psf_solve_info *info);

/* ---------------- learned preconditioner: the network ---------------- */
/* No counterpart in the reference (its solvers have no learned part).  A
 * 4-level U-Net on the node grid (H x W nodes, H and W odd so that the levels
 * nest: H = 8k+1, W = 8m+1), base width c0 (16: channels 16, 32, 64, 128), bf16 weights and
 * activations with fp32 accumulation on the tensor cores, trained with Adam on
 * the GPU.  Inputs are [B][H][W][8] (density, the two residual components,
 * the moduli of the four surrounding elements, one zero channel), outputs [B][H][W][2].  The parameter vector is laid out
 * per layer as W[co][tap][ci] then b[co] (oracle/unet_oracle.c restates the
 * network on the CPU). */
typedef struct psf_unet psf_unet;
psf_status psf_unet_create(int c0, int H, int W, int batch, uint64_t seed, psf_unet **net);
psf_status psf_unet_destroy(psf_unet *net);
int psf_unet_nparams(const psf_unet *net);
psf_status psf_unet_set_params(psf_unet *net, const float *host, int n);
psf_status psf_unet_get_params(const psf_unet *net, float *host, int n);
/* the factor the preconditioner applies to the network output (the rms of the
 * training targets, set by psf_learned_train); saved beside the parameters */
psf_status psf_unet_get_out_scale(const psf_unet *net, float *scale);
psf_status psf_unet_set_out_scale(psf_unet *net, float scale);
/* forward of B host samples (B <= batch of psf_unet_create) */
psf_status psf_unet_forward_host(psf_unet *net, int B, const float *in, float *out);
/* forward, masked mean squared error against tgt, backward: loss, output and
 * parameter gradient (any output pointer may be NULL; mask may be NULL) */
psf_status psf_unet_loss_grad_host(psf_unet *net, int B, const float *in, const float *tgt,
                                   const float *mask, double *loss, float *out, float *grad);
/* one tensor-core convolution on host arrays (test and tuning hook):
 * y[b][o][n] = act(bias[n] + sum_tap sum_ci w[n][tap][ci] x[b][src(o, tap)][ci]) with
 * src by mode: 0 stride 1, 1 stride 2, 2 transposed stride 1, 3 transposed stride 2;
 * x [B][hin][win][cin] (cin a multiple of 8), y [B][hout][wout][N], N in
 * {16, 32, 48, 64, 96, 128, 192}; inputs and weights are rounded to bf16 */
psf_status psf_unet_conv(int mode, int N, int cin, int hin, int win, int hout, int wout, int B,
                         const float *x, const float *w, const float *bias, int relu, float *y);

/* ---------------- learned preconditioner: training and use ---------------- */
/* No counterpart in the reference.  PSF_SOLVE_IR_LEARNED_F32 runs flexible CG
 * in FP64 whose preconditioner is a pre-stage in FP32 (pre_mg = 1: one
 * multigrid V-cycle; 0: nu_pre l1-Jacobi sweeps), a U-Net correction of the
 * remaining residual (bf16), and nu_post l1-Jacobi sweeps; the FP64 true
 * residual decides convergence; after a stall (fallback_after iterations, 0:
 * twice the previous converged solve, < 0: never) it falls back to FP64 Jacobi
 * PCG and reports fell_back.  use_net = 0 keeps the same cycle without the
 * network (the ablation).  The network's grid must be (nx+1) x (ny+1) nodes of a
 * 2D problem and must outlive the context's use of it. */
psf_status psf_learned_attach(psf_ctx *ctx, psf_unet *net, int pre_mg, int nu_pre, int nu_post, int use_net,
                              int fallback_after);
/* one application z = M(r) of the attached preconditioner to a host vector of
 * free dofs (diagnostics and tests; fallback_after < 0 disables the fallback) */
psf_status psf_learned_apply(psf_ctx *ctx, const double *r, double *z);

/* Training pairs on the device, grid H x W nodes: input (density, D^-1/2 r1 / s),
 * target D^1/2 K^-1 r1 / s, per-pair weighted mask. */
typedef struct psf_trainset psf_trainset;
psf_status psf_trainset_create(int H, int W, int capacity, psf_trainset **ts);
psf_status psf_trainset_destroy(psf_trainset *ts);
int psf_trainset_size(const psf_trainset *ts);
/* npairs pairs from the context's current design: residuals of the multigrid
 * FCG after iters[k % niters] iterations from zero (NULL: 0, 2, 4, 6), smoothed
 * by the attached preconditioner's pre-stage (default: one V-cycle), and the
 * FP64 solutions of what remains (multigrid FCG
 * to 1e-8).  The context's displacement is left unchanged. */
psf_status psf_learned_harvest(psf_ctx *ctx, psf_trainset *ts, int npairs, const int *iters, int niters);
/* steps of Adam (batch samples drawn with a seeded generator, warm-up then
 * cosine decay from lr).  loss_mode 0: mean squared error of the target
 * D^1/2 K^-1 r1 / s; 1: energy norm of the correction's error,
 * (y - t) . K^ (y - t) / t . K^ t with K^ = D^-1/2 K D^-1/2 (the norm flexible
 * CG minimises); 2: its scale-free form 1 - (y . rhat)^2 / ((y . K^ y)(t . rhat)),
 * the error left by the best multiple of the correction (the solver applies the
 * correction with that energy-optimal step; batch <= 16).  loss_hist (may be NULL)
 * receives per step the loss relative to that of a zero output (1 = nothing learned) */
psf_status psf_learned_train(psf_unet *net, psf_trainset *ts, int steps, int batch, float lr, uint64_t seed,
                             int loss_mode, double *loss_hist);
/* mean over pairs [first, first + count) of the energy-norm error of the
 * network's correction relative to that of no correction (1 = no gain):
 * mode 1 as the network outputs it, mode 2 with the energy-optimal step the
 * solver applies */
psf_status psf_learned_eval(psf_unet *net, psf_trainset *ts, int first, int count, int mode,
                            double *mean_rel_energy);

/* ---------------- VTK output ---------------- */
/* Replaces the per-iteration dump of sample_optimize_density_oc.cpp:173-181
 * (ExportToVTK.h:19-141): writes the current iteration (points, cells, cell
 * types, point vectors "u" and "r" = K u over all dofs, cell scalars "s" = the
 * filtered density) as a legacy ASCII VTK file with the reference writer's
 * formatting.  async = 1 returns after queueing the device->host copy; a host
 * thread writes the file (psf_export_wait, or the next export, joins it). */
psf_status psf_export_vtk(psf_ctx *ctx, const char *path, int async);
psf_status psf_export_wait(psf_ctx *ctx);

/* ---------------- batched heat-conduction SIMP ---------------- */
/* No counterpart in the reference (its samples run one problem per process).
 * ninst independent 2D heat-sink problems (HeatTransfer Q4, unit elements,
 * uniform unit source lumped to the nodes, zero-temperature patch of nodes
 * patch_i0 .. patch_i0 + patch_w on edge 0: j = 0, 1: j = side, 2: i = 0,
 * 3: i = side; even sides whose halving reaches <= 64 nodes), each with its own
 * volume fraction.  A team of `cluster` CTAs (1, 2, 4 or 8: a thread-block
 * cluster) of `threads` (128, 256 or 512) threads owns an instance in each
 * phase; one SIMP iteration of all instances (filter + conductivities,
 * multigrid-preconditioned FCG to the FP64 true residual cg_eps, compliance +
 * sensitivities, OC) is captured as one CUDA graph by psf_batch_begin. */
typedef struct psf_batch psf_batch;
psf_status psf_batch_create(int ninst, const int *side, const int *edge, const int *patch_w, const int *patch_i0,
                            const double *vf, int threads, int cluster, psf_batch **batch);
psf_status psf_batch_destroy(psf_batch *batch);
/* shared parameters: E1 = k0, E0 = kmin, p, R, OC parameters, cg_eps, cg_itmax,
 * warm_start (optimizer must be 0); starts every instance at s = vf */
psf_status psf_batch_begin(psf_batch *batch, const psf_simp_params *prm);
/* iters SIMP iterations of every instance (graph replays); device seconds */
psf_status psf_batch_step(psf_batch *batch, int iters, double *seconds);
/* per instance 10 values: f, g, OC lambda, solver iterations, FP64 relative
 * residual, solve converged, refinement passes, bisection steps, the compliance of
 * the last update, done (IsConvergence held, OC.h:67-73: the instance's design is
 * no longer updated, as the samples leave their loop there) */
psf_status psf_batch_results(psf_batch *batch, double *out);
/* one SIMP iteration without the graph, device seconds of the four phases
 * (filter + conductivities, solve, sensitivities, OC) */
psf_status psf_batch_profile(psf_batch *batch, double *phase_seconds);
psf_status psf_batch_fields(psf_batch *batch, int instance, double *s, double *rho, double *T);

#ifdef __cplusplus
}
#endif
#endif
