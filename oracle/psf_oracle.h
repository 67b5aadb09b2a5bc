/*
 * psf_oracle.h -- CPU oracle for the SIMP topology-optimisation path of PANSFEM2.
 *
 * TEST INFRASTRUCTURE, NOT PRODUCT CODE.  This is a plain-C restatement of the
 * reference algorithm, used only as the checker by tests/, by
 * __graft_entry__.smoke() and by bench.py's CPU-baseline / reference leg.  The
 * GPU library never links, loads or calls it.
 *
 * Every function follows one reference routine and keeps its floating-point
 * operation order (built with -ffp-contract=off for the parity build), so that
 * the oracle reproduces the reference bit for bit on the same host.  Citations
 * are paths inside the PANSFEM2 source tree.
 */
#ifndef PSF_ORACLE_H
#define PSF_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* element kinds (shared numbering with the GPU library) */
enum { ORC_Q4_PLANE_STRAIN = 0, ORC_Q4_HEAT = 1, ORC_H8_SOLID = 2, ORC_T3_PLANE_STRAIN = 3 };

/* ---------------- mesh: src/PrePost/Mesher/SquareMesh.h:61-106 ---------------- */
void orc_q4_nodes(double lx, double ly, int nx, int ny, double *xy);
void orc_q4_elements(int nx, int ny, int *conn);
/* 3D analogue with the same i-major convention: node ((ny+1)*i+j)*(nz+1)+k */
void orc_h8_nodes(double lx, double ly, double lz, int nx, int ny, int nz, double *xyz);
void orc_h8_elements(int nx, int ny, int nz, int *conn);

/* ------------- numbering: BoundaryCondition.h:19-25 + Assembling.h:175-186 ------------- */
int orc_renumber(int nnodes, int ndof, const unsigned char *fixed, int *n2g);

/* ---------------- element matrices ---------------- */
/* PlaneStrainStiffness<ShapeFunction4Square, Gauss4Square>  (src/FEM/Equation/PlaneStrain.h:20-58) */
void orc_ke_planestrain_q4(const double *X, double E, double V, double t, double *Ke);
/* HeatTransfer<ShapeFunction4Square, Gauss4Square>  (src/FEM/Equation/HeatTransfer.h:19-43) */
void orc_ke_planestrain_t3(const double *X, double E, double V, double t, double *Ke);   /* T3, Gauss1Triangle */
void orc_ke_heat_q4(const double *X, double alpha, double t, double *Ke);
/* SolidLinearIsotropicElastic<ShapeFunction8Cubic, Gauss8Cubic>  (src/FEM/Equation/Solid.h:20-64) */
void orc_ke_solid_h8(const double *X, double E, double V, double *Ke);
/* dispatch by kind: nen nodes, ndof dofs per node, dim coordinates */
void orc_kind_shape(int kind, int *nen, int *ndof, int *dim);
void orc_ke(int kind, const double *X, double E, double V, double t, double *Ke);

/* -------- assembly: Assembling.h:46-66, LILCSR.h:91-114, CSR.h:92-105, Assembling.h:151-158 -------- */
typedef struct {
    int rows;
    long long nnz;
    int *indptr;
    int *indices;
    double *data;
} orc_csr;

/* Assemble K (free x free, CSR with sorted columns) and the Dirichlet lift
 * into F for every element in ascending order, exactly as the reference's
 * element loop with LILCSR get/set does.  E_e holds the per-element modulus
 * (conductivity for heat).  ufixed (nnodes*ndof, may be NULL = zeros) holds the
 * prescribed values.  F (length N) must be zeroed by the caller.  Returns 0. */
int orc_assemble(int kind, int ne, const int *conn, const double *coords, const double *E_e,
                 double V, double t, const int *n2g, const double *ufixed, int N,
                 orc_csr *out, double *F);
/* the same with a uniform body force (PlaneStrainBodyForce) per element (body != 0) */
int orc_assemble_body(int kind, int ne, const int *conn, const double *coords, const double *E_e,
                      double V, double t, const int *n2g, const double *ufixed, int N, int body, double bfx,
                      double bfy, orc_csr *out, double *F);
void orc_body_force(int kind, const double *X, double fx, double fy, double t, double *Fe);
/* uniform traction on 2-node edges (PlaneStrainSurfaceForce<ShapeFunction2Line, Gauss1Line>) into F */
void orc_edge_loads(int nedge, const int *edges, const double *coords, double tx, double ty, double t,
                    const int *n2g, double *F);
void orc_csr_free(orc_csr *A);
void orc_neumann(int nload, const int *node, const int *dof, const double *val, int ndof,
                 const int *n2g, double *F);

/* ---------------- linear algebra: src/LinearAlgebra/Solvers/CG.h ---------------- */
void orc_spmv(const orc_csr *A, const double *x, double *y);                 /* CSR.h:108-122 */
double orc_csr_get(const orc_csr *A, int row, int col);                      /* CSR.h:154-167 */
int orc_csr_set(orc_csr *A, int row, int col, double v);                     /* CSR.h:125-151 */
/* Each solver writes the last iterate into x and returns the iteration count
 * (k+1 at convergence) or -1 on "Convergence:faild" after itmax iterations. */
int orc_scaling_cg(const orc_csr *A, const double *b, int itmax, double eps, double *x); /* :419-453 */
int orc_cg(const orc_csr *A, const double *b, int itmax, double eps, double *x);         /* :123-154 */
int orc_bicgstab(const orc_csr *A, const double *b, int itmax, double eps, double *x);   /* :158-193 */
int orc_bicgstab2(const orc_csr *A, const double *b, int itmax, double eps, double *x);  /* :197-253 */
int orc_scaling_bicgstab(const orc_csr *A, const double *b, int itmax, double eps, double *x);   /* :457-495 */
int orc_ilu0_bicgstab(const orc_csr *A, const orc_csr *M, const double *b, int itmax, double eps,
                      double *x);                                                          /* :356-391 */
int orc_ilu0(const orc_csr *A, orc_csr *M);                                              /* :257-284 */
void orc_pre_ilu0(const orc_csr *M, const double *b, double *v);                         /* :288-315 */
int orc_ilu0_cg(const orc_csr *A, const orc_csr *M, const double *b, int itmax, double eps,
                double *x);                                                              /* :319-352 */
/* relative FP64 true residual ||b - A x|| / ||b|| */
double orc_true_residual(const orc_csr *A, const double *b, const double *x);

/* ---------------- filters: src/Optimize/Filter/*.h ---------------- */
/* CenterOfGravity (General.h:70-77) for every element */
void orc_centroids(int ne, int nen, int dim, const int *conn, const double *coords, double *cg);
/* Neighbour lists of the samples (sample_optimize_density_oc.cpp:50-60): every j
 * with |cg_i - cg_j| <= R in ascending j, weight (R - d)/R.  grid = {nx,ny,nz}
 * (nz = 0 for 2D) enables a windowed search that yields the identical lists;
 * grid = NULL runs the all-pairs loop.  ptr has ne+1 entries; idx/w are
 * allocated here (free with orc_free). Returns the total entry count. */
long long orc_neighbors(int ne, int dim, const double *cg, double R, const int *grid,
                        int *ptr, int **idx, double **w);
void orc_free(void *p);
void orc_density_filter(int n, const int *ptr, const int *idx, const double *w,
                        const double *s, double *rho);                       /* DensityFilter.h:44-56 */
void orc_sensitivity_filter(int n, const int *ptr, const int *idx, const double *w, const double *s,
                            const double *d, int mode, double *out);
void orc_density_filter_sens(int n, const int *ptr, const int *idx, const double *w,
                             const double *dfdrho, double *dfds);            /* DensityFilter.h:59-71 */
void orc_heaviside_filter(int n, const int *ptr, const int *idx, const double *w, double beta,
                          const double *s, double *rho);                     /* HeavisideFilter.h:60-73 */
void orc_heaviside_filter_sens(int n, const int *ptr, const int *idx, const double *w, double beta,
                               const double *s, const double *dfdrho, double *dfds); /* :76-98 */

/* ---------------- SIMP objective: sample_optimize_density_oc.cpp:136-162 ---------------- */
/* Reaction r = sum_e Ke(E_e) u_e over all dofs, f = scale0 * sum_nodes u.r and
 * dfdrho_e = -scale0*p*(E1 - E0)*rho^(p-1) * u_e.(Ke(1) u_e).  u is the nodal
 * field (nnodes*ndof).  Returns f; writes r (may be NULL) and dfdrho. */
double orc_compliance_sens(int kind, int nnodes, int ne, const int *conn, const double *coords,
                           const double *rho, double E1, double E0, double p, double V, double t,
                           double scale0, const double *u, double *r, double *dfdrho);

/* ---------------- optimisers ---------------- */
/* OC::UpdateVariables (src/Optimize/Solver/OC.h:76-107); the volume callback
 * of the samples (sample_optimize_density_oc.cpp:198-207) with a density
 * filter: g(x) = sum_i scale1*rho_i/(vf*n) - scale1.  Returns the last lambda. */
double orc_oc_update(int n, double iota, double lmin, double lmax, double leps, double move,
                     double *xk, const double *dfdx, const double *dgdx,
                     const int *ptr, const int *idx, const double *w,
                     double vf, double scale1, int heaviside, double beta);
int orc_is_convergence(double f, double prev, double eps);                   /* OC.h:67-73 */

/* MMA (src/Optimize/Solver/MMA.h:18-509), general m, both Newton branches. */
typedef struct orc_mma orc_mma;
orc_mma *orc_mma_create(int n, int m, double a0, const double *a, const double *c, const double *d,
                        const double *xmin, const double *xmax);
void orc_mma_set_parameters(orc_mma *o, double raa0, double albefa, double move, double asyinit,
                            double asydecr, double asyincr, double epsvalue);
int orc_mma_is_convergence(orc_mma *o, double f);
/* dgdx is m rows of n.  Returns the number of interior-point Newton steps. */
int orc_mma_update(orc_mma *o, double *xk, double f, const double *dfdx, const double *g,
                   const double *dgdx);
void orc_mma_destroy(orc_mma *o);

/* CONLIN (src/Optimize/Solver/CONLIN.h:17-455), general m, both Newton branches. */
typedef struct orc_conlin orc_conlin;
orc_conlin *orc_conlin_create(int n, int m, double a0, const double *a, const double *c, const double *d,
                              const double *xmin, const double *xmax);
void orc_conlin_set_parameters(orc_conlin *o, double move, double epsvalue);
int orc_conlin_is_convergence(orc_conlin *o, double f);
/* dgdx is m rows of n.  Returns the number of interior-point Newton steps. */
int orc_conlin_update(orc_conlin *o, double *xk, double f, const double *dfdx, const double *g,
                      const double *dgdx);
void orc_conlin_destroy(orc_conlin *o);

/* ---------------- whole SIMP loop (the sample drivers, configurable) ---------------- */
typedef struct {
    int kind;                 /* ORC_* element kind */
    int nx, ny, nz;           /* elements per axis (nz = 0 in 2D) */
    double lx, ly, lz;
    double V, t;              /* Poisson ratio, thickness */
    double E1, E0, p;         /* E = E1*rho^p + E0*(1 - rho^p) (sample law) */
    double vf, R, scale0, scale1, rho0;
    int optimizer;            /* 0 = OC, 1 = MMA, 2 = CONLIN (a0, c, d, xmin, xmax, move, eps: the mma_ fields) */
    double oc_iota, oc_lmin, oc_lmax, oc_leps, oc_move;
    double mma_raa0, mma_albefa, mma_move, mma_asyinit, mma_asydecr, mma_asyincr, mma_eps;
    double mma_a0, mma_c, mma_d, mma_xmin, mma_xmax;
    int cg_itmax;
    double cg_eps;
    int heaviside;            /* 0 = DensityFilter, 1 = HeavisideFilter with beta doubling every 40 its */
    /* boundary conditions: prescribed value 0 at (node, dof); point loads */
    int nfix;
    const int *fix_node, *fix_dof;
    int nload;
    const int *load_node, *load_dof;
    const double *load_val;
} orc_simp_cfg;

typedef struct {
    /* per-iteration scalars (length iters) */
    double *f, *g, *lambda;
    int *cg_iters, *mma_newton;
    double *true_res;
    /* per-iteration fields, optional (NULL to skip): iters*ne / iters*nnodes*ndof */
    double *rho, *dfdrho, *dfds, *s_after, *u;
    /* final design (ne) */
    double *s_final;
    /* phase timings in seconds, summed over the run (optional, length 8):
       filter, assemble, csr, solve, reaction+sens, filter_sens, update, other */
    double *phase_seconds;
} orc_simp_out;

/* Runs `iters` SIMP iterations (no early stop unless stop_on_convergence).
 * Returns the number of iterations done. */
int orc_simp_run(const orc_simp_cfg *cfg, int iters, int stop_on_convergence, orc_simp_out *out);

/* OpenMP threads the SpMV uses (0 = runtime default) */
void orc_set_threads(int n);
int orc_get_threads(void);

#ifdef __cplusplus
}
#endif
#endif
