// psf_capi.cu -- the extern "C" boundary (include/pansfem2_gpu.h) and the
// on-device SIMP iteration (the loop body of sample_optimize_density_oc.cpp:83-208
// and sample_optimize_density_mma.cpp:88-204).
#include <cmath>
#include <cstring>
#include <new>

#include "psf_internal.cuh"

namespace psf {
psf_status set_dirichlet(Ctx *c, int n, const int *node, const int *dof, const double *value);  // psf_mesh.cu
psf_status filter_setup(Ctx *c, double R);                                                      // psf_opt.cu
psf_status filter_moduli(Ctx *c, const double *s, double *rho, double *E, double E1, double E0, double p,
                         double vf, double scale1, double *g_dev);
psf_status fill(Ctx *c, double *x, long long n, double v);
}  // namespace psf

using namespace psf;

#define CTX_CHECK(ctx)                                                        \
    do {                                                                      \
        if (!(ctx)) { set_error("null context"); return PSF_BAD_INPUT; }      \
    } while (0)

static psf_status h2d(Ctx *c, void *dst, const void *src, size_t bytes) {
    PSF_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, c->stream));
    return PSF_OK;
}
static psf_status d2h_sync(Ctx *c, void *dst, const void *src, size_t bytes) {
    PSF_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, c->stream));
    PSF_CUDA(cudaStreamSynchronize(c->stream));
    return PSF_OK;
}

extern "C" {

const char *psf_last_error(void) { return last_error(); }

psf_status psf_kernel_launches(long long *n) {
    if (!n) { set_error("psf_kernel_launches: null output"); return PSF_BAD_INPUT; }
    *n = launches();
    return PSF_OK;
}

psf_status psf_set_launch_shape(psf_ctx *h, int kernel, int a, int b, int c) {
    if (!h) { set_error("psf_set_launch_shape: null context"); return PSF_BAD_INPUT; }
    Ctx *x = &h->c;
    if (c < 1 || c > 8) { set_error("psf_set_launch_shape: blocks per SM must be in [1, 8]"); return PSF_BAD_INPUT; }
    if (kernel == PSF_KERNEL_PCG_CSR) {
        if ((a != 1 && a != 4 && a != 8 && a != 16) || (b != 256 && b != 512 && b != 1024)) {
            set_error("psf_set_launch_shape: PCG lanes per row must be 1 (sliced copy), 4, 8 or 16 and threads "
                      "256, 512 or 1024");
            return PSF_BAD_INPUT;
        }
        x->pcg_lanes = a;
        x->pcg_threads = b;
        x->pcg_blocks_per_sm = c;
        return PSF_OK;
    }
    if (kernel == PSF_KERNEL_OPT) {
        x->opt_blocks_per_sm = c;
        return PSF_OK;
    }
    set_error("psf_set_launch_shape: unknown kernel family");
    return PSF_BAD_INPUT;
}

psf_status psf_diag_barrier_timeout(psf_ctx *h, int blocks, int64_t spin_limit) {
    if (!h) { set_error("psf_diag_barrier_timeout: null context"); return PSF_BAD_INPUT; }
    if (spin_limit < 1 || spin_limit > (1ll << 23)) {
        set_error("psf_diag_barrier_timeout: spin_limit must be in [1, 2^23]");
        return PSF_BAD_INPUT;
    }
    return diag_barrier_timeout(&h->c, blocks, (long long)spin_limit);
}

psf_status psf_get_launch_shape(const psf_ctx *h, int kernel, int *a, int *b, int *c) {
    if (!h || !a || !b || !c) { set_error("psf_get_launch_shape: null argument"); return PSF_BAD_INPUT; }
    const Ctx *x = &h->c;
    if (kernel == PSF_KERNEL_PCG_CSR) {
        *a = x->pcg_lanes; *b = x->pcg_threads; *c = x->pcg_blocks_per_sm;
        return PSF_OK;
    }
    if (kernel == PSF_KERNEL_OPT) {
        *a = 0; *b = 256; *c = x->opt_blocks_per_sm;
        return PSF_OK;
    }
    set_error("psf_get_launch_shape: unknown kernel family");
    return PSF_BAD_INPUT;
}

psf_status psf_create(psf_ctx **out, int kind, int nx, int ny, int nz, double lx, double ly, double lz, double V,
                      double t) {
    if (!out) { set_error("psf_create: null output"); return PSF_BAD_INPUT; }
    *out = nullptr;
    if (kind < 0 || kind > 2 || nx < 1 || ny < 1 || (kind == PSF_H8_SOLID && nz < 1) || !(lx > 0) || !(ly > 0) ||
        (kind == PSF_H8_SOLID && !(lz > 0))) {
        set_error("psf_create: invalid kind or grid");
        return PSF_BAD_INPUT;
    }
    psf_ctx *h = new (std::nothrow) psf_ctx;
    if (!h) { set_error("psf_create: out of host memory"); return PSF_BAD_INPUT; }
    Ctx *c = &h->c;
    c->kind = kind;
    c->nx = nx; c->ny = ny; c->nz = kind == PSF_H8_SOLID ? nz : 0;
    c->lx = lx; c->ly = ly; c->lz = kind == PSF_H8_SOLID ? lz : 0.0;
    c->V = V; c->t = t;
    c->nen = kind == PSF_H8_SOLID ? 8 : 4;
    c->ndof = kind == PSF_Q4_PLANE_STRAIN ? 2 : (kind == PSF_Q4_HEAT ? 1 : 3);
    c->dim = kind == PSF_H8_SOLID ? 3 : 2;
    const bool is3d = kind == PSF_H8_SOLID;
    c->ne = is3d ? (long long)nx * ny * nz : (long long)nx * ny;
    c->nnodes = is3d ? (long long)(nx + 1) * (ny + 1) * (nz + 1) : (long long)(nx + 1) * (ny + 1);
    c->ndofs = c->nnodes * c->ndof;
    if (c->ndofs > 0x7fffffffll) { delete h; set_error("psf_create: grid exceeds int32 dof numbering"); return PSF_BAD_INPUT; }
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&c->ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&c->ev1);
    if (e == cudaSuccess) e = cudaEventCreate(&c->evk0);
    if (e == cudaSuccess) e = cudaEventCreate(&c->evk1);
    if (e != cudaSuccess) { delete h; return cuda_status(e, "psf_create"); }
    const long long padn = is3d ? (long long)(nx + 2) * (ny + 2) * (nz + 2) : (long long)(nx + 2) * (ny + 2);
    psf_status st = PSF_OK;
#define A(x) if (st == PSF_OK) st = (x)
    A(dzalloc(c, &c->n2g, c->ndofs));
    A(dzalloc(c, &c->fixed, c->ndofs));
    A(dzalloc(c, &c->ufixed, c->ndofs));
    A(dzalloc(c, &c->Ke0, 576));
    A(dzalloc(c, &c->Fn, c->ndofs));
    A(dzalloc(c, &c->un, c->ndofs));
    A(dzalloc(c, &c->E, c->ne));
    A(dzalloc(c, &c->Ef, c->ne));
    A(dzalloc(c, &c->Epad, padn));
    A(dzalloc(c, &c->Epadf, padn));
    A(dzalloc(c, &c->Dn, c->ndofs));
    A(dzalloc(c, &c->Dnf, c->ndofs));
    A(dzalloc(c, &c->Dl1f, c->ndofs));
    A(dzalloc(c, &c->w64[0], 7 * c->ndofs));   // the CSR PCG's workspace (7 vectors)
    for (int k = 1; k < 8; k++) A(dzalloc(c, &c->w64[k], c->ndofs));
    for (int k = 0; k < 8; k++) A(dzalloc(c, &c->w32[k], c->ndofs));
    A(dzalloc(c, &c->gs, 1));
    A(dzalloc(c, &c->partials, (size_t)kPartialSlots * 8192));   // grid_sync partials for up to 8192 blocks
    A(dzalloc(c, &c->scal, 64));
    A(dzalloc(c, &c->filt_wsum, c->ne));
    A(dzalloc(c, &c->filt_vw, c->ne));
    A(dzalloc(c, &c->oc_bp, c->ne));
    A(dzalloc(c, &c->oc_cs, 2 * ((c->ne + kChunk - 1) / kChunk)));
    for (double **p : {&c->s, &c->rho, &c->dfdrho, &c->dgdrho, &c->dfds, &c->dgds, &c->snew}) A(dzalloc(c, p, c->ne));
    if (st == PSF_OK) st = ke_element0(c, 1.0, c->Ke0);
    if (st == PSF_OK) {
        const int nk = c->nen * c->ndof;
        c->Ke0_host.assign(nk * nk, 0.0);
        st = d2h_sync(c, c->Ke0_host.data(), c->Ke0, sizeof(double) * nk * nk);
    }
#undef A
    if (st != PSF_OK) {
        psf_destroy(h);
        return st;
    }
    *out = h;
    return PSF_OK;
}

psf_status psf_destroy(psf_ctx *h) {
    if (!h) return PSF_OK;
    Ctx *c = &h->c;
    if (c->stream) cudaStreamSynchronize(c->stream);
    vtk_free(c);
    mg_free(c);
    learned_free(c);
    for (void *p : c->allocs) cudaFree(p);
    for (void *p : {(void *)c->g2n, (void *)c->indptr, (void *)c->indices, (void *)c->diag, (void *)c->data,
                    (void *)c->F, (void *)c->u, (void *)c->sell_ptr, (void *)c->sell_col, (void *)c->sell_val})
        if (p) cudaFree(p);
    if (c->ev0) cudaEventDestroy(c->ev0);
    if (c->ev1) cudaEventDestroy(c->ev1);
    if (c->evk0) cudaEventDestroy(c->evk0);
    if (c->evk1) cudaEventDestroy(c->evk1);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete h;
    return PSF_OK;
}

psf_status psf_sizes(const psf_ctx *h, int64_t *ne, int64_t *nnodes, int *ndof, int64_t *nfree, int64_t *nnz) {
    CTX_CHECK(h);
    const Ctx *c = &h->c;
    if (ne) *ne = c->ne;
    if (nnodes) *nnodes = c->nnodes;
    if (ndof) *ndof = c->ndof;
    if (nfree) *nfree = c->nfree;
    if (nnz) *nnz = c->nnz;
    return PSF_OK;
}

psf_status psf_set_dirichlet(psf_ctx *h, int n, const int *node, const int *dof, const double *value,
                             int32_t *n2g_out) {
    CTX_CHECK(h);
    Ctx *c = &h->c;
    if (n < 0 || (n > 0 && (!node || !dof))) { set_error("psf_set_dirichlet: bad arrays"); return PSF_BAD_INPUT; }
    PSF_CHECK(set_dirichlet(c, n, node, dof, value));
    if (n2g_out) PSF_CHECK(d2h_sync(c, n2g_out, c->n2g, sizeof(int) * c->ndofs));
    return PSF_OK;
}

psf_status psf_set_loads(psf_ctx *h, int n, const int *node, const int *dof, const double *value) {
    CTX_CHECK(h);
    Ctx *c = &h->c;
    if (n < 0 || (n > 0 && (!node || !dof || !value))) { set_error("psf_set_loads: bad arrays"); return PSF_BAD_INPUT; }
    for (int k = 0; k < n; k++)
        if (node[k] < 0 || node[k] >= c->nnodes || dof[k] < 0 || dof[k] >= c->ndof) {
            set_error("psf_set_loads: (node, dof) out of range");
            return PSF_BAD_INPUT;
        }
    c->load_node.assign(node, node + n);
    c->load_dof.assign(dof, dof + n);
    c->load_val.assign(value, value + n);
    if (c->have_bc) PSF_CHECK(build_rhs(c));
    return PSF_OK;
}

psf_status psf_element_matrix(psf_ctx *h, double E, double *Ke_out) {
    CTX_CHECK(h);
    Ctx *c = &h->c;
    if (!Ke_out) { set_error("psf_element_matrix: null output"); return PSF_BAD_INPUT; }
    double *tmp = nullptr;
    PSF_CUDA(cudaMallocAsync((void **)&tmp, 576 * sizeof(double), c->stream));
    PSF_CHECK(ke_element0(c, E, tmp));
    const int nk = c->nen * c->ndof;
    psf_status st = d2h_sync(c, Ke_out, tmp, sizeof(double) * nk * nk);
    cudaFreeAsync(tmp, c->stream);
    return st;
}

psf_status psf_build_csr(psf_ctx *h, int32_t *indptr_out, int32_t *indices_out) {
    CTX_CHECK(h);
    Ctx *c = &h->c;
    PSF_CHECK(build_pattern(c));
    if (indptr_out) PSF_CHECK(d2h_sync(c, indptr_out, c->indptr, sizeof(int) * (c->nfree + 1)));
    if (indices_out) PSF_CHECK(d2h_sync(c, indices_out, c->indices, sizeof(int) * c->nnz));
    return PSF_OK;
}

psf_status psf_assemble(psf_ctx *h, const double *E_e, double *data_out, double *F_out) {
    CTX_CHECK(h);
    Ctx *c = &h->c;
    if (!E_e) { set_error("psf_assemble: null E_e"); return PSF_BAD_INPUT; }
    if (!c->have_bc) { set_error("psf_assemble: call psf_set_dirichlet first"); return PSF_BAD_INPUT; }
    PSF_CHECK(h2d(c, c->E, E_e, sizeof(double) * c->ne));
    PSF_CHECK(assemble_values(c, c->E));
    if (data_out) PSF_CHECK(d2h_sync(c, data_out, c->data, sizeof(double) * c->nnz));
    if (F_out) PSF_CHECK(d2h_sync(c, F_out, c->F, sizeof(double) * c->nfree));
    PSF_CUDA(cudaStreamSynchronize(c->stream));
    return PSF_OK;
}

psf_status psf_spmv(psf_ctx *h, const double *x, double *y) {
    CTX_CHECK(h);
    Ctx *c = &h->c;
    if (!c->have_values) { set_error("psf_spmv: assemble first"); return PSF_BAD_INPUT; }
    if (!x || !y) { set_error("psf_spmv: null vector"); return PSF_BAD_INPUT; }
    double *dx = c->w64[6], *dy = c->w64[7];
    PSF_CHECK(h2d(c, dx, x, sizeof(double) * c->nfree));
    PSF_CHECK(spmv_csr64(c, dx, dy));
    return d2h_sync(c, y, dy, sizeof(double) * c->nfree);
}

psf_status psf_ebe_matvec(psf_ctx *h, const double *x, double *y) {
    CTX_CHECK(h);
    Ctx *c = &h->c;
    if (!c->have_bc) { set_error("psf_ebe_matvec: call psf_set_dirichlet first"); return PSF_BAD_INPUT; }
    if (!x || !y) { set_error("psf_ebe_matvec: null vector"); return PSF_BAD_INPUT; }
    double *dx = c->w64[6], *dy = c->w64[7], *xr = c->w64[5];
    PSF_CHECK(h2d(c, xr, x, sizeof(double) * c->nfree));
    PSF_CHECK(scatter_reduced(c, xr, dx));
    PSF_CHECK(ebe_apply64(c, dx, dy));
    PSF_CHECK(gather_reduced(c, dy, xr));
    return d2h_sync(c, y, xr, sizeof(double) * c->nfree);
}

psf_status psf_mg_precondition(psf_ctx *h, const double *r, double *z) {
    CTX_CHECK(h);
    Ctx *c = &h->c;
    if (!c->have_bc) { set_error("psf_mg_precondition: call psf_set_dirichlet and set the moduli first"); return PSF_BAD_INPUT; }
    if (!r || !z) { set_error("psf_mg_precondition: null vector"); return PSF_BAD_INPUT; }
    double *dx = c->w64[6], *dy = c->w64[7], *xr = c->w64[5];
    PSF_CHECK(h2d(c, xr, r, sizeof(double) * c->nfree));
    PSF_CHECK(scatter_reduced(c, xr, dx));
    PSF_CHECK(mg_precondition(c, dx, dy));
    PSF_CHECK(gather_reduced(c, dy, xr));
    return d2h_sync(c, z, xr, sizeof(double) * c->nfree);
}

psf_status psf_solve(psf_ctx *h, int solver, int itmax, double eps, double *u_out, psf_solve_info *info) {
    CTX_CHECK(h);
    Ctx *c = &h->c;
    if (itmax < 1 || !(eps > 0)) { set_error("psf_solve: itmax >= 1 and eps > 0 required"); return PSF_BAD_INPUT; }
    if (solver != PSF_SOLVE_CSR_JACOBI_F64 && !c->have_values) {
        // matrix-free solvers need the moduli and the load vector only
        if (!c->have_bc) { set_error("psf_solve: set boundary conditions and moduli first"); return PSF_BAD_INPUT; }
    }
    psf_status st = solve(c, solver, itmax, eps, false, info);
    if (st != PSF_OK && st != PSF_NOT_CONVERGED && st != PSF_FELL_BACK) return st;
    if (u_out) PSF_CHECK(d2h_sync(c, u_out, c->u, sizeof(double) * c->nfree));
    return st;
}

psf_status psf_filter_setup(psf_ctx *h, double R) {
    CTX_CHECK(h);
    return filter_setup(&h->c, R);
}

psf_status psf_filter_forward(psf_ctx *h, const double *s, double *rho) {
    CTX_CHECK(h);
    Ctx *c = &h->c;
    if (!s || !rho) { set_error("psf_filter_forward: null array"); return PSF_BAD_INPUT; }
    PSF_CHECK(h2d(c, c->snew, s, sizeof(double) * c->ne));
    PSF_CHECK(filter_apply(c, c->snew, c->dfds, false));
    return d2h_sync(c, rho, c->dfds, sizeof(double) * c->ne);
}

psf_status psf_filter_backward(psf_ctx *h, const double *dfdrho, double *dfds) {
    CTX_CHECK(h);
    Ctx *c = &h->c;
    if (!dfdrho || !dfds) { set_error("psf_filter_backward: null array"); return PSF_BAD_INPUT; }
    PSF_CHECK(h2d(c, c->snew, dfdrho, sizeof(double) * c->ne));
    PSF_CHECK(filter_apply(c, c->snew, c->dfds, true));
    return d2h_sync(c, dfds, c->dfds, sizeof(double) * c->ne);
}

static psf_status heaviside_scratch(Ctx *c) {
    if (c->filt_n <= 0) { set_error("HeavisideFilter: call psf_filter_setup first"); return PSF_BAD_INPUT; }
    if (!c->dH) PSF_CHECK(dalloc(c, &c->dH, c->ne));
    if (!c->tmp_ne) PSF_CHECK(dalloc(c, &c->tmp_ne, c->ne));
    return PSF_OK;
}

psf_status psf_heaviside_forward(psf_ctx *h, double beta, const double *s, double *rho) {
    CTX_CHECK(h);
    Ctx *c = &h->c;
    if (!s || !rho || !(beta > 0.0)) { set_error("psf_heaviside_forward: null array or beta <= 0"); return PSF_BAD_INPUT; }
    PSF_CHECK(heaviside_scratch(c));
    PSF_CHECK(h2d(c, c->snew, s, sizeof(double) * c->ne));
    PSF_CHECK(heaviside_forward(c, beta, c->snew, c->dfds));
    return d2h_sync(c, rho, c->dfds, sizeof(double) * c->ne);
}

psf_status psf_heaviside_backward(psf_ctx *h, double beta, const double *s, const double *dfdrho, double *dfds) {
    CTX_CHECK(h);
    Ctx *c = &h->c;
    if (!s || !dfdrho || !dfds || !(beta > 0.0)) {
        set_error("psf_heaviside_backward: null array or beta <= 0");
        return PSF_BAD_INPUT;
    }
    PSF_CHECK(heaviside_scratch(c));
    PSF_CHECK(h2d(c, c->snew, s, sizeof(double) * c->ne));
    PSF_CHECK(heaviside_forward(c, beta, c->snew, c->dfds));   // dH at filter(s)
    PSF_CHECK(h2d(c, c->snew, dfdrho, sizeof(double) * c->ne));
    PSF_CHECK(heaviside_back(c, c->snew, c->dfds));
    return d2h_sync(c, dfds, c->dfds, sizeof(double) * c->ne);
}

psf_status psf_sensitivity_filter(psf_ctx *h, int mode, const double *s, const double *dfds_in, double *dfds_out) {
    CTX_CHECK(h);
    Ctx *c = &h->c;
    if (!s || !dfds_in || !dfds_out || mode < 0 || mode > 1) {
        set_error("psf_sensitivity_filter: null array or mode not 0/1");
        return PSF_BAD_INPUT;
    }
    if (c->filt_n <= 0) { set_error("psf_sensitivity_filter: call psf_filter_setup first"); return PSF_BAD_INPUT; }
    // scratch: snew (design), dfdrho (input), dfds (output)
    PSF_CHECK(h2d(c, c->snew, s, sizeof(double) * c->ne));
    PSF_CHECK(h2d(c, c->dfdrho, dfds_in, sizeof(double) * c->ne));
    PSF_CHECK(sensitivity_filter(c, c->snew, c->dfdrho, mode, c->dfds));
    return d2h_sync(c, dfds_out, c->dfds, sizeof(double) * c->ne);
}

psf_status psf_compliance_sensitivity(psf_ctx *h, const double *rho, double E1, double E0, double p,
                                      double scale0, double *f, double *dfdrho) {
    CTX_CHECK(h);
    Ctx *c = &h->c;
    if (!rho || !f || !dfdrho) { set_error("psf_compliance_sensitivity: null array"); return PSF_BAD_INPUT; }
    PSF_CHECK(h2d(c, c->rho, rho, sizeof(double) * c->ne));
    PSF_CHECK(moduli_from_rho(c, c->rho, E1, E0, p, c->E));
    PSF_CHECK(compliance_sens(c, c->rho, E1, E0, p, scale0, c->scal + 0, c->dfdrho));
    PSF_CHECK(d2h_sync(c, dfdrho, c->dfdrho, sizeof(double) * c->ne));
    return d2h_sync(c, f, c->scal + 0, sizeof(double));
}

psf_status psf_oc_update(psf_ctx *h, double *x, const double *dfdx, const double *dgdx, double iota, double lmin,
                         double lmax, double leps, double move, double vf, double scale1, double *lambda_out) {
    CTX_CHECK(h);
    Ctx *c = &h->c;
    if (!x || !dfdx || !dgdx) { set_error("psf_oc_update: null array"); return PSF_BAD_INPUT; }
    PSF_CHECK(h2d(c, c->s, x, sizeof(double) * c->ne));
    PSF_CHECK(h2d(c, c->dfds, dfdx, sizeof(double) * c->ne));
    PSF_CHECK(h2d(c, c->dgds, dgdx, sizeof(double) * c->ne));
    PSF_CHECK(oc_update(c, c->s, c->dfds, c->dgds, iota, lmin, lmax, leps, move, vf, scale1, lambda_out));
    return d2h_sync(c, x, c->s, sizeof(double) * c->ne);
}

psf_status psf_mma_init(psf_ctx *h, double a0, double a, double cc, double d, double xmin, double xmax, double raa0,
                        double albefa, double move, double asyinit, double asydecr, double asyincr, double epsvalue) {
    CTX_CHECK(h);
    Ctx *c = &h->c;
    if (!(xmax > xmin)) { set_error("psf_mma_init: xmax must exceed xmin"); return PSF_BAD_INPUT; }
    if (!c->mma_L) {
        PSF_CHECK(dzalloc(c, &c->mma_L, c->ne));
        PSF_CHECK(dzalloc(c, &c->mma_U, c->ne));
        PSF_CHECK(dzalloc(c, &c->mma_xkm1, c->ne));
        PSF_CHECK(dzalloc(c, &c->mma_xkm2, c->ne));
        PSF_CHECK(dzalloc(c, &c->mma_work, 21 * c->ne));
    } else {
        PSF_CUDA(cudaMemsetAsync(c->mma_xkm1, 0, sizeof(double) * c->ne, c->stream));
        PSF_CUDA(cudaMemsetAsync(c->mma_xkm2, 0, sizeof(double) * c->ne, c->stream));
    }
    c->mma_a0 = a0; c->mma_a = a; c->mma_c = cc; c->mma_d = d; c->mma_xmin = xmin; c->mma_xmax = xmax;
    c->mma_raa0 = raa0; c->mma_albefa = albefa; c->mma_move = move; c->mma_asyinit = asyinit;
    c->mma_asydecr = asydecr; c->mma_asyincr = asyincr; c->mma_epsvalue = epsvalue;
    c->mma_k = 0;
    c->mma_prev = 0.0;
    c->mma_ready = true;
    return PSF_OK;
}

psf_status psf_mma_update(psf_ctx *h, double *x, double f, const double *dfdx, double g, const double *dgdx,
                          int *newton_steps) {
    CTX_CHECK(h);
    Ctx *c = &h->c;
    if (!x || !dfdx || !dgdx) { set_error("psf_mma_update: null array"); return PSF_BAD_INPUT; }
    PSF_CHECK(h2d(c, c->s, x, sizeof(double) * c->ne));
    PSF_CHECK(h2d(c, c->dfds, dfdx, sizeof(double) * c->ne));
    PSF_CHECK(h2d(c, c->dgds, dgdx, sizeof(double) * c->ne));
    psf_status st = mma_update(c, c->s, f, c->dfds, g, c->dgds, newton_steps);
    if (st != PSF_OK && st != PSF_NOT_CONVERGED) return st;
    PSF_CHECK(d2h_sync(c, x, c->s, sizeof(double) * c->ne));
    return st;
}

psf_status psf_conlin_init(psf_ctx *h, double a0, double a, double cc, double d, double xmin, double xmax,
                           double move, double epsvalue) {
    CTX_CHECK(h);
    Ctx *c = &h->c;
    if (!(xmax > xmin) || !(xmin > 0.0)) {
        // the approximation has q_j / x_j terms: the design must stay positive
        set_error("psf_conlin_init: need 0 < xmin < xmax");
        return PSF_BAD_INPUT;
    }
    if (!(move > 0.0)) { set_error("psf_conlin_init: move must be positive"); return PSF_BAD_INPUT; }
    if (!c->mma_work) PSF_CHECK(dzalloc(c, &c->mma_work, 21 * c->ne));
    c->cl_a0 = a0; c->cl_a = a; c->cl_c = cc; c->cl_d = d; c->cl_xmin = xmin; c->cl_xmax = xmax;
    c->cl_move = move; c->cl_epsvalue = epsvalue;
    c->cl_k = 0;
    c->cl_prev = 0.0;
    c->cl_ready = true;
    return PSF_OK;
}

psf_status psf_conlin_update(psf_ctx *h, double *x, double f, const double *dfdx, double g, const double *dgdx,
                             int *newton_steps) {
    CTX_CHECK(h);
    Ctx *c = &h->c;
    if (!x || !dfdx || !dgdx) { set_error("psf_conlin_update: null array"); return PSF_BAD_INPUT; }
    PSF_CHECK(h2d(c, c->s, x, sizeof(double) * c->ne));
    PSF_CHECK(h2d(c, c->dfds, dfdx, sizeof(double) * c->ne));
    PSF_CHECK(h2d(c, c->dgds, dgdx, sizeof(double) * c->ne));
    psf_status st = conlin_update(c, c->s, f, c->dfds, g, c->dgds, newton_steps);
    if (st != PSF_OK && st != PSF_NOT_CONVERGED) return st;
    PSF_CHECK(d2h_sync(c, x, c->s, sizeof(double) * c->ne));
    return st;
}

// ------------------------------------------------------------------ SIMP loop
psf_status psf_simp_begin(psf_ctx *h, const psf_simp_params *prm, const double *s0) {
    CTX_CHECK(h);
    Ctx *c = &h->c;
    if (!prm) { set_error("psf_simp_begin: null params"); return PSF_BAD_INPUT; }
    if (!c->have_bc) { set_error("psf_simp_begin: call psf_set_dirichlet / psf_set_loads first"); return PSF_BAD_INPUT; }
    if (!(prm->vf > 0) || !(prm->R > 0) || prm->cg_itmax < 1 || !(prm->cg_eps > 0)) {
        set_error("psf_simp_begin: invalid parameters");
        return PSF_BAD_INPUT;
    }
    c->prm = *prm;
    PSF_CHECK(filter_setup(c, prm->R));
    if (s0) PSF_CHECK(h2d(c, c->s, s0, sizeof(double) * c->ne));
    else PSF_CHECK(fill(c, c->s, c->ne, prm->rho0));
    // dg/drho = scale1/(vf*ne), constant (sample :99-105)
    PSF_CHECK(fill(c, c->dgdrho, c->ne, prm->scale1 / (prm->vf * (double)c->ne)));
    if (prm->solver == PSF_SOLVE_CSR_JACOBI_F64 && !c->have_csr) PSF_CHECK(build_pattern(c));
    PSF_CHECK(build_rhs(c));
    PSF_CUDA(cudaMemsetAsync(c->un, 0, sizeof(double) * c->ndofs, c->stream));
    if (prm->optimizer < 0 || prm->optimizer > 2) { set_error("psf_simp_begin: optimizer must be 0, 1 or 2"); return PSF_BAD_INPUT; }
    if (prm->optimizer == 2)   // sample_optimize_density_CONLIN.cpp:75-80
        PSF_CHECK(psf_conlin_init(h, prm->mma_a0, 0.0, prm->mma_c, prm->mma_d, prm->mma_xmin, prm->mma_xmax,
                                  prm->mma_move, prm->mma_eps));
    if (prm->optimizer == 1)
        PSF_CHECK(psf_mma_init(h, prm->mma_a0, 0.0, prm->mma_c, prm->mma_d, prm->mma_xmin, prm->mma_xmax,
                               prm->mma_raa0, prm->mma_albefa, prm->mma_move, prm->mma_asyinit, prm->mma_asydecr,
                               prm->mma_asyincr, prm->mma_eps));
    c->heav = prm->heaviside ? 1 : 0;
    c->beta = prm->beta;
    if (c->heav && !c->dH) {
        PSF_CHECK(dalloc(c, &c->dH, c->ne));
        PSF_CHECK(dalloc(c, &c->tmp_ne, c->ne));
    }
    c->oc_prev = 0.0;
    c->iter = 0;
    c->simp_ready = true;
    PSF_CUDA(cudaStreamSynchronize(c->stream));
    return PSF_OK;
}

psf_status psf_simp_step(psf_ctx *h, psf_iter_info *info) {
    CTX_CHECK(h);
    Ctx *c = &h->c;
    if (!c->simp_ready) { set_error("psf_simp_step: call psf_simp_begin first"); return PSF_BAD_INPUT; }
    const psf_simp_params &P = c->prm;
    psf_iter_info inf{};
    cudaEvent_t ev[7];
    for (auto &e : ev) PSF_CUDA(cudaEventCreate(&e));
    PSF_CUDA(cudaEventRecord(ev[0], c->stream));
    // beta continuation of the Heaviside projection (sample_optimize_density_oc.cpp:85-88)
    if (c->heav && P.beta_every > 0 && c->iter % P.beta_every == 0) c->beta *= P.beta_mult;
    // filtered densities, moduli, volume constraint (sample :93-105, :123)
    PSF_CHECK(filter_moduli(c, c->s, c->rho, c->E, P.E1, P.E0, P.p, P.vf, P.scale1, c->scal + 1));
    PSF_CUDA(cudaEventRecord(ev[1], c->stream));
    // stiffness (sample :113-131)
    if (P.solver == PSF_SOLVE_CSR_JACOBI_F64) PSF_CHECK(assemble_values(c, c->E));
    else PSF_CHECK(set_moduli(c, c->E));
    PSF_CUDA(cudaEventRecord(ev[2], c->stream));
    // displacement (sample :132-133)
    psf_status sst = solve(c, P.solver, P.cg_itmax, P.cg_eps, P.warm_start != 0, &inf.solve);
    if (sst != PSF_OK && sst != PSF_NOT_CONVERGED && sst != PSF_FELL_BACK) return sst;
    PSF_CUDA(cudaEventRecord(ev[3], c->stream));
    // compliance and sensitivities (sample :136-162)
    PSF_CHECK(compliance_sens(c, c->rho, P.E1, P.E0, P.p, P.scale0, c->scal + 0, c->dfdrho));
    PSF_CUDA(cudaEventRecord(ev[4], c->stream));
    // filtered sensitivities (sample :168-169)
    if (c->heav) {
        PSF_CHECK(heaviside_back(c, c->dfdrho, c->dfds));
        PSF_CHECK(heaviside_back(c, c->dgdrho, c->dgds));
    } else {
        PSF_CHECK(filter_apply(c, c->dfdrho, c->dfds, true));
        PSF_CHECK(filter_apply(c, c->dgdrho, c->dgds, true));
    }
    PSF_CUDA(cudaEventRecord(ev[5], c->stream));
    double fg[2];
    PSF_CHECK(d2h_sync(c, fg, c->scal, 2 * sizeof(double)));
    inf.f = fg[0];
    inf.g = fg[1];
    // IsConvergence (OC.h:67-73, MMA.h:107-113), then the update (sample :192-207)
    if (P.optimizer == 2) {   // CONLIN::IsConvergence (CONLIN.h:82-87), UpdateVariables (sample :192-204)
        inf.converged = std::fabs(inf.f - c->cl_prev) / (inf.f + c->cl_prev) < c->cl_epsvalue;
        if (!inf.converged) {
            psf_status ms = conlin_update(c, c->s, inf.f, c->dfds, inf.g, c->dgds, &inf.newton_steps);
            if (ms != PSF_OK && ms != PSF_NOT_CONVERGED) return ms;
        }
    } else if (P.optimizer == 1) {
        inf.converged = std::fabs(inf.f - c->mma_prev) / (inf.f + c->mma_prev) < c->mma_epsvalue;
        if (!inf.converged) {
            psf_status ms = mma_update(c, c->s, inf.f, c->dfds, inf.g, c->dgds, &inf.newton_steps);
            if (ms != PSF_OK && ms != PSF_NOT_CONVERGED) return ms;
        }
    } else {
        inf.converged = std::fabs(inf.f - c->oc_prev) / (inf.f + c->oc_prev) < 1.0e-5;
        if (!inf.converged) {
            PSF_CHECK(oc_update(c, c->s, c->dfds, c->dgds, P.oc_iota, P.oc_lmin, P.oc_lmax, P.oc_leps, P.oc_move,
                                P.vf, P.scale1, &inf.lambda));
            c->oc_prev = inf.f;
        }
    }
    PSF_CUDA(cudaEventRecord(ev[6], c->stream));
    PSF_CUDA(cudaEventSynchronize(ev[6]));
    for (int k = 0; k < 6; k++) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, ev[k], ev[k + 1]);
        inf.phase_seconds[k] = ms * 1e-3;
    }
    for (auto &e : ev) cudaEventDestroy(e);
    c->iter++;
    if (info) *info = inf;
    if (!std::isfinite(inf.f)) { set_error("non-finite compliance"); return PSF_NOT_FINITE; }
    return sst == PSF_OK ? PSF_OK : sst;
}

psf_status psf_simp_step_host(psf_ctx *h, const double *s_in, double *s_out, double *rho_out, double *u_out,
                              psf_iter_info *info) {
    CTX_CHECK(h);
    Ctx *c = &h->c;
    if (s_in) {
        // a non-finite design entry would run through the filter, the moduli and the solve as NaN
        // (the reference lets it); it is rejected before any device work
        for (long long e = 0; e < c->ne; e++)
            if (!std::isfinite(s_in[e])) {
                set_error("psf_simp_step_host: non-finite design entry " + std::to_string(e));
                return PSF_NOT_FINITE;
            }
        PSF_CHECK(h2d(c, c->s, s_in, sizeof(double) * c->ne));
    }
    // keep the pre-update densities for rho_out: psf_simp_step overwrites s only
    psf_status st = psf_simp_step(h, info);
    if (st != PSF_OK && st != PSF_NOT_CONVERGED && st != PSF_FELL_BACK) return st;
    if (s_out) PSF_CUDA(cudaMemcpyAsync(s_out, c->s, sizeof(double) * c->ne, cudaMemcpyDeviceToHost, c->stream));
    if (rho_out) PSF_CUDA(cudaMemcpyAsync(rho_out, c->rho, sizeof(double) * c->ne, cudaMemcpyDeviceToHost, c->stream));
    if (u_out) PSF_CUDA(cudaMemcpyAsync(u_out, c->un, sizeof(double) * c->ndofs, cudaMemcpyDeviceToHost, c->stream));
    PSF_CUDA(cudaStreamSynchronize(c->stream));
    return st;
}

psf_status psf_simp_fields(psf_ctx *h, double *s, double *rho, double *dfdrho, double *dfds, double *u_nodal) {
    CTX_CHECK(h);
    Ctx *c = &h->c;
    if (s) PSF_CUDA(cudaMemcpyAsync(s, c->s, sizeof(double) * c->ne, cudaMemcpyDeviceToHost, c->stream));
    if (rho) PSF_CUDA(cudaMemcpyAsync(rho, c->rho, sizeof(double) * c->ne, cudaMemcpyDeviceToHost, c->stream));
    if (dfdrho) PSF_CUDA(cudaMemcpyAsync(dfdrho, c->dfdrho, sizeof(double) * c->ne, cudaMemcpyDeviceToHost, c->stream));
    if (dfds) PSF_CUDA(cudaMemcpyAsync(dfds, c->dfds, sizeof(double) * c->ne, cudaMemcpyDeviceToHost, c->stream));
    if (u_nodal) PSF_CUDA(cudaMemcpyAsync(u_nodal, c->un, sizeof(double) * c->ndofs, cudaMemcpyDeviceToHost, c->stream));
    PSF_CUDA(cudaStreamSynchronize(c->stream));
    return PSF_OK;
}

psf_status psf_device_ptr(psf_ctx *h, const char *name, void **ptr) {
    CTX_CHECK(h);
    Ctx *c = &h->c;
    if (!name || !ptr) { set_error("psf_device_ptr: null argument"); return PSF_BAD_INPUT; }
    if (!strcmp(name, "s")) *ptr = c->s;
    else if (!strcmp(name, "rho")) *ptr = c->rho;
    else if (!strcmp(name, "E")) *ptr = c->E;
    else if (!strcmp(name, "dfdrho")) *ptr = c->dfdrho;
    else if (!strcmp(name, "dfds")) *ptr = c->dfds;
    else if (!strcmp(name, "u")) *ptr = c->un;
    else { set_error("psf_device_ptr: unknown name"); return PSF_BAD_INPUT; }
    return PSF_OK;
}

psf_status psf_sync(psf_ctx *h) {
    CTX_CHECK(h);
    PSF_CUDA(cudaStreamSynchronize(h->c.stream));
    return PSF_OK;
}

}  // extern "C"
