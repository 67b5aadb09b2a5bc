// psf_mg.cu -- multigrid-preconditioned mixed-precision solver (placeholder until built).
#include "psf_internal.cuh"

namespace psf {
psf_status mg_solve_ir(Ctx *c, int itmax, double eps, bool warm, psf_solve_info *info) {
    (void)c; (void)itmax; (void)eps; (void)warm; (void)info;
    set_error("multigrid solver not available in this build");
    return PSF_BAD_INPUT;
}
psf_status mg_free(Ctx *c) { (void)c; return PSF_OK; }
psf_status learned_free(Ctx *c) { (void)c; return PSF_OK; }
}  // namespace psf
