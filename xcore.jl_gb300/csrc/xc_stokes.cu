// Stokes saddle-point solve of fluidmech! (placeholder until the solver lands).
#include "xc_internal.cuh"

struct StokesWork { int dummy; };

int stokes_create(xc_ctx* c) { c->stokes = nullptr; return XC_OK; }
void stokes_destroy(xc_ctx* c) { c->stokes = nullptr; }
int fluidmech_impl(xc_ctx* c, const double coefs[6], double dt, const xc_solver_opts* opts,
                   xc_solver_stats* stats, const MmsData* mms) {
  (void)c; (void)coefs; (void)dt; (void)opts; (void)stats; (void)mms;
  xc_set_error("fluidmech: Stokes solver not built");
  return XC_BAD_ARG;
}
