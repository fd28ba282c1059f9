// film.cu -- Crank-Nicolson / ADI film and brush propagators (in progress).
#include "internal.h"

int film_create(adscf_ctx* ctx) {
  return set_err(ctx, ADSCF_E_ARG, "film and brush geometries are not built yet");
}
void film_destroy(adscf_ctx*) {}
int film_enqueue_propagate(adscf_ctx* ctx, const double*) {
  return set_err(ctx, ADSCF_E_STATE, "film geometry not built");
}
int film_step_single(adscf_ctx* ctx, double*, const double*, double) {
  return set_err(ctx, ADSCF_E_STATE, "film geometry not built");
}
int film_enqueue_chains(adscf_ctx* ctx, const double*) {
  return set_err(ctx, ADSCF_E_STATE, "film geometry not built");
}
int film_enqueue_contour(adscf_ctx* ctx) {
  return set_err(ctx, ADSCF_E_STATE, "film geometry not built");
}
