// ttfld_unet.cu -- learned initial guess for SOLVE_WITH_SOR (no reference
// counterpart).  Placeholder until the conv-net kernels land: no model can
// be loaded, so a learned guess request reports TTFLD_E_NOMODEL.
#include "ttfld_internal.cuh"

namespace ttfld {
int unet_guess(ttfld_ctx*, double*, double*) { return TTFLD_E_NOMODEL; }
void unet_free(ttfld_ctx*) {}
}  // namespace ttfld

extern "C" {
int ttfld_guess_load(ttfld_ctx* c, const void*, size_t) { return c ? TTFLD_E_NOMODEL : TTFLD_E_ARGS; }
int ttfld_guess_save(ttfld_ctx* c, void*, size_t, size_t* needed) {
  if (needed) *needed = 0;
  return c ? TTFLD_E_NOMODEL : TTFLD_E_ARGS;
}
}
