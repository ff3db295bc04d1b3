// Precision form of MDFL Sweby: FP32 fluxes and limiters, FP64 tracer state.
#include "internal.h"

namespace mom5 {

int launch_mdfl_mixed(mom5gpu_domain* d, int n_first, int ntr, int taum1, int tau, int taup1, double dtime,
                      bool fused_update) {
  (void)n_first; (void)ntr; (void)taum1; (void)tau; (void)taup1; (void)dtime; (void)fused_update;
  return fail(d, MOM5GPU_EUNSUPPORTED, "precision form not built yet");
}

}  // namespace mom5
