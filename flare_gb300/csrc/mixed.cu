// Mixed-precision kernel stage.
#include "fgb_internal.h"
#include "fgb_kernels.h"
#include "fgb_model.h"

namespace fgb {
int kernel_stage_mixed(fgb_model_s *, int, const std::vector<int> &, bool,
                       bool, double *, double *, double *, cudaStream_t) {
  set_error("mixed precision stage not built yet");
  return FGB_ENOTSUP;
}
}  // namespace fgb
