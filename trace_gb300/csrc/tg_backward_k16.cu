// Backprojection instances for 16 slices per pass (see tg_backward.cuh).
#include "tg_backward.cuh"

namespace tg {

TG_BACKWARD_ENTRY(16)

}  // namespace tg
