// Backprojection instances for 8 slices per pass (see tg_backward.cuh).
#include "tg_backward.cuh"

namespace tg {

TG_BACKWARD_ENTRY(8)

}  // namespace tg
