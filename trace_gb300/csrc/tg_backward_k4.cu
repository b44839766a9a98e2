// Backprojection instances for 4 slices per pass (see tg_backward.cuh).
#include "tg_backward.cuh"

namespace tg {

TG_BACKWARD_ENTRY(4)

}  // namespace tg
