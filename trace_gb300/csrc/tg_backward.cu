// Backprojection entry point: dispatch on the slices per pass (kernels in
// tg_backward.cuh; K = 8 and K = 16 are compiled in tg_backward_k8.cu and
// tg_backward_k16.cu).
#include "tg_backward.cuh"

namespace tg {

TG_BACKWARD_ENTRY(1)
TG_BACKWARD_ENTRY(2)
TG_BACKWARD_ENTRY(4)

void launch_backward(const IterArgs& A, int batch, const float* recon_cur,
                     float* recon_next, const float* upd, float* rep_num,
                     int epi, cudaStream_t st) {
  switch (A.K) {
    case 1: launch_backward_k1(A, batch, recon_cur, recon_next, upd, rep_num, epi, st); break;
    case 2: launch_backward_k2(A, batch, recon_cur, recon_next, upd, rep_num, epi, st); break;
    case 4: launch_backward_k4(A, batch, recon_cur, recon_next, upd, rep_num, epi, st); break;
    case 8: launch_backward_k8(A, batch, recon_cur, recon_next, upd, rep_num, epi, st); break;
    default: launch_backward_k16(A, batch, recon_cur, recon_next, upd, rep_num, epi, st); break;
  }
}

}  // namespace tg
