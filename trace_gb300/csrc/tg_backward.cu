// Backprojection entry point: dispatch on the slices per pass (kernels in
// tg_backward.cuh; K = 4, 8 and 16 are compiled in tg_backward_k4.cu,
// tg_backward_k8.cu and tg_backward_k16.cu).
#include "tg_backward.cuh"

namespace tg {

TG_BACKWARD_ENTRY(1)
TG_BACKWARD_ENTRY(2)

void launch_backward_multi(const BackItem* items, int n, int64_t blocks, int K,
                           int dlen_kind, int pen, int fh, int comp, cudaStream_t st) {
  switch (K) {
    case 1: launch_backward_multi_k1(items, n, blocks, dlen_kind, pen, fh, comp, st); break;
    case 2: launch_backward_multi_k2(items, n, blocks, dlen_kind, pen, fh, comp, st); break;
    case 4: launch_backward_multi_k4(items, n, blocks, dlen_kind, pen, fh, comp, st); break;
    case 8: launch_backward_multi_k8(items, n, blocks, dlen_kind, pen, fh, comp, st); break;
    default: launch_backward_multi_k16(items, n, blocks, dlen_kind, pen, fh, comp, st); break;
  }
}

int64_t backward_blocks(const IterArgs& A) { return (A.M.ntiles + kWarps - 1) / kWarps; }

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
