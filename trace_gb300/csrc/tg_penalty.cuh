// The 8-neighbour penalty of PML (src/pml/pml.cc:25-201) and the adaptive
// in-plane + axial penalty of APMLR (src/apmlr/apmlr.cc:28-982), evaluated per
// pixel. The reference walks each border region with its own loop; here a
// pixel looks up its region's neighbour list. Within a pixel the neighbours
// are visited in the reference's order and every operation is rounded as the
// reference rounds it, so F and G are bit-identical.
#pragma once
#include "tg_device.cuh"

namespace tg {

struct PenaltyWeights {
  float pml[3][2];        // [interior|edge|corner][orthogonal|diagonal]
  float apmlr[3][2][3];   // [region][axial neighbours 2|1][orth, diag, axial]
  float beta, beta1, delta, delta1;
};

// In-plane neighbour classes: 0 interior, 1 top (y=0), 2 bottom (y=g-1),
// 3 left (x=0), 4 right (x=g-1), 5 top-left, 6 top-right, 7 bottom-left,
// 8 bottom-right. kind: 0 orthogonal, 1 diagonal.
struct NbrTable {
  int8_t n[9];
  int8_t dx[9][8], dy[9][8], kind[9][8];
};

__constant__ NbrTable c_nbr = {
    {8, 5, 5, 5, 5, 3, 3, 3, 3},
    {{1, -1, 0, 0, 1, -1, 1, -1},
     {1, -1, 0, 1, -1},
     {1, -1, 0, 1, -1},
     {1, 0, 0, 1, 1},
     {-1, 0, 0, -1, -1},
     {1, 0, 1},
     {-1, 0, -1},
     {1, 0, 1},
     {-1, 0, -1}},
    {{0, 0, 1, -1, 1, 1, -1, -1},
     {0, 0, 1, 1, 1},
     {0, 0, -1, -1, -1},
     {0, 1, -1, 1, -1},
     {0, 1, -1, 1, -1},
     {0, 1, 1},
     {0, 1, 1},
     {0, -1, -1},
     {0, -1, -1}},
    {{0, 0, 0, 0, 1, 1, 1, 1},
     {0, 0, 0, 1, 1},
     {0, 0, 0, 1, 1},
     {0, 0, 0, 1, 1},
     {0, 0, 0, 1, 1},
     {0, 0, 1},
     {0, 0, 1},
     {0, 0, 1},
     {0, 0, 1}}};

__device__ __forceinline__ int nbr_class(int x, int y, int g, int* region) {
  const bool l = x == 0, r = x == g - 1, t = y == 0, b = y == g - 1;
  if ((l || r) && (t || b)) {
    *region = 2;
    return t ? (l ? 5 : 6) : (l ? 7 : 8);
  }
  if (l || r || t || b) {
    *region = 1;
    return t ? 1 : b ? 2 : l ? 3 : 4;
  }
  *region = 0;
  return 0;
}

// F and G (before G += sum of lengths) of one pixel.
//   rec(dx, dy, dz): the iteration's input reconstruction at the neighbour
//   offset (dz = axial slice offset, APMLR only).
//   up / down: APMLR axial neighbours at +1 / -1 slice present.
template <class Rec>
__device__ __forceinline__ void penalty_fg(bool apmlr, const PenaltyWeights& W,
                                           int x, int y, int g, int up,
                                           int down, Rec&& rec, float& F,
                                           float& G) {
  int region;
  const int cls = nbr_class(x, y, g, &region);
  const float r0 = rec(0, 0, 0);
  float f = 0.f, gg = 0.f;
  const int n = c_nbr.n[cls];
  if (!apmlr) {
    const float twob = fmul(2.f, W.beta);
    for (int q = 0; q < n; ++q) {
      const float w = W.pml[region][c_nbr.kind[cls][q]];
      const float rq = rec(c_nbr.dx[cls][q], c_nbr.dy[cls][q], 0);
      const float tw = fmul(twob, w);
      f = fadd(f, tw);
      gg = fsub(gg, fmul(tw, fadd(r0, rq)));
    }
  } else {
    const int nax = up + down;
    const float* w = W.apmlr[region][nax == 2 ? 0 : 1];
    const float twob = fmul(2.f, W.beta), twob1 = fmul(2.f, W.beta1);
    for (int q = 0; q < n; ++q) {
      const float wq = w[c_nbr.kind[cls][q]];
      const float rq = rec(c_nbr.dx[cls][q], c_nbr.dy[cls][q], 0);
      const float mg = fadd(r0, rq), rg = fsub(r0, rq);
      const float gam = fdiv(1.f, fadd(1.f, fabsf(fdiv(rg, W.delta))));
      const float t = fmul(fmul(twob, wq), gam);
      f = fadd(f, t);
      gg = fsub(gg, fmul(t, mg));
    }
    for (int q = 0; q < 2; ++q) {
      if (q == 0 ? !up : !down) continue;
      const float rq = rec(0, 0, q == 0 ? 1 : -1);
      const float mg = fadd(r0, rq), rg = fsub(r0, rq);
      const float gam = fdiv(1.f, fadd(1.f, fabsf(fdiv(rg, W.delta1))));
      const float t = fmul(fmul(twob1, w[2]), gam);
      f = fadd(f, t);
      gg = fsub(gg, fmul(t, mg));
    }
  }
  F = f;
  G = gg;
}

// Closed-form root of UpdateRecon (pml.cc:18-20, apmlr.cc:20-22).
__device__ __forceinline__ float penalised_root(float F, float G, float num) {
  const float disc = fsub(fmul(G, G), fmul(fmul(8.f, num), F));
  return fdiv(fadd(-G, fsqrt(disc)), fmul(4.f, F));
}

}  // namespace tg
