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

// Rounded arithmetic for the penalty in the reconstruction's type: float
// keeps the reference's individually rounded single operations, double is
// the FP64 mode.
template <class T> struct Ar;
template <> struct Ar<float> {
  static __device__ __forceinline__ float mul(float a, float b) { return fmul(a, b); }
  static __device__ __forceinline__ float add(float a, float b) { return fadd(a, b); }
  static __device__ __forceinline__ float sub(float a, float b) { return fsub(a, b); }
  static __device__ __forceinline__ float div(float a, float b) { return fdiv(a, b); }
  static __device__ __forceinline__ float sqrt(float a) { return fsqrt(a); }
  static __device__ __forceinline__ float abs(float a) { return fabsf(a); }
};
template <> struct Ar<double> {
  static __device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
  static __device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
  static __device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
  static __device__ __forceinline__ double div(double a, double b) { return __ddiv_rn(a, b); }
  static __device__ __forceinline__ double sqrt(double a) { return __dsqrt_rn(a); }
  static __device__ __forceinline__ double abs(double a) { return ::fabs(a); }
};

// F and G (before G += sum of lengths) of one pixel.
//   rec(dx, dy, dz): the iteration's input reconstruction at the neighbour
//   offset (dz = axial slice offset, APMLR only).
//   up / down: APMLR axial neighbours at +1 / -1 slice present.
template <class T, class Rec>
__device__ __forceinline__ void penalty_fg(bool apmlr, const PenaltyWeights& W,
                                           int x, int y, int g, int up,
                                           int down, Rec&& rec, T& F, T& G) {
  using A = Ar<T>;
  int region;
  const int cls = nbr_class(x, y, g, &region);
  const T r0 = rec(0, 0, 0);
  T f = 0, gg = 0;
  const int n = c_nbr.n[cls];
  if (!apmlr) {
    const T twob = A::mul(T(2), T(W.beta));
    for (int q = 0; q < n; ++q) {
      const T w = W.pml[region][c_nbr.kind[cls][q]];
      const T rq = rec(c_nbr.dx[cls][q], c_nbr.dy[cls][q], 0);
      const T tw = A::mul(twob, w);
      f = A::add(f, tw);
      gg = A::sub(gg, A::mul(tw, A::add(r0, rq)));
    }
  } else {
    const int nax = up + down;
    const float* w = W.apmlr[region][nax == 2 ? 0 : 1];
    const T twob = A::mul(T(2), T(W.beta)), twob1 = A::mul(T(2), T(W.beta1));
    for (int q = 0; q < n; ++q) {
      const T wq = w[c_nbr.kind[cls][q]];
      const T rq = rec(c_nbr.dx[cls][q], c_nbr.dy[cls][q], 0);
      const T mg = A::add(r0, rq), rg = A::sub(r0, rq);
      const T gam = A::div(T(1), A::add(T(1), A::abs(A::div(rg, T(W.delta)))));
      const T t = A::mul(A::mul(twob, wq), gam);
      f = A::add(f, t);
      gg = A::sub(gg, A::mul(t, mg));
    }
    for (int q = 0; q < 2; ++q) {
      if (q == 0 ? !up : !down) continue;
      const T rq = rec(0, 0, q == 0 ? 1 : -1);
      const T mg = A::add(r0, rq), rg = A::sub(r0, rq);
      const T gam = A::div(T(1), A::add(T(1), A::abs(A::div(rg, T(W.delta1)))));
      const T t = A::mul(A::mul(twob1, T(w[2])), gam);
      f = A::add(f, t);
      gg = A::sub(gg, A::mul(t, mg));
    }
  }
  F = f;
  G = gg;
}

// Closed-form root of UpdateRecon (pml.cc:18-20, apmlr.cc:20-22): the
// positive root of 2F x^2 + G x + num = 0, in the reference's form.
template <class T>
__device__ __forceinline__ T penalised_root(T F, T G, T num) {
  using A = Ar<T>;
  const T disc = A::sub(A::mul(G, G), A::mul(A::mul(T(8), num), F));
  return A::div(A::add(-G, A::sqrt(disc)), A::mul(T(4), F));
}

// The same root without cancellation. With a small penalty, G (about the
// total length through the pixel, ~P) dwarfs the root, and -G + sqrt(...)
// in float keeps only a few digits (relative error ~ eps * G / root, about
// 3e-4 at 2048 x 1500 with beta = 0.05). Multiplying through by
// G + sqrt(...) gives -2 num / (G + sqrt(...)), exact in form for G >= 0.
__device__ __forceinline__ float penalised_root_stable(float F, float G,
                                                       float num) {
  const float s = sqrtf(fmaf(G, G, -8.f * num * F));
  return G >= 0.f ? (-2.f * num) / (G + s) : (s - G) / (4.f * F);
}

}  // namespace tg
