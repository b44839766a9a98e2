// Device-side building blocks shared by the trace_gb300 kernels: rounding-
// explicit float arithmetic, segment-length codecs, the parallel-beam ray
// tracer, and the (pixel, angle) ray window of the backward matrix.
#pragma once
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

namespace tg {

// ---- IEEE single operations that the compiler may not contract ------------
// The reference is compiled for x86-64 without FMA, so each of its float
// multiplies and adds rounds separately. These wrappers pin that.
__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }

// Kahan's compensated summation: s += x, with c carrying the low-order part
// the rounded additions lost (s - c is the corrected sum).
__device__ __forceinline__ void kahan_add(float& s, float& c, float x) {
  const float y = fsub(x, c);
  const float t = fadd(s, y);
  c = fsub(fsub(t, s), y);
  s = t;
}
__device__ __forceinline__ float fdiv(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ float fsqrt(float a) { return __fsqrt_rn(a); }

// ---- geometry ---------------------------------------------------------------
struct DevGeom {
  int C;        // detector columns == grid size g
  int P;        // angles
  int gpa;      // ray groups (of 32 columns) per angle
  int gpr;      // pixel groups (of 32 columns) per grid row
  float halfg;  // g/2 (exact)
  float mgrids; // (float)(g/2.) as trace_utils.cc:170
  float off;    // (1-C)/2 + mov: detector offset of column 0
  const float* yi;    // [C] source-frame offset per column (sirt.cc:129)
  const float* sinq;  // [P]
  const float* cosq;  // [P]
  const int* quad;    // [P]
};

// Grid line n (gridx == gridy), -g/2 + n: exact in float for g < 2^23.
__device__ __forceinline__ float grid_line(const DevGeom& G, int n) {
  return fsub((float)n, G.halfg);
}

// Streams the segments of ray (a, c) to emit(idx, len, len2, ix, iy) (ix,
// iy: column and row of cell idx = iy * g + ix) in the order of
// the reference tracer (trace_utils.cc:48-216 composed as sirt.cc:126-160).
// Returns the number of segments emitted.
//
// Crossings with horizontal grid lines ("a" points) and vertical grid lines
// ("b" points) are walked by two cursors over the crossings inside the open
// grid square; the a cursor runs backwards for quadrant-0 angles (the
// reversed a list of SortIntersectionPoints) and ties go to b.
//
// Each list's coordinate is a monotone function of the line index (rounded
// subtraction, multiplication by a constant and addition are monotone), so
// the crossings strictly inside the square are one contiguous run of line
// indices. The first one is found by bisection, and a cursor stops at the
// first crossing outside: the same points the reference's trim keeps,
// without evaluating the lines outside the square.

// First k in [0, n] with pred(k) for a predicate that is false up to some k
// and true from there on; n + 1 if none.
template <class Pred>
__device__ __forceinline__ int first_true(int n, Pred&& pred) {
  int lo = 0, hi = n + 1;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (pred(mid)) hi = mid;
    else lo = mid + 1;
  }
  return lo;
}

template <class Emit>
__device__ __forceinline__ int trace_ray(const DevGeom& G, int a, int c,
                                         Emit&& emit) {
  const int g = G.C;
  const float xi = -1e6f;
  const float yi = G.yi[c];
  const float s = G.sinq[a], co = G.cosq[a];
  const float srcx = fsub(fmul(xi, co), fmul(yi, s));
  const float srcy = fadd(fmul(xi, s), fmul(yi, co));
  const float detx = -fadd(fmul(xi, co), fmul(yi, s));
  const float dety = fadd(fmul(-xi, s), fmul(yi, co));
  const float slope = fdiv(fsub(srcy, dety), fsub(srcx, detx));
  const float islope = fdiv(1.0f, slope);
  const float lo = grid_line(G, 0), hi = grid_line(G, g);

  auto eval_a = [&](int n) { return fadd(fmul(islope, fsub(grid_line(G, n), srcy)), srcx); };
  auto eval_b = [&](int n) { return fadd(fmul(slope, fsub(grid_line(G, n), srcx)), srcy); };
  auto inside = [&](float v) { return v > lo && v < hi; };

  // a list: line na0 + k*da for k = 0..g, coordinate non-decreasing in k
  // when islope*da >= 0 (NaN and infinities at 0 and 90 degrees keep the
  // predicates below monotone; no such point is inside)
  const int da = G.quad[a] ? 1 : -1;
  const int na0 = G.quad[a] ? 0 : g;
  const bool a_up = da > 0 ? !signbit(islope) : signbit(islope);
  const int ka = first_true(g, [&](int k) {
    const float v = eval_a(na0 + k * da);
    return a_up ? v > lo : v < hi;
  });
  int na = na0 + ka * da;  // out of [0, g] when the list is exhausted
  float ax = 0.f;
  if (ka <= g) {
    ax = eval_a(na);
    if (!inside(ax)) na = -1;
  }
  // b list: line nb for nb = 0..g, non-decreasing when slope >= 0
  const bool b_up = !signbit(slope);
  int nb = first_true(g, [&](int k) {
    const float v = eval_b(k);
    return b_up ? v > lo : v < hi;
  });
  float by = 0.f;
  if (nb <= g) {
    by = eval_b(nb);
    if (!inside(by)) nb = g + 1;
  }

  int nseg = 0;
  bool have_prev = false;
  float px = 0.f, py = 0.f;
  for (;;) {
    const bool va = (na >= 0 && na <= g), vb = (nb <= g);
    if (!va && !vb) break;
    const bool take_a = va && (!vb || ax < grid_line(G, nb));
    float x, y;
    if (take_a) {
      x = ax;
      y = grid_line(G, na);
      na += da;
      if (na >= 0 && na <= g) {
        ax = eval_a(na);
        if (!inside(ax)) na = -1;  // the run of inside crossings ended
      }
    } else {
      x = grid_line(G, nb);
      y = by;
      ++nb;
      if (nb <= g) {
        by = eval_b(nb);
        if (!inside(by)) nb = g + 1;
      }
    }
    if (have_prev) {
      const float dx = fsub(x, px), dy = fsub(y, py);
      // (x + px)/2. in the reference: float sum, exact halving
      const float midx = fmul(fadd(x, px), 0.5f);
      const float midy = fmul(fadd(y, py), 0.5f);
      const float len2 = fadd(fmul(dx, dx), fmul(dy, dy));
      const float len = fsqrt(len2);
      const int ix = __float2int_rz(fadd(midx, G.mgrids));
      const int iy = __float2int_rz(fadd(midy, G.mgrids));
      const int idx = ix + iy * g;
      // A stray segment whose cell index falls outside the grid (the
      // reference indexes its arrays out of bounds there) is dropped.
      if ((unsigned)idx < (unsigned)g * (unsigned)g) {
        // the cell idx names (a stray segment's column can lie outside the
        // grid while its index is inside: then idx, not ix, decides)
        if ((unsigned)ix < (unsigned)g) emit(idx, len, len2, ix, iy);
        else emit(idx, len, len2, idx % g, idx / g);
        ++nseg;
      }
    }
    px = x;
    py = y;
    have_prev = true;
  }
  return nseg;
}

// Column and row of cell idx in [0, g*g), g < 2^23, without an integer
// division: the float quotient estimate is off by at most one (its relative
// error is a few 2^-24, i.e. below 1/g in absolute terms) and is corrected
// exactly from the remainder.
__device__ __forceinline__ void cell_xy(int idx, int g, float inv_g, int& ix, int& iy) {
  int q = __float2int_rz(__fmul_rn(__int2float_rn(idx), inv_g));
  int rem = idx - q * g;
  if (rem < 0) {
    --q;
    rem += g;
  } else if (rem >= g) {
    ++q;
    rem -= g;
  }
  ix = rem;
  iy = q;
}

// First detector column of the two-column window that holds every ray
// crossing pixel (x, y) at angle a:
//   c0 = round(v + 1/2) (about floor(v) + 1),  v = -sin*x + cos*y + D,
//   D  = (g/2 - 1/2)(sin - cos) - (|sin| + |cos|)/2 - 1/4 - off,
// i.e. the detector coordinate of the pixel centre minus half the pixel's
// footprint (|sin|+|cos| <= sqrt(2) wide) minus a 1/4-column margin for the
// reference's float jitter: the crossing columns lie strictly inside
// (v + 0.19, v + 1.78), so {c0, c0 + 1} holds all of them (also when v is
// an integer and the rounding tie goes either way). coef = {-sin, cos,
// D + 1/2} per angle (host-computed); the rounding is one add of the exact
// constant 1.5 * 2^23 (valid for |v| < 2^22) instead of two conversions.
// Construction and use call this same function, so they agree bit for bit.
__device__ __forceinline__ int window_c0(float4 coef, float xf, float yf) {
  const float v = __fmaf_rn(coef.y, yf, __fmaf_rn(coef.x, xf, coef.z));
  return __float_as_int(__fadd_rn(v, 12582912.0f)) - 0x4B400000;
}

// Backward-matrix pair index (two slots) of angle a, tile t, lane l: angles
// in groups of four per lane, so one 16-byte load brings four angles.
__device__ __forceinline__ int64_t dense_pair(int ntiles, int a, int t, int l) {
  return (((int64_t)(a >> 2) * ntiles + t) * 32 + l) * 4 + (a & 3);
}

// Exact float value of a 16-bit integer (magic-number conversion).
__device__ __forceinline__ float u16_to_float(uint32_t q) {
  return __uint_as_float(0x4B000000u | q) - 8388608.0f;
}

// Backward-matrix position of pixel (x, y): tiles of 32 pixels, 2^tw_shift
// wide and 2^(5 - tw_shift) high (16x2, 8x4 or 4x8), one warp per tile,
// tiles row-major; entry (angle, tile, lane) is one 32-lane row.
__device__ __forceinline__ void pixel_tile(int x, int y, int tiles_x, int tw_shift,
                                           int* tile, int* lane) {
  const int th_shift = 5 - tw_shift;
  *tile = (y >> th_shift) * tiles_x + (x >> tw_shift);
  *lane = ((y & ((1 << th_shift) - 1)) << tw_shift) | (x & ((1 << tw_shift) - 1));
}

// The pixel of lane `lane` in tile `tile` (inverse of pixel_tile).
__device__ __forceinline__ void tile_pixel(int tile, int lane, int tiles_x, int tw_shift,
                                           int* x, int* y) {
  *x = ((tile % tiles_x) << tw_shift) + (lane & ((1 << tw_shift) - 1));
  *y = ((tile / tiles_x) << (5 - tw_shift)) + (lane >> tw_shift);
}

// ---- segment-length storage -------------------------------------------------
enum LenKind { LK_F32 = 0, LK_BF16 = 1, LK_F16 = 2, LK_U16 = 3 };

template <int LK>
__device__ __forceinline__ float decode_len(uint16_t v, float inv_scale) {
  if constexpr (LK == LK_BF16) return __bfloat162float(__ushort_as_bfloat16(v));
  else if constexpr (LK == LK_F16) return __half2float(__ushort_as_half(v));
  else return u16_to_float(v) * inv_scale;  // exact conversion, no I2F
}

// 16-bit codes; `kind` is warp-uniform so the switch does not diverge.
__device__ __forceinline__ float decode16(uint16_t v, int kind, float inv_scale) {
  if (kind == LK_BF16) return __bfloat162float(__ushort_as_bfloat16(v));
  if (kind == LK_F16) return __half2float(__ushort_as_half(v));
  return u16_to_float(v) * inv_scale;
}
__device__ __forceinline__ uint16_t encode16(float x, int kind, float scale) {
  if (kind == LK_BF16) return __bfloat16_as_ushort(__float2bfloat16_rn(x));
  if (kind == LK_F16) return __half_as_ushort(__float2half_rn(x));
  float q = rintf(x * scale);
  q = fminf(fmaxf(q, 0.f), 65535.f);
  return (uint16_t)q;
}

// ---- k-slice vector loads ----------------------------------------------------
template <int K>
struct Vec {
  float v[K];
};

template <int K>
__device__ __forceinline__ Vec<K> load_vec(const float* p) {
  Vec<K> r;
  if constexpr (K == 1) {
    r.v[0] = __ldg(p);
  } else if constexpr (K == 2) {
    float2 t = __ldg(reinterpret_cast<const float2*>(p));
    r.v[0] = t.x;
    r.v[1] = t.y;
  } else if constexpr (K == 8 || K == 16) {
    // 256-bit read-only loads: a single L1 sector lookup per 8 slices
#pragma unroll
    for (int j = 0; j < K; j += 8)
      asm("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
          : "=f"(r.v[j]), "=f"(r.v[j + 1]), "=f"(r.v[j + 2]), "=f"(r.v[j + 3]),
            "=f"(r.v[j + 4]), "=f"(r.v[j + 5]), "=f"(r.v[j + 6]), "=f"(r.v[j + 7])
          : "l"(p + j));
  } else {
#pragma unroll
    for (int j = 0; j < K; j += 4) {
      float4 t = __ldg(reinterpret_cast<const float4*>(p + j));
      r.v[j] = t.x;
      r.v[j + 1] = t.y;
      r.v[j + 2] = t.z;
      r.v[j + 3] = t.w;
    }
  }
  return r;
}

template <int K>
__device__ __forceinline__ void store_vec(float* p, const Vec<K>& r) {
  if constexpr (K == 1) {
    p[0] = r.v[0];
  } else if constexpr (K == 2) {
    *reinterpret_cast<float2*>(p) = make_float2(r.v[0], r.v[1]);
  } else {
#pragma unroll
    for (int j = 0; j < K; j += 4)
      *reinterpret_cast<float4*>(p + j) =
          make_float4(r.v[j], r.v[j + 1], r.v[j + 2], r.v[j + 3]);
  }
}

// K floats read once (streaming loads: evict-first).
template <int K>
__device__ __forceinline__ Vec<K> load_vec_cs(const float* p) {
  Vec<K> r;
  if constexpr (K == 1) {
    r.v[0] = __ldcs(p);
  } else if constexpr (K == 2) {
    const float2 t = __ldcs(reinterpret_cast<const float2*>(p));
    r.v[0] = t.x;
    r.v[1] = t.y;
  } else {
#pragma unroll
    for (int j = 0; j < K; j += 4) {
      const float4 t = __ldcs(reinterpret_cast<const float4*>(p + j));
      r.v[j] = t.x;
      r.v[j + 1] = t.y;
      r.v[j + 2] = t.z;
      r.v[j + 3] = t.w;
    }
  }
  return r;
}

// acc[j] += l * v[j] for the K slices (fast mode). Scalar FMAs: the paired
// FP32 FMA of sm_100 (__ffma2_rn) measured slower here - packing the
// operands into register pairs costs more moves than it saves issue slots.
template <int K>
__device__ __forceinline__ void fma_slices(float (&acc)[K], float l, const float (&v)[K]) {
#pragma unroll
  for (int j = 0; j < K; ++j) acc[j] = fmaf(v[j], l, acc[j]);
}

// ---- k-slice vectors stored as IEEE halves (16-bit gather operands) ------
__device__ __forceinline__ float2 half2_bits_to_float2(uint32_t w) {
  __half2 h;
  memcpy(&h, &w, 4);
  return __half22float2(h);
}
__device__ __forceinline__ uint32_t float2_to_half2_bits(float a, float b) {
  const __half2 h = __floats2half2_rn(a, b);
  uint32_t w;
  memcpy(&w, &h, 4);
  return w;
}

// K halves (2K bytes, one aligned load) -> K floats. SHARED: plain load
// (shared memory), else a read-only global load.
template <int K, bool SHARED>
__device__ __forceinline__ Vec<K> load_hvec(const __half* p) {
  Vec<K> r;
  if constexpr (K == 1) {
    r.v[0] = __half2float(SHARED ? *p : __ldg(p));
  } else if constexpr (K == 2) {
    const uint32_t w = SHARED ? *reinterpret_cast<const uint32_t*>(p)
                              : __ldg(reinterpret_cast<const unsigned int*>(p));
    const float2 f = half2_bits_to_float2(w);
    r.v[0] = f.x;
    r.v[1] = f.y;
  } else if constexpr (K == 4) {
    const uint2 w = SHARED ? *reinterpret_cast<const uint2*>(p)
                           : __ldg(reinterpret_cast<const uint2*>(p));
    const float2 a = half2_bits_to_float2(w.x), b = half2_bits_to_float2(w.y);
    r.v[0] = a.x; r.v[1] = a.y; r.v[2] = b.x; r.v[3] = b.y;
  } else if constexpr (K == 8) {
    const uint4 w = SHARED ? *reinterpret_cast<const uint4*>(p)
                           : __ldg(reinterpret_cast<const uint4*>(p));
    const uint32_t ws[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const float2 f = half2_bits_to_float2(ws[i]);
      r.v[2 * i] = f.x;
      r.v[2 * i + 1] = f.y;
    }
  } else {  // 16: 32 bytes
    uint32_t ws[8];
    if constexpr (SHARED) {
      const uint4 a = reinterpret_cast<const uint4*>(p)[0];
      const uint4 b = reinterpret_cast<const uint4*>(p)[1];
      ws[0] = a.x; ws[1] = a.y; ws[2] = a.z; ws[3] = a.w;
      ws[4] = b.x; ws[5] = b.y; ws[6] = b.z; ws[7] = b.w;
    } else {
      asm("ld.global.nc.v8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
          : "=r"(ws[0]), "=r"(ws[1]), "=r"(ws[2]), "=r"(ws[3]), "=r"(ws[4]),
            "=r"(ws[5]), "=r"(ws[6]), "=r"(ws[7])
          : "l"(p));
    }
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const float2 f = half2_bits_to_float2(ws[i]);
      r.v[2 * i] = f.x;
      r.v[2 * i + 1] = f.y;
    }
  }
  return r;
}

// K floats -> K halves (round to nearest), one aligned store.
template <int K>
__device__ __forceinline__ void store_hvec(__half* p, const Vec<K>& r) {
  if constexpr (K == 1) {
    *p = __float2half_rn(r.v[0]);
  } else if constexpr (K == 2) {
    *reinterpret_cast<uint32_t*>(p) = float2_to_half2_bits(r.v[0], r.v[1]);
  } else if constexpr (K == 4) {
    *reinterpret_cast<uint2*>(p) = make_uint2(float2_to_half2_bits(r.v[0], r.v[1]),
                                              float2_to_half2_bits(r.v[2], r.v[3]));
  } else {  // 8 or 16: one 16-byte store per 8 slices
#pragma unroll
    for (int j = 0; j < K; j += 8)
      *reinterpret_cast<uint4*>(p + j) = make_uint4(
          float2_to_half2_bits(r.v[j], r.v[j + 1]), float2_to_half2_bits(r.v[j + 2], r.v[j + 3]),
          float2_to_half2_bits(r.v[j + 4], r.v[j + 5]), float2_to_half2_bits(r.v[j + 6], r.v[j + 7]));
  }
}

__device__ __forceinline__ int warp_max_i(int v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
__device__ __forceinline__ float warp_max_f(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

}  // namespace tg
