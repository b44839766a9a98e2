// Backprojection (pixel-driven) with the algorithms' UpdateRecon fused into
// its epilogue.
//
// One thread per pixel, one warp per 32-pixel tile (8x4 by default; 16x2
// or 4x8 as the plan chooses), eight tiles per block.
// For every angle a thread reads the lengths of the (at most two) rays
// through its pixel - one contiguous 32-lane row of the backward matrix per
// warp - and gathers those rays' factors. The sum over angles in column
// order is the reference's replica[2p] accumulation (sirt.cc:58,
// mlem.cc:58, pml.cc:243); the total length per pixel (replica[2p+1]) is a
// per-geometry constant. No atomics: every pixel is owned by one thread.
// The tile shape keeps the rays a warp touches at one angle within a short
// detector window, so the factor gathers share L1 sectors.
//
// With half factors (fast mode, ratio algorithms) each factor is read as the
// half (factor - 1) - half the gather bytes - and sum(len * factor) is
// rebuilt as W + sum(len * (factor - 1)), the products taken by
// mixed-precision FMAs straight from the halves; the plan then stores the
// backward matrix's lengths as halves too (MatrixDev::dlen_kind), so both
// FMA operands come from memory as they are.
//
// Epilogue per slice: SIRT recon += num/W (sirt.cc:21-33), MLEM
// recon *= num/W (mlem.cc:21-34), PML/APMLR the closed-form root with the
// penalty's F and G (pml.cc:3-23, apmlr.cc:3-26), written to the other
// reconstruction buffer so neighbours read by the stencil stay unmodified.
#pragma once
#include "tg_kernels.cuh"

namespace tg {

namespace {

constexpr int kWarps = 8;
constexpr int kBlock = kWarps * 32;
constexpr int kCoefChunk = 512;  // angles of window coefficients per stage
// Resident blocks per SM the register allocation is sized for (48 registers
// a thread at 5): at 6 the 8-slice variants spill inside the angle loop.
constexpr int kMinBlocks = 5;
constexpr int kMinBlocks16 = 4;  // 16 slices per pass: 16 accumulators more

// Four angles of one lane's backward-matrix entries: 16 bytes for 16-bit
// codes (two per angle), 32 bytes for floats. The entries of angles
// 4i..4i+3, tile t, lane l are the 16-byte words (i*ntiles + t)*32 + l
// (times two for floats): one contiguous 512-byte row per warp.
template <int LK>
struct Quad {
  static constexpr int kWords = LK == LK_F32 ? 2 : 1;
  uint4 w[kWords];
};

template <int LK>
__device__ __forceinline__ void load_quad(const uint4* p, Quad<LK>& q) {
#pragma unroll
  for (int i = 0; i < Quad<LK>::kWords; ++i) q.w[i] = __ldcs(p + i);
}

__device__ __forceinline__ uint32_t pick(const uint4& v, int i) {
  return i == 0 ? v.x : i == 1 ? v.y : i == 2 ? v.z : v.w;
}

// Lengths of angle j of the quad. SCALED: 16-bit fixed-point codes are
// returned unscaled (the scale is applied once to the pixel's sums).
template <int LK, bool SCALED>
__device__ __forceinline__ void quad_pair(const Quad<LK>& q, int j, float inv_scale,
                                          float& l0, float& l1, bool& h0, bool& h1) {
  if constexpr (LK == LK_F32) {
    const uint32_t a = pick(q.w[j >> 1], (j & 1) * 2), b = pick(q.w[j >> 1], (j & 1) * 2 + 1);
    // a stored -0.0f marks a zero-length segment (present, adds 0*factor)
    h0 = a != 0u;
    h1 = b != 0u;
    l0 = __uint_as_float(a);
    l1 = __uint_as_float(b);
  } else {
    const uint32_t w = pick(q.w[0], j);
    h0 = (w & 0xffffu) != 0u;
    h1 = (w >> 16) != 0u;
    if constexpr (LK == LK_U16 && SCALED) {
      l0 = u16_to_float(w & 0xffffu);
      l1 = u16_to_float(w >> 16);
    } else {
      l0 = decode_len<LK>((uint16_t)(w & 0xffffu), inv_scale);
      l1 = decode_len<LK>((uint16_t)(w >> 16), inv_scale);
    }
  }
}

// acc[j] += l * d[j] for K halves d (one aligned load) with the
// mixed-precision FMA of sm_100 and later (f16 x f16 + f32 -> f32, exact
// product, one rounding): no half-to-float conversions. The length is
// rounded to a half; the epilogue adds, and normalises by, the total of the
// same half-rounded lengths (Wh), so the backprojection uses one consistent
// set of lengths: sum(lh * factor) = Wh + sum(lh * (factor - 1)).
template <int K>
__device__ __forceinline__ void fma_halves(float (&acc)[K], float l, const __half* p) {
  const unsigned short lh = __half_as_ushort(__float2half_rn(l));
  if constexpr (K == 1) {
    const unsigned short d = __ldg(reinterpret_cast<const unsigned short*>(p));
    asm("fma.rn.f32.f16 %0, %1, %2, %0;" : "+f"(acc[0]) : "h"(d), "h"(lh));
  } else {
    uint32_t ws[K / 2];
    if constexpr (K == 2) {
      ws[0] = __ldg(reinterpret_cast<const unsigned int*>(p));
    } else if constexpr (K == 4) {
      const uint2 w = __ldg(reinterpret_cast<const uint2*>(p));
      ws[0] = w.x;
      ws[1] = w.y;
    } else {
#pragma unroll
      for (int b = 0; b < K / 8; ++b) {
        const uint4 w = __ldg(reinterpret_cast<const uint4*>(p) + b);
        ws[4 * b] = w.x;
        ws[4 * b + 1] = w.y;
        ws[4 * b + 2] = w.z;
        ws[4 * b + 3] = w.w;
      }
    }
#pragma unroll
    for (int i = 0; i < K / 2; ++i)
      asm("{ .reg .b16 lo, hi; mov.b32 {lo, hi}, %2; fma.rn.f32.f16 %0, lo, %3, %0;"
          " fma.rn.f32.f16 %1, hi, %3, %1; }"
          : "+f"(acc[2 * i]), "+f"(acc[2 * i + 1])
          : "r"(ws[i]), "h"(lh));
  }
}

// K halves as K/2 32-bit words (one aligned load), for the pipelined loop.
template <int K>
__device__ __forceinline__ void load_hwords(uint32_t (&w)[K / 2], const __half* p) {
  if constexpr (K == 2) {
    w[0] = __ldg(reinterpret_cast<const unsigned int*>(p));
  } else if constexpr (K == 4) {
    const uint2 v = __ldg(reinterpret_cast<const uint2*>(p));
    w[0] = v.x; w[1] = v.y;
  } else {
    const uint4 v = __ldg(reinterpret_cast<const uint4*>(p));
    w[0] = v.x; w[1] = v.y; w[2] = v.z; w[3] = v.w;
  }
}

// FH: the factors are halves (factor - 1) or (factor), see k_fwd_finish; in
// the first case the missing sum of lengths is the pixel's total length W,
// added in the epilogue.
template <int K, bool EXACT, bool PEN, bool FH>
__device__ __forceinline__ void accumulate(float (&acc)[K], const float (&rf)[K],
                                           float l, const float* ub) {
  if constexpr (FH && !EXACT) {
    fma_halves<K>(acc, l, reinterpret_cast<const __half*>(ub));
    return;
  }
  Vec<K> u;
  if constexpr (FH)
    u = load_hvec<K, false>(reinterpret_cast<const __half*>(ub));
  else
    u = load_vec<K>(ub);
  if constexpr (EXACT) {
#pragma unroll
    for (int j = 0; j < K; ++j)
      acc[j] = PEN ? fsub(acc[j], fmul(fmul(rf[j], l), u.v[j]))
                   : fadd(acc[j], fmul(l, u.v[j]));
  } else {
    fma_slices<K>(acc, l, u.v);
  }
}

// Resident blocks per SM for each variant: compensated sums keep two more
// K-float arrays per thread (the quad's sum and the Kahan correction).
template <int K, bool COMP>
constexpr int min_blocks() {
  return COMP ? (K >= 16 ? 2 : 4) : (K >= 16 ? kMinBlocks16 : kMinBlocks);
}

// COMP: compensated summation - each quad's (four angles') products are an
// FMA chain added to the pixel's sum with Kahan's correction.
// One block's work (8 pixel tiles, from tile block * kWarps);
// s_coef: the block's kCoefChunk-entry shared buffer of window coefficients.
template <int K, int LK, bool EXACT, bool PEN, bool FH, bool COMP>
__device__ __forceinline__ void backward_block(const IterArgs& A, int batch, int block,
                                               const float* __restrict__ cur,
                                               float* __restrict__ next,
                                               const float* __restrict__ upd,
                                               float* __restrict__ rep_num, int epi,
                                               float4* s_coef) {
  const DevGeom& G = A.G;
  const int g = G.C;
  const int64_t g2 = (int64_t)g * g;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int tile = block * kWarps + warp;
  int x, y;
  tile_pixel(tile, lane, A.M.tiles_x, A.M.tw_shift, &x, &y);
  const bool valid = tile < A.M.ntiles && x < g && y < g;
  const int64_t p = (int64_t)y * g + x;
  const float xf = (float)x, yf = (float)y;
  const int fslot0 = batch * K + A.fshift;  // multiple of K
  const float* fsrc = cur + ((int64_t)(fslot0 / K) * g2 + p) * K;
  float rf[K];
#pragma unroll
  for (int j = 0; j < K; ++j) rf[j] = 0.f;
  if (PEN && EXACT && valid) {
    const Vec<K> v = load_vec<K>(fsrc);
#pragma unroll
    for (int j = 0; j < K; ++j) rf[j] = v.v[j];
  }
  float acc[K], cmp[K];
#pragma unroll
  for (int j = 0; j < K; ++j) acc[j] = cmp[j] = 0.f;
  // the fixed-point scale of 16-bit codes is applied once, at the end
  // (half factors take the scaled length: it is rounded to a half)
  constexpr bool kScaled = (LK == LK_U16) && !EXACT && !FH;
  const int P4 = A.M.P4;
  // walking pointers: this lane's matrix words and the factor rows of the
  // current four angles
  constexpr int QW = Quad<LK>::kWords;
  const uint32_t qstep = (uint32_t)A.M.ntiles * 32 * QW;  // words per 4 angles
  const uint4* qp = reinterpret_cast<const uint4*>(A.M.dlen) + ((int64_t)tile * 32 + lane) * QW;
  const int ck = G.C * K;  // factor floats per angle
  const float* ua = upd;
  for (int a0 = 0; a0 < P4; a0 += kCoefChunk) {
    const int na = min(kCoefChunk, P4 - a0);  // a multiple of 4
    __syncthreads();
    for (int i = threadIdx.x; i < na; i += kBlock) s_coef[i] = A.M.wcoef[a0 + i];
    __syncthreads();
    if (!valid) continue;
    Quad<LK> q;
    load_quad<LK>(qp, q);
    for (int a4 = 0; a4 < na; a4 += 4) {
      Quad<LK> nq;
      if (a4 + 4 < na) load_quad<LK>(qp + qstep, nq);
      // the quad's four angles into t
      auto quad_body = [&](float (&t)[K]) {
      if constexpr (FH && !EXACT && K >= 2 && K <= 8) {
        // software pipeline over the quad's 4 angles: the factor loads of
        // angle j + 1 are in flight while angle j's FMAs run
        // lw[b]: the two half lengths of the angle (slot 0 low, slot 1 high)
        uint32_t w0[2][K / 2], w1[2][K / 2], lw[2];
        auto issue = [&](int j, int b) {
          bool h0, h1;
          if constexpr (LK == LK_F16) {
            // stored as halves: the FMA operands as they are
            lw[b] = pick(q.w[0], j);
            h0 = (lw[b] & 0xffffu) != 0u;
            h1 = (lw[b] >> 16) != 0u;
          } else {
            float l0, l1;
            quad_pair<LK, false>(q, j, A.M.inv_scale, l0, l1, h0, h1);
            lw[b] = float2_to_half2_bits(l0, l1);
          }
          const int c0 = window_c0(s_coef[a4 + j], xf, yf);
          const __half* hb = reinterpret_cast<const __half*>(ua) + j * ck + c0 * K;
#pragma unroll
          for (int i = 0; i < K / 2; ++i) { w0[b][i] = 0u; w1[b][i] = 0u; }
          if (h0) load_hwords<K>(w0[b], hb);
          if (h1) load_hwords<K>(w1[b], hb + K);
        };
        auto consume = [&](int b) {
#pragma unroll
          for (int i = 0; i < K / 2; ++i) {
            asm("{ .reg .b16 lo, hi, l0, l1; mov.b32 {lo, hi}, %2; mov.b32 {l0, l1}, %3;"
                " fma.rn.f32.f16 %0, lo, l0, %0; fma.rn.f32.f16 %1, hi, l0, %1; }"
                : "+f"(t[2 * i]), "+f"(t[2 * i + 1]) : "r"(w0[b][i]), "r"(lw[b]));
            asm("{ .reg .b16 lo, hi, l0, l1; mov.b32 {lo, hi}, %2; mov.b32 {l0, l1}, %3;"
                " fma.rn.f32.f16 %0, lo, l1, %0; fma.rn.f32.f16 %1, hi, l1, %1; }"
                : "+f"(t[2 * i]), "+f"(t[2 * i + 1]) : "r"(w1[b][i]), "r"(lw[b]));
          }
        };
        issue(0, 0);
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          if (j < 3) issue(j + 1, (j + 1) & 1);
          consume(j & 1);
        }
      } else {
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        float l0, l1;
        bool h0, h1;
        quad_pair<LK, kScaled>(q, j, A.M.inv_scale, l0, l1, h0, h1);
        if (h0 | h1) {
          const int c0 = window_c0(s_coef[a4 + j], xf, yf);
          const int e = j * ck + c0 * K;  // factor element of ray c0
          const float* ub = FH ? reinterpret_cast<const float*>(
                                     reinterpret_cast<const __half*>(ua) + e)
                               : ua + e;
          const float* ub1 = FH ? reinterpret_cast<const float*>(
                                      reinterpret_cast<const __half*>(ub) + K)
                                : ub + K;
          if (h0) accumulate<K, EXACT, PEN, FH>(t, rf, l0, ub);
          if (h1) accumulate<K, EXACT, PEN, FH>(t, rf, l1, ub1);
        }
      }
      }
      };
      if constexpr (COMP) {
        float qa[K];
#pragma unroll
        for (int j = 0; j < K; ++j) qa[j] = 0.f;
        quad_body(qa);
#pragma unroll
        for (int j = 0; j < K; ++j) kahan_add(acc[j], cmp[j], qa[j]);
      } else {
        quad_body(acc);
      }
      q = nq;
      qp += qstep;
      ua = FH ? reinterpret_cast<const float*>(reinterpret_cast<const __half*>(ua) + 4 * ck)
              : ua + 4 * ck;
    }
  }
  if (!valid) return;
  if constexpr (COMP) {
#pragma unroll
    for (int j = 0; j < K; ++j) acc[j] = fsub(acc[j], cmp[j]);
  }
  // with half factors the lengths are taken as halves: their own total
  const float Wp = FH ? A.M.Wh[p] : A.M.W[p];
  if constexpr (kScaled) {
#pragma unroll
    for (int j = 0; j < K; ++j) acc[j] *= A.M.inv_scale;
  }
  // segments outside the pixel's window (stored apart, true lengths)
  for_each_exception(A.M, tile, lane, [&](float l, int ea, int ec) {
    const int64_t e = ((int64_t)ea * G.C + ec) * K;
    const float* ub = FH ? reinterpret_cast<const float*>(
                               reinterpret_cast<const __half*>(upd) + e)
                         : upd + e;
    accumulate<K, EXACT, PEN, FH>(acc, rf, l, ub);
  });
  if constexpr (FH) {
    if (A.half_factors == FACT_HALF_M1) {
#pragma unroll
      for (int j = 0; j < K; ++j) acc[j] += Wp;
    }
  }
  if (PEN && !EXACT) {  // the reconstruction factor, applied once per pixel
    const Vec<K> v = load_vec<K>(fsrc);
#pragma unroll
    for (int j = 0; j < K; ++j) acc[j] = -(v.v[j] * acc[j]);
  }
#pragma unroll
  for (int j = 0; j < K; ++j) {
    const int s = batch * K + j;
    if (s >= A.S) break;
    const float num = acc[j];
    if (epi == EPI_REPLICA) {
      rep_num[(int64_t)s * g2 + p] = num;
      continue;
    }
    const int ts = s + A.vshift;
    const int64_t at = slot_addr(ts, p, g2, K);
    const float old = cur[at];
    float nv;
    if constexpr (!PEN) {
      nv = A.alg == 0 ? fadd(old, fdiv(num, Wp)) : fmul(old, fdiv(num, Wp));
    } else {
      int up = 0, down = 0;
      if (A.alg == 3) apmlr_axial(A, s, &up, &down);
      float F, Gv;
      penalty_fg(A.alg == 3, A.pw, x, y, g, up, down,
                 [&](int dx, int dy, int dz) {
                   return cur[slot_addr(ts + dz, p + dx + (int64_t)dy * g, g2, K)];
                 },
                 F, Gv);
      Gv = fadd(Gv, Wp);
      nv = EXACT ? penalised_root(F, Gv, num) : penalised_root_stable(F, Gv, num);
    }
    next[at] = nv;
  }
}

template <int K, int LK, bool EXACT, bool PEN, bool FH, bool COMP>
__global__ void __launch_bounds__(kBlock, (min_blocks<K, COMP>()))
    k_backward(IterArgs A, int batch, const float* __restrict__ cur,
               float* __restrict__ next, const float* __restrict__ upd,
               float* __restrict__ rep_num, int epi) {
  __shared__ float4 s_coef[kCoefChunk];
  backward_block<K, LK, EXACT, PEN, FH, COMP>(A, batch, blockIdx.x, cur, next, upd,
                                              rep_num, epi, s_coef);
}

// Many plans' fused backprojection + update in one launch (fast mode):
// block -> work item (a plan's slice batch).
template <int K, int LK, bool PEN, bool FH, bool COMP>
__global__ void __launch_bounds__(kBlock, (min_blocks<K, COMP>()))
    k_backward_multi(const BackItem* __restrict__ items, int nitems) {
  __shared__ float4 s_coef[kCoefChunk];
  const BackItem& it = items[item_of(items, nitems, blockIdx.x)];
  backward_block<K, LK, false, PEN, FH, COMP>(it.A, it.batch, (int)(blockIdx.x - it.first),
                                              it.cur, it.next, it.upd, nullptr, EPI_UPDATE,
                                              s_coef);
}

// Multi-plan launches for plans with 16-bit fixed-point lengths: their
// backward matrix holds u16 codes, or IEEE halves with half gathers.
template <int K>
void back_multi(const BackItem* items, int n, int64_t blocks, int dlen_kind, int pen,
                int fh, int comp, cudaStream_t st) {
#define TG_BM(LKK, PN, FHH, CP) \
  k_backward_multi<K, LKK, PN, FHH, CP><<<(unsigned)blocks, kBlock, 0, st>>>(items, n)
  constexpr bool kComp = K <= 8;  // compensated sums: up to 8 slices per pass
#define TG_BM_PC(LKK, FHH)                                                               \
  do {                                                                                   \
    if (pen) { if (kComp && comp) TG_BM(LKK, true, FHH, kComp); else TG_BM(LKK, true, FHH, false); } \
    else { if (kComp && comp) TG_BM(LKK, false, FHH, kComp); else TG_BM(LKK, false, FHH, false); }   \
  } while (0)
  if (dlen_kind == LK_F16) {
    if (fh) TG_BM_PC(LK_F16, true); else TG_BM_PC(LK_F16, false);
  } else {
    TG_BM_PC(LK_U16, false);
  }
#undef TG_BM_PC
#undef TG_BM
}

template <int K, int LK>
void back_launch(const IterArgs& A, int batch, const float* cur, float* next,
                 const float* upd, float* rep_num, int epi, cudaStream_t st) {
  const int blocks = (A.M.ntiles + kWarps - 1) / kWarps;
  const bool pen = A.alg >= 2;
#define TG_BACK(E, PN, FH, CP)                                                        \
  k_backward<K, LK, E, PN, FH, CP><<<blocks, kBlock, 0, st>>>(A, batch, cur, next, upd, \
                                                             rep_num, epi)
  // compensated sums: up to 8 slices per pass (plan creation checks)
  constexpr bool kComp = K <= 8;
  if (A.exact) {
    if (pen) TG_BACK(true, true, false, false); else TG_BACK(true, false, false, false);
  } else if (kComp && A.comp) {
    if (A.half_factors) {
      if (pen) TG_BACK(false, true, true, kComp); else TG_BACK(false, false, true, kComp);
    } else {
      if (pen) TG_BACK(false, true, false, kComp); else TG_BACK(false, false, false, kComp);
    }
  } else if (A.half_factors) {
    if (pen) TG_BACK(false, true, true, false); else TG_BACK(false, false, true, false);
  } else {
    if (pen) TG_BACK(false, true, false, false); else TG_BACK(false, false, false, false);
  }
#undef TG_BACK
}

template <int K>
void back_kind(const IterArgs& A, int batch, const float* cur, float* next,
               const float* upd, float* rep_num, int epi, cudaStream_t st) {
  switch (A.M.dlen_kind) {
    case LK_F32: back_launch<K, LK_F32>(A, batch, cur, next, upd, rep_num, epi, st); break;
    case LK_BF16: back_launch<K, LK_BF16>(A, batch, cur, next, upd, rep_num, epi, st); break;
    case LK_F16: back_launch<K, LK_F16>(A, batch, cur, next, upd, rep_num, epi, st); break;
    default: back_launch<K, LK_U16>(A, batch, cur, next, upd, rep_num, epi, st); break;
  }
}

}  // namespace

// Backprojection launches for one K, each K compiled in its own translation
// unit (tg_backward*.cu) so the template instances build in parallel.
#define TG_BACKWARD_ENTRY(KK)                                                           \
  void launch_backward_k##KK(const IterArgs& A, int batch, const float* recon_cur,     \
                             float* recon_next, const float* upd, float* rep_num,      \
                             int epi, cudaStream_t st) {                               \
    back_kind<KK>(A, batch, recon_cur, recon_next, upd, rep_num, epi, st);             \
  }                                                                                     \
  void launch_backward_multi_k##KK(const BackItem* items, int n, int64_t blocks,       \
                                   int dlen_kind, int pen, int fh, int comp,            \
                                   cudaStream_t st) {                                   \
    back_multi<KK>(items, n, blocks, dlen_kind, pen, fh, comp, st);                     \
  }

}  // namespace tg
