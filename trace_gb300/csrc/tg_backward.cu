// Backprojection (pixel-driven) with the algorithms' UpdateRecon fused into
// its epilogue.
//
// One thread per pixel, one warp per 8x4 pixel tile, eight tiles per block.
// For every angle a thread reads the lengths of the (at most two) rays
// through its pixel - one contiguous 32-lane row of the backward matrix per
// warp - and gathers those rays' factors. The sum over angles in column
// order is the reference's replica[2p] accumulation (sirt.cc:58,
// mlem.cc:58, pml.cc:243); the total length per pixel (replica[2p+1]) is a
// per-geometry constant. No atomics: every pixel is owned by one thread.
// The tile shape keeps the rays a warp touches at one angle within a short
// detector window, so the factor gathers share L1 sectors.
//
// Epilogue per slice: SIRT recon += num/W (sirt.cc:21-33), MLEM
// recon *= num/W (mlem.cc:21-34), PML/APMLR the closed-form root with the
// penalty's F and G (pml.cc:3-23, apmlr.cc:3-26), written to the other
// reconstruction buffer so neighbours read by the stencil stay unmodified.
#include "tg_kernels.cuh"

namespace tg {

namespace {

constexpr int kWarps = 8;
constexpr int kBlock = kWarps * 32;
constexpr int kCoefChunk = 512;  // angles of window coefficients per stage

// Four angles of one lane's backward-matrix entries: 16 bytes for 16-bit
// codes (two per angle), 32 bytes for floats.
template <int LK>
struct Quad {
  uint4 w[LK == LK_F32 ? 2 : 1];
};

template <int LK>
__device__ __forceinline__ void load_quad(const void* dlen, int64_t pair, Quad<LK>& q) {
  if constexpr (LK == LK_F32) {
    const uint4* p = reinterpret_cast<const uint4*>(reinterpret_cast<const float2*>(dlen) + pair);
    q.w[0] = __ldcs(p);
    q.w[1] = __ldcs(p + 1);
  } else {
    q.w[0] = __ldcs(reinterpret_cast<const uint4*>(reinterpret_cast<const uint32_t*>(dlen) + pair));
  }
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

template <int K, bool EXACT, bool PEN>
__device__ __forceinline__ void accumulate(float (&acc)[K], const float (&rf)[K],
                                           float l, const float* ub) {
  const Vec<K> u = load_vec<K>(ub);
#pragma unroll
  for (int j = 0; j < K; ++j) {
    if (EXACT)
      acc[j] = PEN ? fsub(acc[j], fmul(fmul(rf[j], l), u.v[j]))
                   : fadd(acc[j], fmul(l, u.v[j]));
    else
      acc[j] = fmaf(l, u.v[j], acc[j]);
  }
}

template <int K, int LK, bool EXACT, bool PEN>
__global__ void __launch_bounds__(kBlock, 6)
    k_backward(IterArgs A, int batch, const float* __restrict__ cur,
               float* __restrict__ next, const float* __restrict__ upd,
               float* __restrict__ rep_num, int epi) {
  __shared__ float4 s_coef[kCoefChunk];
  const DevGeom& G = A.G;
  const int g = G.C;
  const int64_t g2 = (int64_t)g * g;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int tile = blockIdx.x * kWarps + warp;
  const int x = (tile % A.M.tiles_x) * 8 + (lane & 7);
  const int y = (tile / A.M.tiles_x) * 4 + (lane >> 3);
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
  float acc[K];
#pragma unroll
  for (int j = 0; j < K; ++j) acc[j] = 0.f;
  // the fixed-point scale of 16-bit codes is applied once, at the end
  constexpr bool kScaled = (LK == LK_U16) && !EXACT;
  const int P4 = A.M.P4;
  const int64_t qstride = (int64_t)A.M.ntiles * 32 * 4;  // pairs per 4 angles
  for (int a0 = 0; a0 < P4; a0 += kCoefChunk) {
    const int na = min(kCoefChunk, P4 - a0);  // a multiple of 4
    __syncthreads();
    for (int i = threadIdx.x; i < na; i += kBlock) s_coef[i] = A.M.wcoef[a0 + i];
    __syncthreads();
    if (!valid) continue;
    const float* ua = upd + (int64_t)a0 * G.C * K;
    int64_t pair = dense_pair(A.M.ntiles, a0, tile, lane);
    Quad<LK> q;
    load_quad<LK>(A.M.dlen, pair, q);
    for (int a4 = 0; a4 < na; a4 += 4) {
      Quad<LK> nq;
      if (a4 + 4 < na) load_quad<LK>(A.M.dlen, pair + qstride, nq);
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        float l0, l1;
        bool h0, h1;
        quad_pair<LK, kScaled>(q, j, A.M.inv_scale, l0, l1, h0, h1);
        if (h0 | h1) {
          const int c0 = window_c0(s_coef[a4 + j], xf, yf);
          const float* ub = ua + ((int64_t)j * G.C + c0) * K;
          if (h0) accumulate<K, EXACT, PEN>(acc, rf, l0, ub);
          if (h1) accumulate<K, EXACT, PEN>(acc, rf, l1, ub + K);
        }
      }
      q = nq;
      pair += qstride;
      ua += (int64_t)4 * G.C * K;
    }
  }
  if (!valid) return;
  if constexpr (kScaled) {
#pragma unroll
    for (int j = 0; j < K; ++j) acc[j] *= A.M.inv_scale;
  }
  if (PEN && !EXACT) {
    const Vec<K> v = load_vec<K>(fsrc);
#pragma unroll
    for (int j = 0; j < K; ++j) rf[j] = v.v[j];
  }
  const float Wp = A.M.W[p];
#pragma unroll
  for (int j = 0; j < K; ++j) {
    const int s = batch * K + j;
    if (s >= A.S) break;
    float num = acc[j];
    if (PEN && !EXACT) num = -(rf[j] * acc[j]);
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

template <int K, int LK>
void back_launch(const IterArgs& A, int batch, const float* cur, float* next,
                 const float* upd, float* rep_num, int epi, cudaStream_t st) {
  const int blocks = (A.M.ntiles + kWarps - 1) / kWarps;
  const bool pen = A.alg >= 2;
#define TG_BACK(E, PN) \
  k_backward<K, LK, E, PN><<<blocks, kBlock, 0, st>>>(A, batch, cur, next, upd, rep_num, epi)
  if (A.exact) {
    if (pen) TG_BACK(true, true); else TG_BACK(true, false);
  } else {
    if (pen) TG_BACK(false, true); else TG_BACK(false, false);
  }
#undef TG_BACK
}

template <int K>
void back_kind(const IterArgs& A, int batch, const float* cur, float* next,
               const float* upd, float* rep_num, int epi, cudaStream_t st) {
  switch (A.M.len_kind) {
    case LK_F32: back_launch<K, LK_F32>(A, batch, cur, next, upd, rep_num, epi, st); break;
    case LK_BF16: back_launch<K, LK_BF16>(A, batch, cur, next, upd, rep_num, epi, st); break;
    case LK_F16: back_launch<K, LK_F16>(A, batch, cur, next, upd, rep_num, epi, st); break;
    default: back_launch<K, LK_U16>(A, batch, cur, next, upd, rep_num, epi, st); break;
  }
}

}  // namespace

void launch_backward(const IterArgs& A, int batch, const float* recon_cur,
                     float* recon_next, const float* upd, float* rep_num,
                     int epi, cudaStream_t st) {
  switch (A.K) {
    case 1: back_kind<1>(A, batch, recon_cur, recon_next, upd, rep_num, epi, st); break;
    case 2: back_kind<2>(A, batch, recon_cur, recon_next, upd, rep_num, epi, st); break;
    case 4: back_kind<4>(A, batch, recon_cur, recon_next, upd, rep_num, epi, st); break;
    default: back_kind<8>(A, batch, recon_cur, recon_next, upd, rep_num, epi, st); break;
  }
}

}  // namespace tg
