// Iteration kernels: forward projection (ray-driven), backprojection
// (pixel-driven) with the algorithms' UpdateRecon fused into its epilogue,
// the operator-level penalty / update kernels, and layout conversions.
//
// K slices are processed per read of the (slice-invariant) matrix: slice j
// of a batch lives at lane j of a K-float vector per pixel / per ray, so one
// vector gather serves all K slices.
#include "tg_kernels.cuh"

namespace tg {

namespace {

constexpr int kBlock = 256;

template <int K>
__device__ __forceinline__ void zero(float (&a)[K]) {
#pragma unroll
  for (int j = 0; j < K; ++j) a[j] = 0.f;
}

// ---- forward projection ------------------------------------------------------
// One warp per 32-ray group; lane = ray. Sums recon[idx]*len along the ray in
// the reference's order (CalculateSimdata, sirt.cc:4-19), then stores the
// per-ray factor of the backprojection: (ray - sim)/a2 for SIRT
// (sirt.cc:50-53), ray/sim otherwise (mlem.cc:50, pml.cc:234), or sim.
template <int K, bool L16, bool EXACT, bool DELTA>
__global__ void __launch_bounds__(kBlock)
    k_forward(DevGeom G, MatrixDev M, int ngroups,
              const float* __restrict__ recon, const float* __restrict__ sino,
              float* __restrict__ out, int out_mode) {
  const int grp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (grp >= ngroups) return;  // warp-uniform
  const int a = grp / G.gpa;
  const int c = (grp - a * G.gpa) * 32 + lane;
  const bool valid = c < G.C;
  const int64_t r = (int64_t)a * G.C + c;
  const int n = valid ? M.rnseg[r] : 0;
  const int cap = M.rcap[grp];
  const int64_t base = M.roff[grp] + lane;
  const int g = G.C;
  float acc[K];
  zero(acc);
  int idx = 0;
  int64_t cbase = 0;
  uint32_t word = 0;
  if (DELTA) {
    cbase = M.rcoff[grp] + lane;
    if (n > 0) idx = M.rstart[r];
  }
  const float* len32 = reinterpret_cast<const float*>(M.rlen);
  const uint16_t* len16 = reinterpret_cast<const uint16_t*>(M.rlen);
#pragma unroll 4
  for (int s = 0; s < cap; ++s) {
    if (s < n) {
      const int64_t e = base + (int64_t)s * 32;
      if (DELTA) {
        if ((s & 7) == 0) word = __ldcs(M.rcode + cbase + (int64_t)(s >> 3) * 32);
        if (s > 0) {
          const uint32_t code = (word >> (4 * (s & 7))) & 15u;
          idx += (int)(code & 1u) + ((int)(code >> 1) - 1) * g;
        }
      } else {
        idx = __ldcs(M.ridx + e);
      }
      const float l = L16 ? decode16(__ldcs(len16 + e), M.len_kind, M.inv_scale)
                          : __ldcs(len32 + e);
      const Vec<K> v = load_vec<K>(recon + (int64_t)idx * K);
#pragma unroll
      for (int j = 0; j < K; ++j)
        acc[j] = EXACT ? fadd(acc[j], fmul(v.v[j], l)) : fmaf(v.v[j], l, acc[j]);
    }
  }
  if (!valid) return;
  Vec<K> o;
  if (out_mode == FWD_SIM) {
#pragma unroll
    for (int j = 0; j < K; ++j) o.v[j] = acc[j];
  } else {
    const Vec<K> ray = load_vec<K>(sino + r * K);
    if (out_mode == FWD_SIRT) {
      const float a2 = M.ra2[r];
#pragma unroll
      for (int j = 0; j < K; ++j) o.v[j] = fdiv(fsub(ray.v[j], acc[j]), a2);
    } else {
#pragma unroll
      for (int j = 0; j < K; ++j) o.v[j] = fdiv(ray.v[j], acc[j]);
    }
  }
  store_vec<K>(out + r * K, o);
}

// ---- backprojection + update -------------------------------------------------
__device__ __forceinline__ int64_t slot_addr(int slot, int64_t p, int64_t g2,
                                             int K) {
  return ((int64_t)(slot / K) * g2 + p) * K + (slot % K);
}

__device__ __forceinline__ void apmlr_axial(const IterArgs& A, int s, int* up,
                                            int* down) {
  const int beg = A.slice_id, end = A.slice_id + A.S - 1;
  const int final_index = A.slice_id + A.num_total_slices - 1;
  const bool top = (beg == 0 && s == 0);
  const bool bottom =
      !top && (final_index == end && final_index != 0 && s == A.S - 1);
  *up = !bottom;
  *down = !top;
}

// One thread per pixel, one warp per 32 adjacent pixels of a row. For every
// angle it reads the lengths of the (at most two) rays through its pixel and
// gathers their per-ray factors; the sum over angles in column order is the
// reference's replica[2p] accumulation (sirt.cc:58, mlem.cc:58, pml.cc:243).
// No atomics: every pixel is owned by one thread.
template <int K, bool L16, bool EXACT, bool PEN>
__global__ void __launch_bounds__(kBlock)
    k_backward(IterArgs A, int batch, const float* __restrict__ cur,
               float* __restrict__ next, const float* __restrict__ upd,
               float* __restrict__ rep_num, int epi) {
  const DevGeom& G = A.G;
  const int g = G.C;
  const int64_t g2 = (int64_t)g * g;
  const int pg = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  const int y = pg / G.gpr;
  if (y >= g) return;  // warp-uniform
  const int x = (pg - y * G.gpr) * 32 + lane;
  if (x >= g) return;
  const int64_t p = (int64_t)y * g + x;
  const int fslot0 = batch * K + A.fshift;  // multiple of K
  float rf[K];
  if (PEN) {
    const Vec<K> v = load_vec<K>(cur + ((int64_t)(fslot0 / K) * g2 + p) * K);
#pragma unroll
    for (int j = 0; j < K; ++j) rf[j] = v.v[j];
  }
  float acc[K];
  zero(acc);
  const float* d32 = reinterpret_cast<const float*>(A.M.dlen);
  const uint32_t* d16 = reinterpret_cast<const uint32_t*>(A.M.dlen);
#pragma unroll 2
  for (int a = 0; a < G.P; ++a) {
    const int64_t e = (int64_t)a * g2 + p;
    float l0, l1;
    bool h0, h1;
    if (L16) {
      const uint32_t w = __ldcs(d16 + e);
      h0 = (w & 0xffffu) != 0;
      h1 = (w >> 16) != 0;
      l0 = decode16((uint16_t)(w & 0xffffu), A.M.len_kind, A.M.inv_scale);
      l1 = decode16((uint16_t)(w >> 16), A.M.len_kind, A.M.inv_scale);
    } else {
      const float2 v = __ldcs(reinterpret_cast<const float2*>(d32) + e);
      l0 = v.x;
      l1 = v.y;
      // a stored -0.0f marks a zero-length segment (present, adds 0*upd)
      h0 = __float_as_uint(v.x) != 0;
      h1 = __float_as_uint(v.y) != 0;
    }
    if (h0 | h1) {
      const int c0 = window_c0(G, a, x, y);
      const float* ub = upd + ((int64_t)a * G.C + c0) * K;
      if (h0) {
        const Vec<K> u = load_vec<K>(ub);
#pragma unroll
        for (int j = 0; j < K; ++j) {
          if (EXACT)
            acc[j] = PEN ? fsub(acc[j], fmul(fmul(rf[j], l0), u.v[j]))
                         : fadd(acc[j], fmul(l0, u.v[j]));
          else
            acc[j] = fmaf(l0, u.v[j], acc[j]);
        }
      }
      if (h1) {
        const Vec<K> u = load_vec<K>(ub + K);
#pragma unroll
        for (int j = 0; j < K; ++j) {
          if (EXACT)
            acc[j] = PEN ? fsub(acc[j], fmul(fmul(rf[j], l1), u.v[j]))
                         : fadd(acc[j], fmul(l1, u.v[j]));
          else
            acc[j] = fmaf(l1, u.v[j], acc[j]);
        }
      }
    }
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
    if (A.alg == 0) {
      nv = fadd(old, fdiv(num, Wp));
    } else if (A.alg == 1) {
      nv = fmul(old, fdiv(num, Wp));
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
      nv = penalised_root(F, Gv, num);
    }
    next[at] = nv;
  }
}

// ---- operator-level penalty and update ---------------------------------------
__global__ void k_fg(IterArgs A, const float* __restrict__ recon,
                     const float* __restrict__ W, float* __restrict__ F,
                     float* __restrict__ Gv) {
  const int g = A.G.C;
  const int64_t g2 = (int64_t)g * g;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (int64_t)A.S * g2) return;
  const int s = (int)(i / g2);
  const int64_t p = i - (int64_t)s * g2;
  const int x = (int)(p % g), y = (int)(p / g);
  const int ts = s + A.vshift;
  int up = 0, down = 0;
  if (A.alg == 3) apmlr_axial(A, s, &up, &down);
  float f, gg;
  penalty_fg(A.alg == 3, A.pw, x, y, g, up, down,
             [&](int dx, int dy, int dz) {
               return recon[slot_addr(ts + dz, p + dx + (int64_t)dy * g, g2, A.K)];
             },
             f, gg);
  F[i] = f;
  Gv[i] = fadd(gg, W[p]);
}

__global__ void k_update(IterArgs A, float* __restrict__ recon,
                         const float* __restrict__ W,
                         const float* __restrict__ F,
                         const float* __restrict__ Gv,
                         const float* __restrict__ rep_num) {
  const int g = A.G.C;
  const int64_t g2 = (int64_t)g * g;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (int64_t)A.S * g2) return;
  const int s = (int)(i / g2);
  const int64_t p = i - (int64_t)s * g2;
  const int64_t at = slot_addr(s + A.vshift, p, g2, A.K);
  const float num = rep_num[i];
  if (A.alg == 0)
    recon[at] = fadd(recon[at], fdiv(num, W[p]));
  else if (A.alg == 1)
    recon[at] = fmul(recon[at], fdiv(num, W[p]));
  else
    recon[at] = penalised_root(F[i], Gv[i], num);
}

// ---- layouts -----------------------------------------------------------------
// [P][S][C] -> [ceil(S/K)][P*C][K]
__global__ void k_sino_pack(const float* __restrict__ in, float* __restrict__ out,
                            int P, int S, int C, int K, int apply_abs) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t n = (int64_t)P * S * C;
  if (i >= n) return;
  const int c = (int)(i % C);
  const int64_t t = i / C;
  const int s = (int)(t % S), a = (int)(t / S);
  const int64_t R = (int64_t)P * C;
  float v = in[i];
  if (apply_abs) v = fabsf(v);
  out[((int64_t)(s / K) * R + (int64_t)a * C + c) * K + (s % K)] = v;
}

__global__ void k_sino_unpack(const float* __restrict__ in,
                              float* __restrict__ out, int P, int S, int C,
                              int K) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t n = (int64_t)P * S * C;
  if (i >= n) return;
  const int c = (int)(i % C);
  const int64_t t = i / C;
  const int s = (int)(t % S), a = (int)(t / S);
  const int64_t R = (int64_t)P * C;
  out[i] = in[((int64_t)(s / K) * R + (int64_t)a * C + c) * K + (s % K)];
}

// user slice u (reference layout, halo included) <-> internal slot u + slot0
__global__ void k_recon_pack(const float* __restrict__ in, float* __restrict__ out,
                             int nuser, int64_t g2, int K, int slot0) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (int64_t)nuser * g2) return;
  const int u = (int)(i / g2);
  const int64_t p = i - (int64_t)u * g2;
  out[slot_addr(u + slot0, p, g2, K)] = in[i];
}

__global__ void k_recon_unpack(const float* __restrict__ in,
                               float* __restrict__ out, int nuser, int64_t g2,
                               int K, int slot0) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (int64_t)nuser * g2) return;
  const int u = (int)(i / g2);
  const int64_t p = i - (int64_t)u * g2;
  out[i] = in[slot_addr(u + slot0, p, g2, K)];
}

__global__ void k_fill(float* p, int64_t n, float v) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) p[i] = v;
}

__global__ void k_replica_interleave(const float* __restrict__ rep_num,
                                     const float* __restrict__ W,
                                     float* __restrict__ out, int S,
                                     int64_t g2) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (int64_t)S * g2) return;
  const int64_t p = i % g2;
  out[2 * i] = rep_num[i];
  out[2 * i + 1] = W[p];
}

inline int blocks_for(int64_t n, int b = kBlock) { return (int)((n + b - 1) / b); }

template <int K>
void fwd_dispatch(const IterArgs& A, const float* recon, const float* sino,
                  float* out, int out_mode, cudaStream_t st) {
  const int ngroups = A.G.P * A.G.gpa;
  const int blocks = blocks_for((int64_t)ngroups * 32);
  const bool l16 = A.M.len_kind != LK_F32;
#define TG_FWD(L, E, D)                                                     \
  k_forward<K, L, E, D><<<blocks, kBlock, 0, st>>>(A.G, A.M, ngroups, recon, \
                                                   sino, out, out_mode)
  if (A.delta_index) {
    if (l16) { if (A.exact) TG_FWD(true, true, true); else TG_FWD(true, false, true); }
    else { if (A.exact) TG_FWD(false, true, true); else TG_FWD(false, false, true); }
  } else {
    if (l16) { if (A.exact) TG_FWD(true, true, false); else TG_FWD(true, false, false); }
    else { if (A.exact) TG_FWD(false, true, false); else TG_FWD(false, false, false); }
  }
#undef TG_FWD
}

template <int K>
void back_dispatch(const IterArgs& A, int batch, const float* cur, float* next,
                   const float* upd, float* rep_num, int epi, cudaStream_t st) {
  const int blocks = blocks_for((int64_t)A.G.C * A.G.gpr * 32);
  const bool l16 = A.M.len_kind != LK_F32;
  const bool pen = A.alg >= 2;
#define TG_BACK(L, E, PN)                                                   \
  k_backward<K, L, E, PN><<<blocks, kBlock, 0, st>>>(A, batch, cur, next, upd, \
                                                     rep_num, epi)
  if (l16) {
    if (A.exact) { if (pen) TG_BACK(true, true, true); else TG_BACK(true, true, false); }
    else { if (pen) TG_BACK(true, false, true); else TG_BACK(true, false, false); }
  } else {
    if (A.exact) { if (pen) TG_BACK(false, true, true); else TG_BACK(false, true, false); }
    else { if (pen) TG_BACK(false, false, true); else TG_BACK(false, false, false); }
  }
#undef TG_BACK
}

}  // namespace

void launch_forward(const IterArgs& A, const float* recon_batch,
                    const float* sino_batch, float* out, int out_mode,
                    cudaStream_t st) {
  switch (A.K) {
    case 1: fwd_dispatch<1>(A, recon_batch, sino_batch, out, out_mode, st); break;
    case 2: fwd_dispatch<2>(A, recon_batch, sino_batch, out, out_mode, st); break;
    case 4: fwd_dispatch<4>(A, recon_batch, sino_batch, out, out_mode, st); break;
    default: fwd_dispatch<8>(A, recon_batch, sino_batch, out, out_mode, st); break;
  }
}

void launch_backward(const IterArgs& A, int batch, const float* recon_cur,
                     float* recon_next, const float* upd, float* rep_num,
                     int epi, cudaStream_t st) {
  switch (A.K) {
    case 1: back_dispatch<1>(A, batch, recon_cur, recon_next, upd, rep_num, epi, st); break;
    case 2: back_dispatch<2>(A, batch, recon_cur, recon_next, upd, rep_num, epi, st); break;
    case 4: back_dispatch<4>(A, batch, recon_cur, recon_next, upd, rep_num, epi, st); break;
    default: back_dispatch<8>(A, batch, recon_cur, recon_next, upd, rep_num, epi, st); break;
  }
}

void launch_fg(const IterArgs& A, const float* recon, const float* W, float* F,
               float* Gv, cudaStream_t st) {
  const int64_t n = (int64_t)A.S * A.G.C * A.G.C;
  k_fg<<<blocks_for(n), kBlock, 0, st>>>(A, recon, W, F, Gv);
}

void launch_update(const IterArgs& A, float* recon, const float* W,
                   const float* F, const float* Gv, const float* rep_num,
                   cudaStream_t st) {
  const int64_t n = (int64_t)A.S * A.G.C * A.G.C;
  k_update<<<blocks_for(n), kBlock, 0, st>>>(A, recon, W, F, Gv, rep_num);
}

void launch_sino_pack(const float* in, float* out, int P, int S, int C, int K,
                      int apply_abs, cudaStream_t st) {
  const int64_t n = (int64_t)P * S * C;
  k_sino_pack<<<blocks_for(n), kBlock, 0, st>>>(in, out, P, S, C, K, apply_abs);
}

void launch_sino_unpack(const float* in, float* out, int P, int S, int C,
                        int K, cudaStream_t st) {
  const int64_t n = (int64_t)P * S * C;
  k_sino_unpack<<<blocks_for(n), kBlock, 0, st>>>(in, out, P, S, C, K);
}

void launch_recon_pack(const float* in, float* out, int nuser, int g2, int K,
                       int slot0, int /*nslots*/, cudaStream_t st) {
  const int64_t n = (int64_t)nuser * g2;
  k_recon_pack<<<blocks_for(n), kBlock, 0, st>>>(in, out, nuser, g2, K, slot0);
}

void launch_recon_unpack(const float* in, float* out, int nuser, int g2, int K,
                         int slot0, cudaStream_t st) {
  const int64_t n = (int64_t)nuser * g2;
  k_recon_unpack<<<blocks_for(n), kBlock, 0, st>>>(in, out, nuser, g2, K, slot0);
}

void launch_fill(float* p, size_t n, float v, cudaStream_t st) {
  if (n == 0) return;
  k_fill<<<blocks_for((int64_t)n), kBlock, 0, st>>>(p, (int64_t)n, v);
}

void launch_replica_interleave(const float* rep_num, const float* W,
                               float* out, int S, int g2, cudaStream_t st) {
  const int64_t n = (int64_t)S * g2;
  k_replica_interleave<<<blocks_for(n), kBlock, 0, st>>>(rep_num, W, out, S, g2);
}

}  // namespace tg
