// Backprojection with the per-ray factors staged in shared memory (fast mode).
//
// A block covers 16 x 16 pixels (eight 8x4 warp tiles). At one angle the rays
// through those pixels are a window of at most 24 consecutive detector
// columns, starting at the smallest window_c0 over the block's corners
// (window_c0 is monotone in the pixel position). Angles are processed in
// chunks of 32: while a chunk is consumed, the next chunk's windows (32
// columns x K floats per angle) are copied from global memory into the other
// half of a double buffer with cp.async, so every factor gather of the main
// loop is a shared-memory read instead of an L1 lookup. Arithmetic and
// accumulation order per pixel are those of k_backward (fast mode).
#include "tg_kernels.cuh"

namespace tg {

namespace {

constexpr int kWarps = 8;
constexpr int kBlock = kWarps * 32;
constexpr int kBlockPx = 16;  // block side in pixels (2 x 4 warp tiles)
constexpr int kAC = 32;       // angles per chunk
constexpr int kWin = 24;      // detector columns staged per angle (<= 23 used)

// A staged ray's K factors sit at a stride of kRay floats: 12 (48 B) for
// K = 8, so the two 16-byte halves of 8 consecutive rays fall in distinct
// bank groups (3 * ray mod 8); K floats otherwise (already conflict-free).
template <int K>
struct Stage {
  static constexpr int kRay = K == 8 ? 12 : K == 16 ? 20 : K;
  static constexpr int kUnitBytes = K >= 4 ? 16 : K * 4;
  static constexpr int kUnitsPerRay = K * 4 / kUnitBytes;
  static constexpr int kUnits = kAC * kWin * kUnitsPerRay;  // per chunk
  static constexpr int kFloats = kAC * kWin * kRay;
};

__device__ __forceinline__ void cp_async(void* smem, const void* gmem, int bytes,
                                         bool valid) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  const int src = valid ? bytes : 0;  // 0 source bytes: the copy writes zeros
  if (bytes == 16)
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(s), "l"(gmem), "r"(src));
  else if (bytes == 8)
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;" ::"r"(s), "l"(gmem), "r"(src));
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(s), "l"(gmem), "r"(src));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

template <int K>
__device__ __forceinline__ Vec<K> lds_vec(const float* p) {
  Vec<K> r;
  if constexpr (K >= 4) {
#pragma unroll
    for (int j = 0; j < K; j += 4) {
      const float4 t = *reinterpret_cast<const float4*>(p + j);
      r.v[j] = t.x;
      r.v[j + 1] = t.y;
      r.v[j + 2] = t.z;
      r.v[j + 3] = t.w;
    }
  } else if constexpr (K == 2) {
    const float2 t = *reinterpret_cast<const float2*>(p);
    r.v[0] = t.x;
    r.v[1] = t.y;
  } else {
    r.v[0] = *p;
  }
  return r;
}

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

template <int LK>
__device__ __forceinline__ void quad_pair(const Quad<LK>& q, int j, float inv_scale,
                                          float& l0, float& l1, bool& h0, bool& h1) {
  if constexpr (LK == LK_F32) {
    const uint32_t a = pick(q.w[j >> 1], (j & 1) * 2), b = pick(q.w[j >> 1], (j & 1) * 2 + 1);
    h0 = a != 0u;
    h1 = b != 0u;
    l0 = __uint_as_float(a);
    l1 = __uint_as_float(b);
  } else {
    const uint32_t w = pick(q.w[0], j);
    h0 = (w & 0xffffu) != 0u;
    h1 = (w >> 16) != 0u;
    if constexpr (LK == LK_U16) {  // scale applied once at the end
      l0 = u16_to_float(w & 0xffffu);
      l1 = u16_to_float(w >> 16);
    } else {
      l0 = decode_len<LK>((uint16_t)(w & 0xffffu), inv_scale);
      l1 = decode_len<LK>((uint16_t)(w >> 16), inv_scale);
    }
  }
}

// Window starts of one chunk (thread i < kAC handles angle a0 + i) and
// the asynchronous copy of the chunk's factor windows into `buf`.
template <int K>
__device__ __forceinline__ void stage_chunk(const IterArgs& A, const float* upd,
                                            int a0, int bx0, int by0, float4* s_coef,
                                            int* s_ws, float* buf) {
  const int P4 = A.M.P4;
  if (threadIdx.x < kAC) {
    const int a = a0 + threadIdx.x;
    float4 cf = make_float4(0.f, 0.f, 0.f, 0.f);
    int ws = 0;
    if (a < P4) {
      cf = A.M.wcoef[a];
      const float x0 = (float)bx0, y0 = (float)by0;
      const float x1 = x0 + (kBlockPx - 1), y1 = y0 + (kBlockPx - 1);
      ws = min(min(window_c0(cf, x0, y0), window_c0(cf, x1, y0)),
               min(window_c0(cf, x0, y1), window_c0(cf, x1, y1)));
    }
    s_coef[threadIdx.x] = cf;
    s_ws[threadIdx.x] = ws;
  }
  __syncthreads();
  using St = Stage<K>;
  const int C = A.G.C, P = A.G.P;
  for (int u = threadIdx.x; u < St::kUnits; u += kBlock) {
    const int ai = u / (kWin * St::kUnitsPerRay);
    const int rem = u - ai * (kWin * St::kUnitsPerRay);
    const int ri = rem / St::kUnitsPerRay;
    const int ui = rem - ri * St::kUnitsPerRay;
    const int a = a0 + ai;
    const int col = s_ws[ai] + ri;
    const bool valid = a < P && col >= 0 && col < C;
    const float* src = valid ? upd + ((int64_t)a * C + col) * K + ui * (St::kUnitBytes / 4) : upd;
    cp_async(buf + ((ai * kWin + ri) * St::kRay + ui * (St::kUnitBytes / 4)), src,
             St::kUnitBytes, valid);
  }
  cp_async_commit();
}

template <int K, int LK, bool PEN>
__global__ void __launch_bounds__(kBlock)
    k_backward_staged(IterArgs A, int batch, const float* __restrict__ cur,
                      float* __restrict__ next, const float* __restrict__ upd,
                      float* __restrict__ rep_num, int epi) {
  extern __shared__ float4 dyn[];
  float* s_upd = reinterpret_cast<float*>(dyn);                 // [2][kAC][kWin][K]
  float4* s_coef = reinterpret_cast<float4*>(s_upd + 2 * Stage<K>::kFloats);  // [2][kAC]
  int* s_ws = reinterpret_cast<int*>(s_coef + 2 * kAC);         // [2][kAC]
  const DevGeom& G = A.G;
  const int g = G.C;
  const int64_t g2 = (int64_t)g * g;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int bx0 = blockIdx.x * kBlockPx, by0 = blockIdx.y * kBlockPx;
  const int tx = blockIdx.x * 2 + (warp & 1), ty = blockIdx.y * 4 + (warp >> 1);
  const int tile = ty * A.M.tiles_x + tx;
  const int x = tx * 8 + (lane & 7), y = ty * 4 + (lane >> 3);
  const bool valid = tx < A.M.tiles_x && x < g && y < g;
  const int64_t p = (int64_t)y * g + x;
  const float xf = (float)x, yf = (float)y;
  float acc[K];
#pragma unroll
  for (int j = 0; j < K; ++j) acc[j] = 0.f;
  const int P4 = A.M.P4;
  const int nchunks = (P4 + kAC - 1) / kAC;
  const int64_t qstride = (int64_t)A.M.ntiles * 32 * 4;
  int64_t pair = valid ? dense_pair(A.M.ntiles, 0, tile, lane) : 0;
  Quad<LK> q;  // current four angles of this lane's matrix row; next one prefetched
  if (valid && P4 > 0) load_quad<LK>(A.M.dlen, pair, q);
  stage_chunk<K>(A, upd, 0, bx0, by0, s_coef, s_ws, s_upd);
  for (int ch = 0; ch < nchunks; ++ch) {
    const int b = ch & 1;
    cp_async_wait_all();
    __syncthreads();  // chunk ch resident; everyone done with chunk ch-1
    if (ch + 1 < nchunks)
      stage_chunk<K>(A, upd, (ch + 1) * kAC, bx0, by0, s_coef + (b ^ 1) * kAC,
                     s_ws + (b ^ 1) * kAC, s_upd + (b ^ 1) * Stage<K>::kFloats);
    if (valid) {
      const float* su = s_upd + b * Stage<K>::kFloats;
      const float4* sc = s_coef + b * kAC;
      const int* sw = s_ws + b * kAC;
      const int na = min(kAC, P4 - ch * kAC);  // a multiple of 4
      for (int a4 = 0; a4 < na; a4 += 4) {
        Quad<LK> nq;
        if (ch * kAC + a4 + 4 < P4) load_quad<LK>(A.M.dlen, pair + qstride, nq);
        pair += qstride;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          float l0, l1;
          bool h0, h1;
          quad_pair<LK>(q, j, A.M.inv_scale, l0, l1, h0, h1);
          if (h0 | h1) {
            const int ai = a4 + j;
            int rel = window_c0(sc[ai], xf, yf) - sw[ai];
            rel = min(max(rel, 0), kWin - 2);  // in range by construction
            const float* sb = su + (ai * kWin + rel) * Stage<K>::kRay;
            if (h0) {
              const Vec<K> u = lds_vec<K>(sb);
              fma_slices<K>(acc, l0, u.v);
            }
            if (h1) {
              const Vec<K> u = lds_vec<K>(sb + Stage<K>::kRay);
              fma_slices<K>(acc, l1, u.v);
            }
          }
        }
        q = nq;
      }
    }
  }
  if (!valid) return;
  if constexpr (LK == LK_U16) {
#pragma unroll
    for (int k = 0; k < K; ++k) acc[k] *= A.M.inv_scale;
  }
  // segments outside the pixel's window (stored apart, true lengths)
  for_each_exception(A.M, tile, lane, [&](float l, int ea, int ec) {
    const Vec<K> u = load_vec<K>(upd + ((int64_t)ea * G.C + ec) * K);
    fma_slices<K>(acc, l, u.v);
  });
  float rf[K];
  if (PEN) {
    const Vec<K> v = load_vec<K>(cur + ((int64_t)((batch * K + A.fshift) / K) * g2 + p) * K);
#pragma unroll
    for (int k = 0; k < K; ++k) rf[k] = v.v[k];
  }
  const float Wp = A.M.W[p];
#pragma unroll
  for (int k = 0; k < K; ++k) {
    const int s = batch * K + k;
    if (s >= A.S) break;
    float num = acc[k];
    if (PEN) num = -(rf[k] * acc[k]);
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
      nv = penalised_root_stable(F, Gv, num);
    }
    next[at] = nv;
  }
}

template <int K, int LK>
void staged_launch(const IterArgs& A, int batch, const float* cur, float* next,
                   const float* upd, float* rep_num, int epi, cudaStream_t st) {
  const int tiles_y = (A.G.C + 3) / 4;
  const dim3 grid((A.M.tiles_x + 1) / 2, (tiles_y + 3) / 4);
  const int smem = 2 * Stage<K>::kFloats * 4 + 2 * kAC * 16 + 2 * kAC * 4;
  if (A.alg >= 2) {
    cudaFuncSetAttribute(k_backward_staged<K, LK, true>,
                         cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    k_backward_staged<K, LK, true><<<grid, kBlock, smem, st>>>(A, batch, cur, next, upd,
                                                                rep_num, epi);
  } else {
    cudaFuncSetAttribute(k_backward_staged<K, LK, false>,
                         cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    k_backward_staged<K, LK, false><<<grid, kBlock, smem, st>>>(A, batch, cur, next, upd,
                                                                 rep_num, epi);
  }
}

template <int K>
void staged_kind(const IterArgs& A, int batch, const float* cur, float* next,
                 const float* upd, float* rep_num, int epi, cudaStream_t st) {
  switch (A.M.dlen_kind) {
    case LK_F32: staged_launch<K, LK_F32>(A, batch, cur, next, upd, rep_num, epi, st); break;
    case LK_BF16: staged_launch<K, LK_BF16>(A, batch, cur, next, upd, rep_num, epi, st); break;
    case LK_F16: staged_launch<K, LK_F16>(A, batch, cur, next, upd, rep_num, epi, st); break;
    default: staged_launch<K, LK_U16>(A, batch, cur, next, upd, rep_num, epi, st); break;
  }
}

}  // namespace

void launch_backward_staged(const IterArgs& A, int batch, const float* recon_cur,
                            float* recon_next, const float* upd, float* rep_num,
                            int epi, cudaStream_t st) {
  switch (A.K) {
    case 1: staged_kind<1>(A, batch, recon_cur, recon_next, upd, rep_num, epi, st); break;
    case 2: staged_kind<2>(A, batch, recon_cur, recon_next, upd, rep_num, epi, st); break;
    case 4: staged_kind<4>(A, batch, recon_cur, recon_next, upd, rep_num, epi, st); break;
    case 8: staged_kind<8>(A, batch, recon_cur, recon_next, upd, rep_num, epi, st); break;
    default: staged_kind<16>(A, batch, recon_cur, recon_next, upd, rep_num, epi, st); break;
  }
}

}  // namespace tg
