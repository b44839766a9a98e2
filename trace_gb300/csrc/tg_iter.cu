// Operator-level penalty / update kernels (the reference's CalculateFG and
// UpdateRecon as separate steps) and layout conversions between the
// reference's [P][S][C] / [S][g][g] arrays and the batched device layout.
#include "tg_kernels.cuh"

namespace tg {

namespace {

constexpr int kBlock = 256;

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
    recon[at] = A.exact ? penalised_root(F[i], Gv[i], num)
                        : penalised_root_stable(F[i], Gv[i], num);
}

// ---- layouts -----------------------------------------------------------------
// [P][S][C] -> [ceil(S/K)][P*C][K]
__global__ void k_sino_pack(const float* __restrict__ in, float* __restrict__ out,
                            int P, int S, int C, int K, int apply_abs, int clip,
                            float clip_min) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t n = (int64_t)P * S * C;
  if (i >= n) return;
  const int c = (int)(i % C);
  const int64_t t = i / C;
  const int s = (int)(t % S), a = (int)(t / S);
  const int64_t R = (int64_t)P * C;
  float v = in[i];
  if (apply_abs) v = fabsf(v);
  if (clip && v < clip_min) v = clip_min;  // NaN fails the test and stays NaN
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

}  // namespace

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
                      int apply_abs, int clip, float clip_min, cudaStream_t st) {
  const int64_t n = (int64_t)P * S * C;
  k_sino_pack<<<blocks_for(n), kBlock, 0, st>>>(in, out, P, S, C, K, apply_abs, clip,
                                                 clip_min);
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
