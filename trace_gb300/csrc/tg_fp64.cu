// FP64 mode: the same algorithm with the reconstruction, the per-ray
// factors, every sum and the update in double. The matrices are the float
// ones (the geometry is traced in float exactly as the reference traces it,
// so the index lists are the reference's); lengths are widened. This is the
// "FP64 run of the same algorithm" the mixed-precision paths are measured
// against at sizes where a CPU run would take hours. One slice per pass.
#include "tg_kernels.cuh"

namespace tg {

namespace {

constexpr int kBlock = 256;

__global__ void __launch_bounds__(kBlock)
    k_forward64(DevGeom G, MatrixDev M, const double* ra2d, int ngroups,
                const double* __restrict__ recon, const float* __restrict__ sino,
                double* __restrict__ out, int out_mode) {
  const int grp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (grp >= ngroups) return;
  const int a = grp / G.gpa;
  const int c = (grp - a * G.gpa) * 32 + lane;
  if (c >= G.C) return;
  const int64_t r = (int64_t)a * G.C + c;
  const int n = M.rnseg[r];
  const int64_t base = M.roff[grp] + lane;
  const float* len = reinterpret_cast<const float*>(M.rlen);
  double acc = 0.0;
  for (int s = 0; s < n; ++s) {
    const int64_t e = base + (int64_t)s * 32;
    acc = __dadd_rn(acc, __dmul_rn(recon[__ldcs(M.ridx + e)], (double)__ldcs(len + e)));
  }
  if (out_mode == FWD_SIM) {
    out[r] = acc;
  } else if (out_mode == FWD_SIRT) {
    out[r] = __ddiv_rn(__dsub_rn((double)sino[r], acc), ra2d[r]);
  } else {
    out[r] = __ddiv_rn((double)sino[r], acc);
  }
}

__global__ void k_weights64(DevGeom G, MatrixDev M, double* W) {
  const int g = G.C;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)M.ntiles * 32) return;
  const int tile = (int)(t >> 5), lane = (int)(t & 31);
  int x, y;
  tile_pixel(tile, lane, M.tiles_x, M.tw_shift, &x, &y);
  if (x >= g || y >= g) return;
  const float2* d = reinterpret_cast<const float2*>(M.dlen);
  double sum = 0.0;
  for (int a = 0; a < G.P; ++a) {
    const float2 v = d[dense_pair(M.ntiles, a, tile, lane)];
    sum = __dadd_rn(__dadd_rn(sum, (double)v.x), (double)v.y);
  }
  for_each_exception(M, tile, lane,
                     [&](float l, int, int) { sum = __dadd_rn(sum, (double)l); });
  W[(int64_t)y * g + x] = sum;
}

__global__ void __launch_bounds__(kBlock)
    k_backward64(IterArgs A, int s, const double* __restrict__ cur,
                 double* __restrict__ next, const double* __restrict__ upd,
                 const double* __restrict__ W) {
  const DevGeom& G = A.G;
  const int g = G.C;
  const int64_t g2 = (int64_t)g * g;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int tile = blockIdx.x * 8 + warp;
  if (tile >= A.M.ntiles) return;
  int x, y;
  tile_pixel(tile, lane, A.M.tiles_x, A.M.tw_shift, &x, &y);
  if (x >= g || y >= g) return;
  const int64_t p = (int64_t)y * g + x;
  const bool pen = A.alg >= 2;
  const double rf = cur[(int64_t)(s + A.fshift) * g2 + p];
  const float2* d = reinterpret_cast<const float2*>(A.M.dlen);
  const float xf = (float)x, yf = (float)y;
  double acc = 0.0;
  for (int a = 0; a < G.P; ++a) {
    const float2 v = __ldcs(d + dense_pair(A.M.ntiles, a, tile, lane));
    const bool h0 = __float_as_uint(v.x) != 0u, h1 = __float_as_uint(v.y) != 0u;
    if (!(h0 | h1)) continue;
    const int c0 = window_c0(A.M.wcoef[a], xf, yf);
    const double* ub = upd + (int64_t)a * G.C + c0;
    if (h0)
      acc = pen ? __dsub_rn(acc, __dmul_rn(__dmul_rn(rf, (double)v.x), ub[0]))
                : __dadd_rn(acc, __dmul_rn((double)v.x, ub[0]));
    if (h1)
      acc = pen ? __dsub_rn(acc, __dmul_rn(__dmul_rn(rf, (double)v.y), ub[1]))
                : __dadd_rn(acc, __dmul_rn((double)v.y, ub[1]));
  }
  // segments outside the pixel's window (stored apart)
  for_each_exception(A.M, tile, lane, [&](float l, int ea, int ec) {
    const double u = upd[(int64_t)ea * G.C + ec];
    acc = pen ? __dsub_rn(acc, __dmul_rn(__dmul_rn(rf, (double)l), u))
              : __dadd_rn(acc, __dmul_rn((double)l, u));
  });
  const int ts = s + A.vshift;
  const int64_t at = (int64_t)ts * g2 + p;
  const double old = cur[at];
  const double Wp = W[p];
  double nv;
  if (A.alg == 0) {
    nv = __dadd_rn(old, __ddiv_rn(acc, Wp));
  } else if (A.alg == 1) {
    nv = __dmul_rn(old, __ddiv_rn(acc, Wp));
  } else {
    int up = 0, down = 0;
    if (A.alg == 3) apmlr_axial(A, s, &up, &down);
    double F, Gv;
    penalty_fg(A.alg == 3, A.pw, x, y, g, up, down,
               [&](int dx, int dy, int dz) {
                 return cur[(int64_t)(ts + dz) * g2 + p + dx + (int64_t)dy * g];
               },
               F, Gv);
    Gv = __dadd_rn(Gv, Wp);
    nv = penalised_root(F, Gv, acc);
  }
  next[at] = nv;
}

__global__ void k_convert(const float* __restrict__ in, double* __restrict__ out,
                          int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = (double)in[i];
}
__global__ void k_narrow(const double* __restrict__ in, float* __restrict__ out,
                         int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = (float)in[i];
}
__global__ void k_fill64(double* p, int64_t n, double v) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) p[i] = v;
}

inline int blocks_for(int64_t n) { return (int)((n + kBlock - 1) / kBlock); }

}  // namespace

void launch_forward64(const IterArgs& A, const double* ra2d, const double* recon,
                      const float* sino, double* out, int out_mode,
                      cudaStream_t st) {
  const int ngroups = A.G.P * A.G.gpa;
  k_forward64<<<blocks_for((int64_t)ngroups * 32), kBlock, 0, st>>>(
      A.G, A.M, ra2d, ngroups, recon, sino, out, out_mode);
}

void launch_backward64(const IterArgs& A, int s, const double* cur,
                       double* next, const double* upd, const double* W,
                       cudaStream_t st) {
  k_backward64<<<(A.M.ntiles + 7) / 8, kBlock, 0, st>>>(A, s, cur, next, upd, W);
}

void launch_weights64(const DevGeom& G, const MatrixDev& M, double* W,
                      cudaStream_t st) {
  k_weights64<<<blocks_for((int64_t)M.ntiles * 32), kBlock, 0, st>>>(G, M, W);
}

void launch_convert(const float* in, double* out, int64_t n, cudaStream_t st) {
  if (n) k_convert<<<blocks_for(n), kBlock, 0, st>>>(in, out, n);
}
void launch_narrow(const double* in, float* out, int64_t n, cudaStream_t st) {
  if (n) k_narrow<<<blocks_for(n), kBlock, 0, st>>>(in, out, n);
}
void launch_fill64(double* p, int64_t n, double v, cudaStream_t st) {
  if (n) k_fill64<<<blocks_for(n), kBlock, 0, st>>>(p, n, v);
}

}  // namespace tg
