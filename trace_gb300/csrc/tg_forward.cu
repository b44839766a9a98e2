// Forward projection (ray-driven): one warp per 32-ray group (32 adjacent
// detector columns of one angle), lane = ray. Each lane sums recon[idx]*len
// along its ray in the reference's segment order (CalculateSimdata,
// src/sirt/sirt.cc:4-19) and stores the per-ray factor of the
// backprojection: (ray - sim)/a2 for SIRT (sirt.cc:50-53), ray/sim for
// MLEM/PML/APMLR (mlem.cc:50, pml.cc:234), or sim itself.
//
// K slices share one read of the slice-invariant matrix: slice j of the
// batch is lane j of a K-float vector per pixel, so one gather (a single
// 256-bit load for K = 8) serves all K slices. The matrix rows are streamed
// with evict-first loads so they do not displace the gathered
// reconstruction from L2.
#include "tg_kernels.cuh"

namespace tg {

namespace {

constexpr int kBlock = 256;

template <int LK>
__device__ __forceinline__ float stream_len(const void* base, int64_t e,
                                            float inv_scale) {
  if constexpr (LK == LK_F32)
    return __ldcs(reinterpret_cast<const float*>(base) + e);
  else
    return decode_len<LK>(__ldcs(reinterpret_cast<const uint16_t*>(base) + e),
                          inv_scale);
}

// Per-ray output of the forward kernels: the ray sum (FWD_SIM), SIRT's
// (ray - sim) / a2 (sirt.cc:50) or the ratio ray / sim (mlem.cc:50,
// pml.cc:236, apmlr.cc:1017).
template <int K>
__device__ __forceinline__ void fwd_epilogue(const MatrixDev& M, int64_t r,
                                             const float (&acc)[K], const float* sino,
                                             float* out, int out_mode) {
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

template <int K, int LK, bool EXACT, bool DELTA>
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
#pragma unroll
  for (int j = 0; j < K; ++j) acc[j] = 0.f;
  int idx = 0;
  int64_t cbase = 0;
  uint32_t word = 0;
  if (DELTA) {
    cbase = M.rcoff[grp] + lane;
    if (n > 0) idx = M.rstart[r];
  }
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
      const float l = stream_len<LK>(M.rlen, e, M.inv_scale);
      const Vec<K> v = load_vec<K>(recon + (int64_t)idx * K);
      if constexpr (EXACT) {
#pragma unroll
        for (int j = 0; j < K; ++j) acc[j] = fadd(acc[j], fmul(v.v[j], l));
      } else {
        fma_slices<K>(acc, l, v.v);
      }
    }
  }
  if (!valid) return;
  fwd_epilogue<K>(M, r, acc, sino, out, out_mode);
}

// On-the-fly forward projection: each ray is traced while it is projected
// (tg::trace_ray, the reference's tracer) instead of read from a stored
// matrix. Lengths are the traced float lengths and the sum runs in the
// reference's segment order, so the exact-mode result equals k_forward's
// with f32 lengths bit for bit. No forward matrix is kept on the device;
// the cost moves from streaming the matrix to tracing (ALU).
template <int K, bool EXACT>
__global__ void __launch_bounds__(kBlock)
    k_forward_otf(DevGeom G, MatrixDev M, int ngroups,
                  const float* __restrict__ recon, const float* __restrict__ sino,
                  float* __restrict__ out, int out_mode) {
  const int grp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (grp >= ngroups) return;
  const int a = grp / G.gpa;
  const int c = (grp - a * G.gpa) * 32 + lane;
  if (c >= G.C) return;
  const int64_t r = (int64_t)a * G.C + c;
  float acc[K];
#pragma unroll
  for (int j = 0; j < K; ++j) acc[j] = 0.f;
  trace_ray(G, a, c, [&](int idx, float l, float, int, int) {
    const Vec<K> v = load_vec<K>(recon + (int64_t)idx * K);
    if constexpr (EXACT) {
#pragma unroll
      for (int j = 0; j < K; ++j) acc[j] = fadd(acc[j], fmul(v.v[j], l));
    } else {
      fma_slices<K>(acc, l, v.v);
    }
  });
  fwd_epilogue<K>(M, r, acc, sino, out, out_mode);
}

template <int K, int LK>
void fwd_launch(const IterArgs& A, const float* recon, const float* sino,
                float* out, int out_mode, cudaStream_t st) {
  const int ngroups = A.G.P * A.G.gpa;
  const int blocks = (int)(((int64_t)ngroups * 32 + kBlock - 1) / kBlock);
#define TG_FWD(E, D) \
  k_forward<K, LK, E, D><<<blocks, kBlock, 0, st>>>(A.G, A.M, ngroups, recon, sino, out, out_mode)
  if (A.delta_index) {
    if (A.exact) TG_FWD(true, true); else TG_FWD(false, true);
  } else {
    if (A.exact) TG_FWD(true, false); else TG_FWD(false, false);
  }
#undef TG_FWD
}

template <int K>
void fwd_kind(const IterArgs& A, const float* recon, const float* sino,
              float* out, int out_mode, cudaStream_t st) {
  if (A.M.rlen == nullptr) {  // no stored forward matrix: trace on the fly
    const int ngroups = A.G.P * A.G.gpa;
    const int blocks = (int)(((int64_t)ngroups * 32 + kBlock - 1) / kBlock);
    if (A.exact)
      k_forward_otf<K, true><<<blocks, kBlock, 0, st>>>(A.G, A.M, ngroups, recon, sino,
                                                         out, out_mode);
    else
      k_forward_otf<K, false><<<blocks, kBlock, 0, st>>>(A.G, A.M, ngroups, recon, sino,
                                                          out, out_mode);
    return;
  }
  switch (A.M.len_kind) {
    case LK_F32: fwd_launch<K, LK_F32>(A, recon, sino, out, out_mode, st); break;
    case LK_BF16: fwd_launch<K, LK_BF16>(A, recon, sino, out, out_mode, st); break;
    case LK_F16: fwd_launch<K, LK_F16>(A, recon, sino, out, out_mode, st); break;
    default: fwd_launch<K, LK_U16>(A, recon, sino, out, out_mode, st); break;
  }
}

}  // namespace

void launch_forward(const IterArgs& A, const float* recon_batch,
                    const float* sino_batch, float* out, int out_mode,
                    cudaStream_t st) {
  switch (A.K) {
    case 1: fwd_kind<1>(A, recon_batch, sino_batch, out, out_mode, st); break;
    case 2: fwd_kind<2>(A, recon_batch, sino_batch, out, out_mode, st); break;
    case 4: fwd_kind<4>(A, recon_batch, sino_batch, out, out_mode, st); break;
    case 8: fwd_kind<8>(A, recon_batch, sino_batch, out, out_mode, st); break;
    default: fwd_kind<16>(A, recon_batch, sino_batch, out, out_mode, st); break;
  }
}

}  // namespace tg
