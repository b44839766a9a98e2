// Tracing kernels: one thread per ray, one warp per 32 adjacent detector
// columns of one angle. They build, once per geometry, the two device forms
// of the system matrix the iterations stream:
//   * forward (ray-major): each ray's segments in the reference's order,
//     stored step-interleaved across the 32 rays of a warp so that every
//     load of the forward projection is one coalesced 128-byte row;
//   * backward (angle, pixel)-major: for every pixel and angle the lengths of
//     the (at most two) rays crossing it, in column order.
// The tracer itself (tg::trace_ray) reproduces src/common/trace_utils.cc:48-216.
#include "tg_kernels.cuh"

namespace tg {

namespace {

constexpr int kTraceBlock = 128;

__global__ void __launch_bounds__(kTraceBlock)
    k_trace_count(DevGeom G, int ngroups, int* nseg, int* rcap,
                  unsigned* maxlen_bits, int tiles_x, TileDiv td, int* ray_nruns) {
  const int grp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (grp >= ngroups) return;  // warp-uniform
  const int a = grp / G.gpa;
  const int c = (grp - a * G.gpa) * 32 + lane;
  int n = 0;
  // the longest segment: the square root is monotone and correctly rounded,
  // so the root of the largest squared length is the largest length (one
  // root per ray instead of one per segment)
  float ml2 = 0.f;
  if (c < G.C) {
    if (ray_nruns) {
      int runs = 0, cur = -1, px = 0, py = 0;
      n = trace_ray(G, a, c, [&](int, float, float l2, int ix, int iy) {
        ml2 = fmaxf(ml2, l2);
        const int t = tile_of_pixel(ix, iy, tiles_x, td);
        if (t != cur || !unit_step(ix, iy, px, py)) {
          ++runs;
          cur = t;
        }
        px = ix;
        py = iy;
      });
      ray_nruns[(int64_t)a * G.C + c] = runs;
    } else {
      n = trace_ray(G, a, c, [&](int, float, float l2, int, int) { ml2 = fmaxf(ml2, l2); });
    }
    nseg[(int64_t)a * G.C + c] = n;
  }
  const int cap = warp_max_i(n);
  const float m = fsqrt(warp_max_f(ml2));
  if (lane == 0) {
    rcap[grp] = cap;
    atomicMax(maxlen_bits, __float_as_uint(m));  // lengths are >= 0
  }
}

// F64: also the FP64 total of the squared lengths per ray (FP64 plans only:
// GB300's double-precision rate is a small fraction of its single one).
template <bool L16, bool DELTA, bool F64>
__global__ void __launch_bounds__(kTraceBlock)
    k_trace_fill(DevGeom G, MatrixDev M, int ngroups, int* ridx,
                 uint32_t* rcode, int* rstart, void* rlen, float* ra2,
                 double* ra2d, void* dlen, unsigned long long* overflow,
                 int4* exc, int* exc_tile, int exc_cap) {
  const int grp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (grp >= ngroups) return;
  const int a = grp / G.gpa;
  const int c = (grp - a * G.gpa) * 32 + lane;
  if (c >= G.C) return;
  const int64_t r = (int64_t)a * G.C + c;
  const int64_t base = M.roff[grp] + lane;
  const float4 coef = M.wcoef[a];
  const int64_t cbase = DELTA ? M.rcoff[grp] + lane : 0;
  float a2 = 0.f;
  double a2d = 0.0;
  int s = 0, pix = 0, piy = 0;
  uint32_t word = 0;
  unsigned long long bad = 0;
  const bool store_fwd = rlen != nullptr;  // no forward matrix when traced on the fly
  trace_ray(G, a, c, [&](int idx, float l, float l2, int ix, int iy) {
    const int64_t e = base + (int64_t)s * 32;
    if (!store_fwd) {
    } else if (DELTA) {
      if (s == 0) {
        rstart[r] = idx;
      } else {
        const int dx = ix - pix, dy = iy - piy;
        if (dx < 0 || dx > 1 || dy < -1 || dy > 1) ++bad;
        word |= (uint32_t)(dx | ((dy + 1) << 1)) << (4 * (s & 7));
      }
      if ((s & 7) == 7) {
        rcode[cbase + (int64_t)(s >> 3) * 32] = word;
        word = 0;
      }
    } else {
      ridx[e] = idx;
    }
    pix = ix;
    piy = iy;
    if (!store_fwd) {
    } else if (L16) {
      reinterpret_cast<uint16_t*>(rlen)[e] = encode16(l, M.len_kind, M.scale);
    } else {
      reinterpret_cast<float*>(rlen)[e] = l;
    }
    a2 = fadd(a2, l2);
    if constexpr (F64) a2d = __dadd_rn(a2d, (double)l2);
    // backward matrix: slot = column offset inside the pixel's window
    const int slot = c - window_c0(coef, (float)ix, (float)iy);
    if (slot < 0 || slot > 1) {
      // an exception entry (overflow[2] counts them; past the capacity the
      // plan is refused)
      int tile, tl;
      pixel_tile(ix, iy, M.tiles_x, M.tw_shift, &tile, &tl);
      const unsigned long long k = atomicAdd(overflow + 2, 1ull);
      if (k < (unsigned long long)exc_cap) {
        exc[k] = make_int4(tl, a, c, __float_as_int(l));
        exc_tile[k] = tile;
      }
    } else {
      // A present entry never stores +0: a zero length is kept as -0 so the
      // backprojection still visits it (0 * a non-finite factor is NaN in
      // the reference too). The 16-bit fixed-point code has no -0.
      int tile, tl;
      pixel_tile(ix, iy, M.tiles_x, M.tw_shift, &tile, &tl);
      const int64_t pos = dense_pair(M.ntiles, a, tile, tl) * 2 + slot;
      if (L16) {
        uint16_t* d = reinterpret_cast<uint16_t*>(dlen);
        const float cur = decode16(d[pos], M.dlen_kind, M.inv_scale);
        uint16_t code = encode16(cur + l, M.dlen_kind, M.scale);
        if (code == 0 && M.dlen_kind != LK_U16) code = 0x8000u;
        d[pos] = code;
      } else {
        float* d = reinterpret_cast<float*>(dlen);
        const float nv = fadd(d[pos], l);
        d[pos] = (__float_as_uint(nv) == 0u) ? -0.0f : nv;
      }
    }
    ++s;
  });
  if (store_fwd && DELTA && (s & 7) != 0 && s > 0)
    rcode[cbase + (int64_t)(s >> 3) * 32] = word;
  ra2[r] = a2;
  if constexpr (F64) ra2d[r] = a2d;
  if (bad) {  // step codes that do not fit 4 bits
    atomicAdd(overflow, bad);
    // the first offending ray (lowest angle, then column) for the message
    atomicMin(overflow + 1, ((unsigned long long)a << 32) | (unsigned)c);
  }
}

// Total length through each pixel: the reference's replica[2p+1]
// (sirt.cc:59), identical for every slice, so computed once.
// HALF: also Wh, the sum of the lengths each rounded to an IEEE half, as
// the backprojection with half factors multiplies them (its total-length
// normaliser, so that its lengths are one consistent set), in the same pass.
template <bool L16, bool HALF>
__global__ void k_weights(DevGeom G, MatrixDev M, int exact, float* W, float* Wh) {
  const int g = G.C;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)M.ntiles * 32) return;
  const int tile = (int)(t >> 5), lane = (int)(t & 31);
  int x, y;
  tile_pixel(tile, lane, M.tiles_x, M.tw_shift, &x, &y);
  if (x >= g || y >= g) return;
  const int64_t p = (int64_t)y * g + x;
  float sum = 0.f, comp = 0.f, sumh = 0.f, comph = 0.f;
  // compensated (Kahan) sum
  auto kahan = [](float& s, float& cm, float l) {
    const float yk = l - cm, tk = s + yk;
    cm = (tk - s) - yk;
    s = tk;
  };
  auto add = [&](float l0, float l1) {
    if constexpr (HALF) {
      kahan(sumh, comph, __half2float(__float2half_rn(l0)));
      kahan(sumh, comph, __half2float(__float2half_rn(l1)));
    }
    if (exact) {
      sum = fadd(fadd(sum, l0), l1);
    } else {
      kahan(sum, comp, l0);
      kahan(sum, comp, l1);
    }
  };
  // four angles per load (the lane's 16 or 32 contiguous bytes), in angle
  // order; the padding angles past P are not added
  for (int a4 = 0; a4 < G.P; a4 += 4) {
    const int64_t pos = dense_pair(M.ntiles, a4, tile, lane);  // pair index
    const int na = min(4, G.P - a4);
    if (L16) {
      const uint4 q = reinterpret_cast<const uint4*>(M.dlen)[pos >> 2];
      const uint32_t w[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
      for (int j = 0; j < 4; ++j)
        if (j < na)
          add(decode16((uint16_t)(w[j] & 0xffffu), M.dlen_kind, M.inv_scale),
              decode16((uint16_t)(w[j] >> 16), M.dlen_kind, M.inv_scale));
    } else {
      const float4* v = reinterpret_cast<const float4*>(M.dlen) + (pos >> 1);
      const float4 u0 = v[0], u1 = v[1];
      if (na > 0) add(u0.x, u0.y);
      if (na > 1) add(u0.z, u0.w);
      if (na > 2) add(u1.x, u1.y);
      if (na > 3) add(u1.z, u1.w);
    }
  }
  for_each_exception(M, tile, lane, [&](float l, int, int) {
    if constexpr (HALF) kahan(sumh, comph, __half2float(__float2half_rn(l)));
    if (exact) {
      sum = fadd(sum, l);
    } else {
      kahan(sum, comp, l);
    }
  });
  W[p] = sum;
  if constexpr (HALF) Wh[p] = sumh;
}

__global__ void __launch_bounds__(kTraceBlock)
    k_trace_export(DevGeom G, int nrays, const int64_t* offsets, int* idx,
                   float* len, float* len2) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nrays) return;
  const int a = (int)(r / G.C), c = (int)(r - (int64_t)a * G.C);
  int64_t o = offsets[r];
  trace_ray(G, a, c, [&](int i, float l, float l2, int, int) {
    idx[o] = i;
    len[o] = l;
    if (len2) len2[o] = l2;
    ++o;
  });
}

}  // namespace

void launch_trace_count(const DevGeom& G, int* nseg, int* rcap,
                        unsigned* maxlen_bits, int tiles_x, int ts, int* ray_nruns,
                        cudaStream_t st) {
  const int ngroups = G.P * G.gpa;
  const int blocks = (ngroups * 32 + kTraceBlock - 1) / kTraceBlock;
  k_trace_count<<<blocks, kTraceBlock, 0, st>>>(G, ngroups, nseg, rcap, maxlen_bits,
                                                 tiles_x, make_tile_div(ts), ray_nruns);
}

void launch_trace_fill(const DevGeom& G, const MatrixDev& M, int* ridx,
                       uint32_t* rcode, int* rstart, void* rlen, float* ra2,
                       double* ra2d, void* dlen, unsigned long long* overflow,
                       int4* exc, int* exc_tile, int exc_cap, cudaStream_t st) {
  const int ngroups = G.P * G.gpa;
  const int blocks = (ngroups * 32 + kTraceBlock - 1) / kTraceBlock;
  const bool l16 = M.len_kind != LK_F32;
  const bool delta = rcode != nullptr;
#define TG_FILL(L, D, F)                                                          \
  k_trace_fill<L, D, F><<<blocks, kTraceBlock, 0, st>>>(                          \
      G, M, ngroups, ridx, rcode, rstart, rlen, ra2, ra2d, dlen, overflow, exc,   \
      exc_tile, exc_cap)
  if (ra2d) {  // FP64 plans (f32 lengths and explicit indices, checked at creation)
    TG_FILL(false, false, true);
  } else if (l16 && delta) {
    TG_FILL(true, true, false);
  } else if (l16) {
    TG_FILL(true, false, false);
  } else if (delta) {
    TG_FILL(false, true, false);
  } else {
    TG_FILL(false, false, false);
  }
#undef TG_FILL
}

void launch_weights(const DevGeom& G, const MatrixDev& M, int exact, float* W,
                    float* Wh, cudaStream_t st) {
  const int blocks = (int)(((int64_t)M.ntiles * 32 + 255) / 256);
  if (M.len_kind != LK_F32) {
    if (Wh)
      k_weights<true, true><<<blocks, 256, 0, st>>>(G, M, exact, W, Wh);
    else
      k_weights<true, false><<<blocks, 256, 0, st>>>(G, M, exact, W, Wh);
  } else {
    if (Wh)
      k_weights<false, true><<<blocks, 256, 0, st>>>(G, M, exact, W, Wh);
    else
      k_weights<false, false><<<blocks, 256, 0, st>>>(G, M, exact, W, Wh);
  }
}

void launch_trace_export(const DevGeom& G, const int64_t* offsets, int* idx,
                         float* len, float* len2, cudaStream_t st) {
  const int nrays = G.P * G.C;
  k_trace_export<<<(nrays + kTraceBlock - 1) / kTraceBlock, kTraceBlock, 0,
                   st>>>(G, nrays, offsets, idx, len, len2);
}

}  // namespace tg
