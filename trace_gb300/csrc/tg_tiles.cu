// Tile-staged forward projection (fast mode).
//
// The ray-major forward kernel gathers each segment's K reconstruction values
// through L1/L2: ~1 sector lookup per segment, and at 2048^2 with 8 slices
// the 134 MB batch no longer stays in L2 next to the streamed matrix. Here
// the image is cut into ts x ts tiles (ts = 64 by default; 32 to 96 in steps
// of 16 by plan option) and each ray's segment list into runs
// (consecutive segments inside one tile). One block per tile loads the
// tile's K-slice reconstruction into shared memory once and walks all runs
// through it: lane = run, 32 runs of adjacent rays per warp. A lane's
// lengths are stored in chunks of 8 consecutive steps (one 16-byte load per
// 8 segments for 16-bit codes) with 8 bytes of step deltas per chunk,
// chunks interleaved across the 32 lanes so each chunk load of a warp is one
// contiguous 512-byte row; the next chunk is loaded while the current one is
// consumed. A run's partial sums (K floats, FMA chain in step order) are
// stored, not accumulated, into the run's own slot (TileMatrixDev: slot of
// run k of ray r = pbase[r / 32] + 32 k + r % 32). tg::launch_fwd_finish adds
// a ray's slots in path order and turns the sums into the per-ray factors
// the backprojection reads. No atomics anywhere, so every launch gives the same
// bits; the sum is the reference's sequential ray sum (sirt.cc:10-17)
// regrouped by tile runs, which is why this path is fast mode only.
//
// Construction (once per geometry): runs per ray are counted by the tracing
// pass that counts segments (k_trace_count); then run records keyed by
// (tile, chunk-count class, ray, ordinal) are emitted, radix-sorted (CUB)
// and packed into 32-lane groups per tile, and the groups' streams are
// filled. Emission and fill walk each ray's segments in the stored
// ray-ordered matrix, or trace the ray again when the plan keeps none.
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>
#include <cuda/std/functional>

#include "tg_kernels.cuh"

namespace tg {

namespace {

constexpr int kBlock = 1024;      // forward: at most 32 warps per tile block
constexpr int kTraceBlock = 128;
// Tiles are ts x ts pixels (TileMatrixDev::ts), kept in shared memory with
// row stride ts + 1 (bank spread).
// A step is stored as the signed byte dx + dy * (ts + 1), the change of the
// shared-memory pixel index (dx in {0, 1}, dy in {-1, 0, 1}: -97 .. 98 at
// the largest tile side, 96), so
// the forward walks a run with one byte extraction and one add per step.
// 0 is "stay", never a real step: every unused byte of the stream (a run's
// first step, steps past a run's end, empty lanes) holds it, with a zero
// length. Per lane and chunk the 8 bytes are one 8-byte word pair.

__device__ __forceinline__ int tile_of(int ix, int iy, int tiles_x, TileDiv d) {
  return tile_of_pixel(ix, iy, tiles_x, d);
}

// ---- construction (runs per ray are counted by k_trace_count) ----------------
// The segments of one ray, in order, as f(idx, ix, iy, length, 16-bit length
// code), idx = iy * g + ix:
// read back from the ray-ordered forward matrix when the plan keeps one
// (delta-coded or explicit indices; the stored code is the one encode16 gives
// the traced length, so both sources yield the same tile stream), traced
// again otherwise (forward traced on the fly, or a stray step the 4-bit code
// cannot hold). LEN: which length the caller takes - none (0 and 0 are
// passed; the matrix's lengths are not read), the 16-bit code (the plan's
// 16-bit storage) or the float length (f32 storage).
enum SegSource { kSrcTrace = 0, kSrcDelta = 1, kSrcIndex = 2 };
enum SegLen { kLenNone = 0, kLenCode = 1, kLenFloat = 2 };

template <int SRC, int LEN, class F>
__device__ __forceinline__ void ray_segments(const DevGeom& G, const MatrixDev& M,
                                             int64_t r, F&& f) {
  const int a = (int)(r / G.C), c = (int)(r - (int64_t)a * G.C);
  if constexpr (SRC == kSrcTrace) {
    trace_ray(G, a, c, [&](int idx, float l, float, int ix, int iy) {
      f(idx, ix, iy, l, LEN == kLenCode ? encode16(l, M.len_kind, M.scale) : (uint16_t)0);
    });
  } else {
    const int g = G.C;
    const int grp = a * G.gpa + (c >> 5), lane = c & 31;
    const int n = M.rnseg[r];
    const int64_t base = M.roff[grp] + lane;
    const int64_t cbase = SRC == kSrcDelta ? M.rcoff[grp] + lane : 0;
    const float inv_g = 1.0f / (float)g;
    int idx = (SRC == kSrcDelta && n > 0) ? M.rstart[r] : 0;
    int ix = 0, iy = 0;
    if (SRC == kSrcDelta && n > 0) cell_xy(idx, g, inv_g, ix, iy);
    if constexpr (SRC == kSrcDelta) {
      // chunks of 8 steps (one step-code word, 8 lengths), the next chunk's
      // loads issued before the current one is walked: the walk is a chain
      // of dependent steps, so a load issued at its step would stall it
      struct Chunk {
        uint32_t word;
        uint32_t len[LEN == kLenNone ? 1 : 8];
      };
      auto load = [&](int ch, Chunk& k) {
        const int s0 = ch * 8;
        k.word = __ldcs(M.rcode + cbase + (int64_t)ch * 32);
        if constexpr (LEN != kLenNone) {
#pragma unroll
          for (int j = 0; j < 8; ++j) {
            const int64_t e = base + (int64_t)(s0 + j) * 32;
            k.len[j] = 0u;
            if (s0 + j < n) {
              if constexpr (LEN == kLenCode)
                k.len[j] = __ldcs(reinterpret_cast<const uint16_t*>(M.rlen) + e);
              else
                k.len[j] = __float_as_uint(__ldcs(reinterpret_cast<const float*>(M.rlen) + e));
            }
          }
        }
      };
      Chunk cur{}, nxt{};
      if (n > 0) load(0, cur);
      for (int ch = 0; ch * 8 < n; ++ch) {
        if ((ch + 1) * 8 < n) load(ch + 1, nxt);
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          const int st = ch * 8 + j;
          if (st >= n) break;
          if (st > 0) {
            const uint32_t code = (cur.word >> (4 * j)) & 15u;
            const int dx = (int)(code & 1u), dy = (int)(code >> 1) - 1;
            ix += dx;
            iy += dy;
            idx += dx + dy * g;
          }
          if constexpr (LEN == kLenCode)
            f(idx, ix, iy, 0.f, (uint16_t)cur.len[j]);
          else if constexpr (LEN == kLenFloat)
            f(idx, ix, iy, __uint_as_float(cur.len[j]), (uint16_t)0);
          else
            f(idx, ix, iy, 0.f, (uint16_t)0);
        }
        cur = nxt;
      }
    } else {
      for (int st = 0; st < n; ++st) {
        const int64_t e = base + (int64_t)st * 32;
        idx = __ldcs(M.ridx + e);
        cell_xy(idx, g, inv_g, ix, iy);
        if constexpr (LEN == kLenCode)
          f(idx, ix, iy, 0.f, __ldcs(reinterpret_cast<const uint16_t*>(M.rlen) + e));
        else if constexpr (LEN == kLenFloat)
          f(idx, ix, iy, __ldcs(reinterpret_cast<const float*>(M.rlen) + e), (uint16_t)0);
        else
          f(idx, ix, iy, 0.f, (uint16_t)0);
      }
    }
  }
}

// A run's sort key: (tile, chunk-count class, ray, ordinal). Within a tile
// runs of equal 8-step chunk counts (longest first) share warp groups, so
// the lanes of a group finish together; inside a class the rays stay in
// order (adjacent rays: shared-memory broadcasts).
__device__ __forceinline__ unsigned long long run_key(RunKey rk, int t, int len,
                                                      int64_t r, int k) {
  const int cls = 31 - min((len + 7) >> 3, 31);
  return ((unsigned long long)t << rk.tile_shift()) |
         ((unsigned long long)cls << rk.class_shift()) |
         ((unsigned long long)r << 8) | (unsigned long long)(k & 255);
}

template <int SRC>
__global__ void __launch_bounds__(kTraceBlock)
    k_runs_emit(DevGeom G, MatrixDev M, int tiles_x, TileDiv td, RunKey rk,
                const int64_t* ray_run_off, unsigned long long* key, int* val,
                uint16_t* run_lp, uint16_t* run_len) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= (int64_t)G.P * G.C) return;
  // the ray's first run index, read once (the stores below may alias it as
  // far as the compiler knows, which would reload it at every run)
  const int64_t first = ray_run_off[r];
  int64_t i = first - 1;
  int cur = -1, k = -1, len = 0, px = 0, py = 0;
  auto close = [&]() {
    if (i >= first) {
      run_len[i] = (uint16_t)len;
      key[i] = run_key(rk, cur, len, r, k);
    }
  };
  ray_segments<SRC, kLenNone>(G, M, r, [&](int, int ix, int iy, float, uint16_t) {
    const int t = tile_of(ix, iy, tiles_x, td);
    const bool step_ok = unit_step(ix, iy, px, py);
    px = ix;
    py = iy;
    if (t != cur || !step_ok) {
      close();
      ++i;
      ++k;
      cur = t;
      len = 0;
      val[i] = (int)i;
      const int ts = td.ts;
      run_lp[i] = (uint16_t)((iy - tdiv(iy, td) * ts) * ts + ix - tdiv(ix, td) * ts);
    }
    ++len;
  });
  close();
}

// Per group of 32 rays: its partial-sum slots, 32 per run ordinal up to the
// group's longest run count.
__global__ void k_group_slots(const int* __restrict__ nruns, int64_t R, int64_t* gslots) {
  const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g * 32 >= R) return;
  int most = 0;
  const int64_t end = min(R, g * 32 + 32);
  for (int64_t r = g * 32; r < end; ++r) most = max(most, nruns[r]);
  gslots[g] = (int64_t)most * 32;
}

// Per run group: its tile-stream entries, 256 per chunk of 8 steps.
__global__ void k_group_entries(const int* __restrict__ gsteps, int groups, int64_t* out) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g < groups) out[g] = (int64_t)((gsteps[g] + 7) / 8) * 256;
}

// out[i] = in[i] >> shift, narrowed to T (values checked on the host first).
template <class T>
__global__ void k_shift_narrow(const int64_t* __restrict__ in, T* out, int64_t n, int shift) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = (T)(in[i] >> shift);
}

// First run of every tile in the sorted order (tile_first[ntiles] = nruns):
// run j opens the tiles after the previous run's tile up to its own, the
// last run closes the rest. Replaces per-run counters during emission.
__global__ void k_tile_bounds(RunKey rk, const unsigned long long* skey, int64_t nruns,
                              int ntiles, int* tile_first) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j > nruns) return;
  const int t = j < nruns ? (int)(skey[j] >> rk.tile_shift()) : ntiles;
  const int prev = j > 0 ? (int)(skey[j - 1] >> rk.tile_shift()) : -1;
  for (int u = prev + 1; u <= t; ++u) tile_first[u] = (int)j;
}

// One thread per run, in the sorted order of its tile: rank r in the tile is
// lane r % 32 of the tile's group r / 32.
__global__ void k_runs_group(RunKey rk, const unsigned long long* skey, const int* sval,
                             int64_t nruns, const int* tile_first_run,
                             const int* group_first, const uint16_t* run_lp,
                             const uint16_t* run_len, const int64_t* ray_run_off,
                             const int* pbase, int* gpart, uint16_t* glp,
                             uint16_t* glen, int* gsteps, int* run_slot) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= nruns) return;
  const unsigned long long k = skey[j];
  const int t = (int)(k >> rk.tile_shift());
  const int rank = (int)(j - tile_first_run[t]);
  const int grp = group_first[t] + rank / 32;
  // i: the run's index in emission order (k_runs_emit numbers ray r's runs
  // ray_run_off[r], ray_run_off[r] + 1, ... along the ray), so its ordinal
  // on the ray is i - ray_run_off[r]
  const int i = sval[j];
  const int64_t slot = (int64_t)grp * 32 + rank % 32;
  const int64_t r = (int64_t)((k >> 8) & ((1ull << rk.ray_bits) - 1));
  const int ord = (int)(i - ray_run_off[r]);
  gpart[slot] = pbase[r >> 5] + ord * 32 + (int)(r & 31);
  glp[slot] = run_lp[i];
  glen[slot] = run_len[i];
  run_slot[i] = (int)slot;
  atomicMax(&gsteps[grp], (int)run_len[i]);
}

template <bool L16, int SRC>
__global__ void __launch_bounds__(kTraceBlock)
    k_runs_fill(DevGeom G, MatrixDev M, int tiles_x, TileDiv td, const int64_t* ray_run_off,
                const int* run_slot, const int64_t* gseg_off,
                const int64_t* gcode_off, void* tlen, uint32_t* tcode) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= (int64_t)G.P * G.C) return;
  const int64_t first = ray_run_off[r];  // read once, as in k_runs_emit
  int64_t i = first - 1;
  int cur = -1, s = 0, px = 0, py = 0;
  int64_t lbase = 0, cbase = 0;
  uint32_t w0 = 0, w1 = 0;  // the chunk's step bytes (steps 0-3, 4-7)
  // the current chunk's 8 lengths as a shift register (oldest in the low
  // bits), stored whole: one 16-byte write per chunk and lane (32 for f32)
  uint32_t q[L16 ? 4 : 8] = {};
  auto push = [&](uint32_t v) {
    if constexpr (L16) {
      q[0] = __funnelshift_r(q[0], q[1], 16);
      q[1] = __funnelshift_r(q[1], q[2], 16);
      q[2] = __funnelshift_r(q[2], q[3], 16);
      q[3] = (q[3] >> 16) | (v << 16);
    } else {
#pragma unroll
      for (int k = 0; k < 7; ++k) q[k] = q[k + 1];
      q[7] = v;
    }
  };
  // entries (chunk c, lane, 0..7): chunks of 8 steps, 32 lanes per chunk
  auto store = [&](int c) {
    const int64_t e = lbase + (int64_t)c * 256;
    if constexpr (L16) {
      *reinterpret_cast<uint4*>(reinterpret_cast<uint16_t*>(tlen) + e) =
          make_uint4(q[0], q[1], q[2], q[3]);
    } else {
      uint4* d = reinterpret_cast<uint4*>(reinterpret_cast<float*>(tlen) + e);
      d[0] = make_uint4(q[0], q[1], q[2], q[3]);
      d[1] = make_uint4(q[4], q[5], q[6], q[7]);
    }
    *reinterpret_cast<uint2*>(tcode + cbase + (int64_t)c * 64) = make_uint2(w0, w1);
  };
  auto flush = [&]() {  // a run's last, partial chunk: zero lengths after it
    if (i >= first && (s & 7) != 0) {
      for (int k = s & 7; k < 8; ++k) push(0u);
      store(s >> 3);
    }
  };
  ray_segments<SRC, L16 ? kLenCode : kLenFloat>(
      G, M, r, [&](int, int ix, int iy, float l, uint16_t code) {
    const int t = tile_of(ix, iy, tiles_x, td);
    if (t != cur || !unit_step(ix, iy, px, py)) {
      flush();
      ++i;
      cur = t;
      s = 0;
      w0 = w1 = 0;
      const int slot = run_slot[i];
      const int grp = slot >> 5, lane = slot & 31;
      lbase = gseg_off[grp] + lane * 8;
      cbase = gcode_off[grp] + lane * 2;
    } else {
      const uint32_t b = (uint32_t)((ix - px) + (iy - py) * (td.ts + 1)) & 0xffu;
      if ((s & 7) < 4) w0 |= b << (8 * (s & 3));
      else w1 |= b << (8 * (s & 3));
    }
    push(L16 ? (uint32_t)code : __float_as_uint(l));
    if ((s & 7) == 7) {
      store(s >> 3);
      w0 = w1 = 0;
    }
    px = ix;
    py = iy;
    ++s;
  });
  flush();
}

// ---- forward -------------------------------------------------------------------
// Shared-memory image of one tile: K floats per pixel as K/4 float4 planes
// (K >= 4) or one float/float2 plane, row stride ts + 1 pixels; with H, K
// halves per pixel in one plane (one 16-byte read per segment at K = 8).
template <int K, bool H = false>
struct TilePlanes {
  static constexpr int kPlanes = K >= 4 ? K / 4 : 1;
  static constexpr int kWidth = K >= 4 ? 4 : K;  // floats per plane entry
  static int bytes(int ts) { return ts * (ts + 1) * K * (H ? 2 : 4); }
};

template <int K>
__device__ __forceinline__ void tile_load_half(__half* sm, const float* __restrict__ recon,
                                               int g, int x0, int y0, int ts) {
  const int rs = ts + 1;
  for (int e = threadIdx.x; e < ts * ts; e += blockDim.x) {
    const int ly = e / ts, lx = e - ly * ts;
    const int x = x0 + lx, y = y0 + ly;
    Vec<K> v;
    if (x < g && y < g) {
      v = load_vec<K>(recon + ((int64_t)y * g + x) * K);
    } else {
#pragma unroll
      for (int j = 0; j < K; ++j) v.v[j] = 0.f;
    }
    store_hvec<K>(sm + (ly * rs + lx) * K, v);
  }
}

template <int K>
__device__ __forceinline__ void tile_fma_half(const __half* sm, int si, float l,
                                              float (&acc)[K]) {
  const Vec<K> v = load_hvec<K, true>(sm + si * K);
  fma_slices<K>(acc, l, v.v);
}

template <int K>
__device__ __forceinline__ void tile_load(float* sm, const float* __restrict__ recon,
                                          int g, int x0, int y0, int ts) {
  constexpr int W = TilePlanes<K>::kWidth;
  constexpr int NP = TilePlanes<K>::kPlanes;
  const int rs = ts + 1;
  for (int e = threadIdx.x; e < ts * ts; e += blockDim.x) {
    const int ly = e / ts, lx = e - ly * ts;
    const int x = x0 + lx, y = y0 + ly;
    const int si = ly * rs + lx;
    const bool in = x < g && y < g;
    const float* src = recon + ((int64_t)y * g + x) * K;
#pragma unroll
    for (int pl = 0; pl < NP; ++pl) {
      float* dst = sm + ((size_t)pl * ts * rs + si) * W;
      if constexpr (W == 4) {
        *reinterpret_cast<float4*>(dst) =
            in ? __ldg(reinterpret_cast<const float4*>(src) + pl)
               : make_float4(0.f, 0.f, 0.f, 0.f);
      } else if constexpr (W == 2) {
        *reinterpret_cast<float2*>(dst) =
            in ? __ldg(reinterpret_cast<const float2*>(src)) : make_float2(0.f, 0.f);
      } else {
        *dst = in ? __ldg(src) : 0.f;
      }
    }
  }
}

// plane: floats of one plane (ts * (ts + 1) pixels x plane width)
template <int K>
__device__ __forceinline__ void tile_fma(const float* sm, int si, float l, int plane,
                                         float (&acc)[K]) {
  constexpr int W = TilePlanes<K>::kWidth;
  constexpr int NP = TilePlanes<K>::kPlanes;
#pragma unroll
  for (int pl = 0; pl < NP; ++pl) {
    const float* src = sm + (size_t)pl * plane + (size_t)si * W;
    if constexpr (W == 4) {
      const float4 v = *reinterpret_cast<const float4*>(src);
      acc[pl * 4 + 0] = fmaf(v.x, l, acc[pl * 4 + 0]);
      acc[pl * 4 + 1] = fmaf(v.y, l, acc[pl * 4 + 1]);
      acc[pl * 4 + 2] = fmaf(v.z, l, acc[pl * 4 + 2]);
      acc[pl * 4 + 3] = fmaf(v.w, l, acc[pl * 4 + 3]);
    } else if constexpr (W == 2) {
      const float2 v = *reinterpret_cast<const float2*>(src);
      acc[0] = fmaf(v.x, l, acc[0]);
      acc[1] = fmaf(v.y, l, acc[1]);
    } else {
      acc[0] = fmaf(*src, l, acc[0]);
    }
  }
}

// A run's K partial sums into its slot (streaming stores: the finish kernel
// reads each slot once).
template <int K>
__device__ __forceinline__ void store_part(float* dst, const float (&acc)[K]) {
  if constexpr (K >= 4) {
#pragma unroll
    for (int j = 0; j < K; j += 4)
      __stcs(reinterpret_cast<float4*>(dst + j),
             make_float4(acc[j], acc[j + 1], acc[j + 2], acc[j + 3]));
  } else if constexpr (K == 2) {
    __stcs(reinterpret_cast<float2*>(dst), make_float2(acc[0], acc[1]));
  } else {
    __stcs(dst, acc[0]);
  }
}

// One chunk (8 steps) of a lane's run: lengths + step codes.
template <int LK>
struct Chunk {
  uint4 len[LK == LK_F32 ? 2 : 1];
  uint2 code;  // step bytes
};

template <int LK>
__device__ __forceinline__ void load_chunk(const TileMatrixDev& T, int64_t lb,
                                           int64_t cb, int c, Chunk<LK>& ch) {
  if constexpr (LK == LK_F32) {
    const uint4* p = reinterpret_cast<const uint4*>(
        reinterpret_cast<const float*>(T.tlen) + lb + (int64_t)c * 256);
    ch.len[0] = __ldcs(p);
    ch.len[1] = __ldcs(p + 1);
  } else {
    ch.len[0] = __ldcs(reinterpret_cast<const uint4*>(
        reinterpret_cast<const uint16_t*>(T.tlen) + lb + (int64_t)c * 256));
  }
  ch.code = __ldcs(reinterpret_cast<const uint2*>(T.tcode + cb + (int64_t)c * 64));
}

template <int LK>
__device__ __forceinline__ float chunk_len(const Chunk<LK>& ch, int j,
                                           float inv_scale) {
  if constexpr (LK == LK_F32) {
    const uint4 q = ch.len[j >> 2];
    const uint32_t w = (j & 3) == 0 ? q.x : (j & 3) == 1 ? q.y : (j & 3) == 2 ? q.z : q.w;
    return __uint_as_float(w);
  } else {
    const uint4 q = ch.len[0];
    const uint32_t w = (j >> 1) == 0 ? q.x : (j >> 1) == 1 ? q.y : (j >> 1) == 2 ? q.z : q.w;
    const uint32_t h = (j & 1) ? (w >> 16) : (w & 0xffffu);
    // fixed-point codes stay unscaled here; the run's sums are scaled once
    if constexpr (LK == LK_U16) return u16_to_float(h);
    else return decode_len<LK>((uint16_t)h, inv_scale);
  }
}

// COMP: compensated summation - each chunk's 8 products are an FMA chain
// added to the run's sum with Kahan's correction (the stored partial sum is
// the corrected one).
// One block's work: tile block / splits of matrix T (see k_forward_tiled).
template <int K, int LK, bool H, bool COMP>
__device__ __forceinline__ void forward_tiled_block(const TileMatrixDev& T, int g,
                                                    float inv_scale, int splits, int block,
                                                    const float* __restrict__ recon,
                                                    float* __restrict__ part) {
  extern __shared__ float4 smem4[];
  float* sm = reinterpret_cast<float*>(smem4);
  __half* smh = reinterpret_cast<__half*>(smem4);
  // `splits` blocks share a tile (small grids: fewer tiles than SMs); each
  // loads the tile and takes every splits-th warp group
  const int t = block / splits, sub = block - t * splits;
  const int ts = T.ts, rs = ts + 1;
  const int x0 = (t % T.tiles_x) * ts, y0 = (t / T.tiles_x) * ts;
  const int plane = ts * rs * TilePlanes<K>::kWidth;
  if constexpr (H)
    tile_load_half<K>(smh, recon, g, x0, y0, ts);
  else
    tile_load<K>(sm, recon, g, x0, y0, ts);
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int g0 = T.group_first[t], g1 = T.group_first[t + 1];
  const int nw = blockDim.x >> 5;  // warps of the block (TileMatrixDev::bw)
  for (int grp = g0 + sub * nw + warp; grp < g1; grp += splits * nw) {
    const int slot = grp * 32 + lane;
    const int pslot = T.gpart[slot];
    const int lp = T.glp[slot];
    const int ly = lp / ts;
    int si = ly * rs + (lp - ly * ts);  // shared-memory index of the current pixel
    const int chunks = (T.gsteps[grp] + 7) >> 3;
    const int64_t lb = T.gseg_off[grp] + lane * 8;
    const int64_t cb = T.gcode_off[grp] + lane * 2;
    float acc[K], cmp[K];
#pragma unroll
    for (int j = 0; j < K; ++j) acc[j] = cmp[j] = 0.f;
    Chunk<LK> cur, nxt;
    if (chunks > 0) load_chunk<LK>(T, lb, cb, 0, cur);
    // one chunk's 8 steps into a
    auto chunk_steps = [&](float (&a)[K]) {
      // No per-step guard: a run's first step and every step past its end
      // carry the "stay" step 0 and a zero length (see k_runs_fill), so
      // lanes of shorter runs add 0 * (a finite pixel value) in place.
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        si += (int)(int8_t)((j < 4 ? cur.code.x : cur.code.y) >> (8 * (j & 3)));
        if constexpr (H)
          tile_fma_half<K>(smh, si, chunk_len<LK>(cur, j, inv_scale), a);
        else
          tile_fma<K>(sm, si, chunk_len<LK>(cur, j, inv_scale), plane, a);
      }
    };
    for (int c = 0; c < chunks; ++c) {
      if (c + 1 < chunks) load_chunk<LK>(T, lb, cb, c + 1, nxt);
      if constexpr (COMP) {
        float ca[K];
#pragma unroll
        for (int j = 0; j < K; ++j) ca[j] = 0.f;
        chunk_steps(ca);
#pragma unroll
        for (int j = 0; j < K; ++j) kahan_add(acc[j], cmp[j], ca[j]);
      } else {
        chunk_steps(acc);
      }
      cur = nxt;
    }
    if constexpr (COMP) {
#pragma unroll
      for (int j = 0; j < K; ++j) acc[j] = fsub(acc[j], cmp[j]);
    }
    if constexpr (LK == LK_U16) {
#pragma unroll
      for (int j = 0; j < K; ++j) acc[j] *= inv_scale;
    }
    if (pslot >= 0) store_part<K>(part + (int64_t)pslot * K, acc);
  }
}

template <int K, int LK, bool H, bool COMP>
__global__ void __launch_bounds__(kBlock)
    k_forward_tiled(TileMatrixDev T, int g, float inv_scale, int splits,
                    const float* __restrict__ recon, float* __restrict__ part) {
  forward_tiled_block<K, LK, H, COMP>(T, g, inv_scale, splits, blockIdx.x, recon, part);
}

// Many plans' forward projections in one launch: block -> work item (a
// plan's slice batch) through the items' first blocks, one block per tile.
template <int K, int LK, bool H, bool COMP>
__global__ void __launch_bounds__(kBlock)
    k_forward_tiled_multi(const FwdItem* __restrict__ items, int nitems) {
  const FwdItem& it = items[item_of(items, nitems, blockIdx.x)];
  forward_tiled_block<K, LK, H, COMP>(it.T, it.g, it.inv_scale, 1,
                                      (int)(blockIdx.x - it.first), it.recon, it.part);
}

// A ray's partial sums (its runs' slots, in path order) -> per-ray factor,
// as k_forward's epilogue. FH (ratio factors only): the factor is stored as
// the half (ray/sim - fofs), fofs = factor_offset(storage).
template <int K, bool FH, bool COMP>
__device__ __forceinline__ void fwd_finish_ray(int64_t r, const int* __restrict__ rnrun,
                                               const int* __restrict__ pbase,
                                               const float* __restrict__ ra2,
                                               const float* __restrict__ part,
                                               const float* __restrict__ sino,
                                               float* __restrict__ out, int out_mode,
                                               float fofs) {
  Vec<K> s;
  float cmp[K];
#pragma unroll
  for (int j = 0; j < K; ++j) s.v[j] = cmp[j] = 0.f;
  const int n = rnrun[r];
  // the warp's 32 rays are one ray group: run k of every lane is one row
  const float* src = part + ((int64_t)pbase[r >> 5] + (r & 31)) * K;
  for (int k = 0; k < n; ++k) {
    const Vec<K> v = load_vec_cs<K>(src + (int64_t)k * 32 * K);
#pragma unroll
    for (int j = 0; j < K; ++j) {
      if constexpr (COMP) kahan_add(s.v[j], cmp[j], v.v[j]);
      else s.v[j] = fadd(s.v[j], v.v[j]);
    }
  }
  if constexpr (COMP) {
#pragma unroll
    for (int j = 0; j < K; ++j) s.v[j] = fsub(s.v[j], cmp[j]);
  }
  Vec<K> o;
  if (out_mode == FWD_SIM) {
    o = s;
  } else {
    const Vec<K> ray = load_vec<K>(sino + r * K);
    const float a2 = out_mode == FWD_SIRT ? ra2[r] : 1.f;
#pragma unroll
    for (int j = 0; j < K; ++j)
      o.v[j] = out_mode == FWD_SIRT ? fdiv(fsub(ray.v[j], s.v[j]), a2)
                                    : fdiv(ray.v[j], s.v[j]);
  }
  if constexpr (FH) {
#pragma unroll
    for (int j = 0; j < K; ++j) o.v[j] -= fofs;
    store_hvec<K>(reinterpret_cast<__half*>(out) + r * K, o);
  } else {
    store_vec<K>(out + r * K, o);
  }
}

template <int K, bool FH, bool COMP>
__global__ void k_fwd_finish(int64_t nrays, const int* __restrict__ rnrun,
                             const int* __restrict__ pbase,
                             const float* __restrict__ ra2,
                             const float* __restrict__ part,
                             const float* __restrict__ sino,
                             float* __restrict__ out, int out_mode, float fofs) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r < nrays)
    fwd_finish_ray<K, FH, COMP>(r, rnrun, pbase, ra2, part, sino, out, out_mode, fofs);
}

// Many plans' finishes in one launch: block -> work item, 256 rays a block.
template <int K, bool COMP>
__global__ void k_fwd_finish_multi(const FinItem* __restrict__ items, int nitems) {
  const FinItem& it = items[item_of(items, nitems, blockIdx.x)];
  const int64_t r = (int64_t)(blockIdx.x - it.first) * blockDim.x + threadIdx.x;
  if (r >= it.nrays) return;
  if (it.fh != FACT_F32)
    fwd_finish_ray<K, true, COMP>(r, it.rnrun, it.pbase, it.ra2, it.part, it.sino, it.out,
                                  it.out_mode, factor_offset(it.fh));
  else
    fwd_finish_ray<K, false, COMP>(r, it.rnrun, it.pbase, it.ra2, it.part, it.sino, it.out,
                                   it.out_mode, 0.f);
}

template <int K, int LK, bool H, bool COMP>
void fwd_tiled_launch(const TileMatrixDev& T, int g, float inv_scale,
                      const float* recon, float* part, cudaStream_t st) {
  const int smem = TilePlanes<K, H>::bytes(T.ts);
  cudaFuncSetAttribute(k_forward_tiled<K, LK, H, COMP>,
                       cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  // at least two blocks per SM when the grid has few tiles
  int sms = 0, dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int splits = max(1, min(16, (2 * sms + T.ntiles - 1) / T.ntiles));
  k_forward_tiled<K, LK, H, COMP><<<T.ntiles * splits, T.bw * 32, smem, st>>>(
      T, g, inv_scale, splits, recon, part);
}

template <int K, bool H, bool COMP>
void fwd_tiled_kind(const TileMatrixDev& T, int g, int len_kind, float inv_scale,
                    const float* recon, float* part, cudaStream_t st) {
  switch (len_kind) {
    case LK_F32: fwd_tiled_launch<K, LK_F32, H, COMP>(T, g, inv_scale, recon, part, st); break;
    case LK_BF16: fwd_tiled_launch<K, LK_BF16, H, COMP>(T, g, inv_scale, recon, part, st); break;
    case LK_F16: fwd_tiled_launch<K, LK_F16, H, COMP>(T, g, inv_scale, recon, part, st); break;
    default: fwd_tiled_launch<K, LK_U16, H, COMP>(T, g, inv_scale, recon, part, st); break;
  }
}

template <int K, bool COMP>
void fwd_tiled_half(const IterArgs& A, const TileMatrixDev& T, const float* recon,
                    float* part, cudaStream_t st) {
  // an f32 tile of 16 slices would not fit shared memory (plan creation
  // requires half_gathers with 16 slices per pass and forward_tiles)
  if (K == 16 || A.half_tile)
    fwd_tiled_kind<K, true, COMP>(T, A.G.C, A.M.len_kind, A.M.inv_scale, recon, part, st);
  else if constexpr (K != 16)
    fwd_tiled_kind<K, false, COMP>(T, A.G.C, A.M.len_kind, A.M.inv_scale, recon, part, st);
}

// compensated sums: up to 8 slices per pass (plan creation checks)
template <int K>
void fwd_tiled_comp(const IterArgs& A, const TileMatrixDev& T, const float* recon,
                    float* part, cudaStream_t st) {
  constexpr bool kComp = K <= 8;
  if (kComp && A.comp) fwd_tiled_half<K, kComp>(A, T, recon, part, st);
  else fwd_tiled_half<K, false>(A, T, recon, part, st);
}

inline int blocks_for(int64_t n, int b) { return (int)((n + b - 1) / b); }

}  // namespace

static int seg_source(const MatrixDev& M) {
  if (M.rlen == nullptr) return kSrcTrace;
  return M.rcode != nullptr ? kSrcDelta : kSrcIndex;
}

void launch_runs_emit(const DevGeom& G, const MatrixDev& M, int tiles_x, int ts, RunKey rk,
                      const int64_t* ray_run_off, unsigned long long* key, int* val,
                      uint16_t* run_lp, uint16_t* run_len, cudaStream_t st) {
  const int64_t R = (int64_t)G.P * G.C;
  const int blocks = blocks_for(R, kTraceBlock);
  const TileDiv td = make_tile_div(ts);
  switch (seg_source(M)) {
    case kSrcDelta:
      k_runs_emit<kSrcDelta><<<blocks, kTraceBlock, 0, st>>>(
          G, M, tiles_x, td, rk, ray_run_off, key, val, run_lp, run_len);
      break;
    case kSrcIndex:
      k_runs_emit<kSrcIndex><<<blocks, kTraceBlock, 0, st>>>(
          G, M, tiles_x, td, rk, ray_run_off, key, val, run_lp, run_len);
      break;
    default:
      k_runs_emit<kSrcTrace><<<blocks, kTraceBlock, 0, st>>>(
          G, M, tiles_x, td, rk, ray_run_off, key, val, run_lp, run_len);
  }
}

int sort_runs(unsigned long long* key_in, unsigned long long* key_out,
              int* val_in, int* val_out, int64_t n, int end_bit,
              cudaStream_t st) {
  size_t bytes = 0;
  if (n > 0x7fffffff) return 3;
  cub::DeviceRadixSort::SortPairs(nullptr, bytes, key_in, key_out, val_in, val_out,
                                  (int)n, 0, end_bit, st);
  void* tmp = nullptr;
  if (cudaMalloc(&tmp, bytes) != cudaSuccess) return 1;
  cub::DeviceRadixSort::SortPairs(tmp, bytes, key_in, key_out, val_in, val_out,
                                  (int)n, 0, end_bit, st);
  cudaStreamSynchronize(st);
  cudaFree(tmp);
  return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

// Exclusive prefix sums for the construction (CUB); tmp == nullptr asks for
// the temporary bytes in *tmp_bytes.
cudaError_t scan_counts(void* tmp, size_t* tmp_bytes, const int* in, int64_t* out, int n,
                        cudaStream_t st) {
  return cub::DeviceScan::ExclusiveScan(tmp, *tmp_bytes, in, out,
                                        ::cuda::std::plus<int64_t>{}, (int64_t)0, n, st);
}
cudaError_t scan_i64(void* tmp, size_t* tmp_bytes, const int64_t* in, int64_t* out, int n,
                     cudaStream_t st) {
  return cub::DeviceScan::ExclusiveSum(tmp, *tmp_bytes, in, out, n, st);
}

void launch_group_slots(const int* nruns, int64_t R, int64_t* gslots, cudaStream_t st) {
  const int64_t groups = (R + 31) / 32;
  k_group_slots<<<blocks_for(groups, 256), 256, 0, st>>>(nruns, R, gslots);
}

void launch_group_entries(const int* gsteps, int groups, int64_t* out, cudaStream_t st) {
  k_group_entries<<<blocks_for(groups, 256), 256, 0, st>>>(gsteps, groups, out);
}

void launch_shift_narrow_i32(const int64_t* in, int* out, int64_t n, int shift,
                             cudaStream_t st) {
  k_shift_narrow<int><<<blocks_for(n, 256), 256, 0, st>>>(in, out, n, shift);
}

void launch_shift_i64(const int64_t* in, int64_t* out, int64_t n, int shift,
                      cudaStream_t st) {
  k_shift_narrow<int64_t><<<blocks_for(n, 256), 256, 0, st>>>(in, out, n, shift);
}

void launch_tile_bounds(RunKey rk, const unsigned long long* skey, int64_t nruns,
                        int ntiles, int* tile_first, cudaStream_t st) {
  k_tile_bounds<<<blocks_for(nruns + 1, 256), 256, 0, st>>>(rk, skey, nruns, ntiles,
                                                            tile_first);
}

void launch_runs_group(RunKey rk, const unsigned long long* skey, const int* sval,
                       int64_t nruns, const int* tile_first_run,
                       const int* group_first, const uint16_t* run_lp,
                       const uint16_t* run_len, const int64_t* ray_run_off,
                       const int* pbase, int* gpart, uint16_t* glp,
                       uint16_t* glen, int* gsteps, int* run_slot, cudaStream_t st) {
  k_runs_group<<<blocks_for(nruns, 256), 256, 0, st>>>(
      rk, skey, sval, nruns, tile_first_run, group_first, run_lp, run_len, ray_run_off,
      pbase, gpart, glp, glen, gsteps, run_slot);
}

template <bool L16>
static void runs_fill(const DevGeom& G, const MatrixDev& M, int tiles_x, int ts,
                      const int64_t* ray_run_off, const int* run_slot,
                      const int64_t* gseg_off, const int64_t* gcode_off, void* tlen,
                      uint32_t* tcode, cudaStream_t st) {
  const int64_t R = (int64_t)G.P * G.C;
  const int blocks = blocks_for(R, kTraceBlock);
  const TileDiv td = make_tile_div(ts);
  switch (seg_source(M)) {
    case kSrcDelta:
      k_runs_fill<L16, kSrcDelta><<<blocks, kTraceBlock, 0, st>>>(
          G, M, tiles_x, td, ray_run_off, run_slot, gseg_off, gcode_off, tlen, tcode);
      break;
    case kSrcIndex:
      k_runs_fill<L16, kSrcIndex><<<blocks, kTraceBlock, 0, st>>>(
          G, M, tiles_x, td, ray_run_off, run_slot, gseg_off, gcode_off, tlen, tcode);
      break;
    default:
      k_runs_fill<L16, kSrcTrace><<<blocks, kTraceBlock, 0, st>>>(
          G, M, tiles_x, td, ray_run_off, run_slot, gseg_off, gcode_off, tlen, tcode);
  }
}

void launch_runs_fill(const DevGeom& G, const MatrixDev& M, int tiles_x, int ts,
                      const int64_t* ray_run_off, const int* run_slot,
                      const int64_t* gseg_off, const int64_t* gcode_off,
                      void* tlen, uint32_t* tcode, cudaStream_t st) {
  if (M.len_kind != LK_F32)
    runs_fill<true>(G, M, tiles_x, ts, ray_run_off, run_slot, gseg_off, gcode_off, tlen,
                    tcode, st);
  else
    runs_fill<false>(G, M, tiles_x, ts, ray_run_off, run_slot, gseg_off, gcode_off, tlen,
                     tcode, st);
}

void launch_forward_tiled(const IterArgs& A, const TileMatrixDev& T,
                          const float* recon_batch, float* part, cudaStream_t st) {
  switch (A.K) {
    case 1: fwd_tiled_comp<1>(A, T, recon_batch, part, st); break;
    case 2: fwd_tiled_comp<2>(A, T, recon_batch, part, st); break;
    case 4: fwd_tiled_comp<4>(A, T, recon_batch, part, st); break;
    case 8: fwd_tiled_comp<8>(A, T, recon_batch, part, st); break;
    default: fwd_tiled_comp<16>(A, T, recon_batch, part, st); break;
  }
}

template <int K>
void fwd_finish_k(const IterArgs& A, const TileMatrixDev& T, const float* part,
                  const float* sino, float* out, int out_mode, cudaStream_t st) {
  const int64_t R = (int64_t)A.G.P * A.G.C;
  const int b = blocks_for(R, 256);
#define TG_FINISH(FH, CP)                                                     \
  k_fwd_finish<K, FH, CP><<<b, 256, 0, st>>>(R, T.rnrun, T.pbase, A.M.ra2, part, sino, \
                                             out, out_mode, factor_offset(A.half_factors))
  const bool fh = A.half_factors != FACT_F32 && out_mode == FWD_RATIO;
  constexpr bool kComp = K <= 8;
  if (kComp && A.comp) {
    if (fh) TG_FINISH(true, kComp); else TG_FINISH(false, kComp);
  } else {
    if (fh) TG_FINISH(true, false); else TG_FINISH(false, false);
  }
#undef TG_FINISH
}

void launch_fwd_finish(const IterArgs& A, const TileMatrixDev& T, const float* part,
                       const float* sino, float* out, int out_mode, cudaStream_t st) {
  switch (A.K) {
    case 1: fwd_finish_k<1>(A, T, part, sino, out, out_mode, st); break;
    case 2: fwd_finish_k<2>(A, T, part, sino, out, out_mode, st); break;
    case 4: fwd_finish_k<4>(A, T, part, sino, out, out_mode, st); break;
    case 8: fwd_finish_k<8>(A, T, part, sino, out, out_mode, st); break;
    default: fwd_finish_k<16>(A, T, part, sino, out, out_mode, st); break;
  }
}

template <int K, int LK, bool H, bool COMP>
static void fwd_multi_launch(const FwdItem* items, int n, int64_t blocks, int ts, int bw,
                             cudaStream_t st) {
  const int smem = TilePlanes<K, H>::bytes(ts);
  cudaFuncSetAttribute(k_forward_tiled_multi<K, LK, H, COMP>,
                       cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  k_forward_tiled_multi<K, LK, H, COMP><<<(unsigned)blocks, bw * 32, smem, st>>>(items, n);
}

// the multi-plan path serves 16-bit fixed-point lengths only
template <int K, bool H, bool COMP>
static void fwd_multi_kind(const FwdItem* items, int n, int64_t blocks, int ts, int bw,
                           cudaStream_t st) {
  fwd_multi_launch<K, LK_U16, H, COMP>(items, n, blocks, ts, bw, st);
}

template <int K>
static void fwd_multi_k(const FwdItem* items, int n, int64_t blocks, int ts, int bw,
                        int half_tile, int comp, cudaStream_t st) {
  constexpr bool kComp = K <= 8;
  if (K == 16 || half_tile) {
    if (kComp && comp) fwd_multi_kind<K, true, kComp>(items, n, blocks, ts, bw, st);
    else fwd_multi_kind<K, true, false>(items, n, blocks, ts, bw, st);
  } else if constexpr (K != 16) {
    if (comp) fwd_multi_kind<K, false, true>(items, n, blocks, ts, bw, st);
    else fwd_multi_kind<K, false, false>(items, n, blocks, ts, bw, st);
  }
}

void launch_forward_tiled_multi(const FwdItem* items, int n, int64_t blocks, int K, int ts,
                                int bw, int half_tile, int comp, cudaStream_t st) {
  switch (K) {
    case 1: fwd_multi_k<1>(items, n, blocks, ts, bw, half_tile, comp, st); break;
    case 2: fwd_multi_k<2>(items, n, blocks, ts, bw, half_tile, comp, st); break;
    case 4: fwd_multi_k<4>(items, n, blocks, ts, bw, half_tile, comp, st); break;
    case 8: fwd_multi_k<8>(items, n, blocks, ts, bw, half_tile, comp, st); break;
    default: fwd_multi_k<16>(items, n, blocks, ts, bw, half_tile, comp, st); break;
  }
}

template <int K>
static void finish_multi_k(const FinItem* items, int n, int64_t blocks, int comp,
                           cudaStream_t st) {
  constexpr bool kComp = K <= 8;
  if (kComp && comp) k_fwd_finish_multi<K, kComp><<<(unsigned)blocks, 256, 0, st>>>(items, n);
  else k_fwd_finish_multi<K, false><<<(unsigned)blocks, 256, 0, st>>>(items, n);
}

void launch_fwd_finish_multi(const FinItem* items, int n, int64_t blocks, int K, int comp,
                             cudaStream_t st) {
  switch (K) {
    case 1: finish_multi_k<1>(items, n, blocks, comp, st); break;
    case 2: finish_multi_k<2>(items, n, blocks, comp, st); break;
    case 4: finish_multi_k<4>(items, n, blocks, comp, st); break;
    case 8: finish_multi_k<8>(items, n, blocks, comp, st); break;
    default: finish_multi_k<16>(items, n, blocks, comp, st); break;
  }
}

}  // namespace tg
