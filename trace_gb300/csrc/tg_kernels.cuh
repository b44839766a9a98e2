// Kernel launchers shared between the kernel translation units and the plan
// (host) code.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "tg_device.cuh"
#include "tg_penalty.cuh"

namespace tg {

// Device view of the traced system matrix of one geometry.
struct MatrixDev {
  // forward matrix, ray-major, one 32-ray group (32 adjacent columns of one
  // angle) per warp; entry (group, step, lane) at roff[group] + step*32 + lane
  const int64_t* roff;
  const int* rcap;     // steps per group (max segment count of its rays)
  const int* rnseg;    // [P*C] segments per ray
  const int* ridx;     // pixel index per entry (explicit form)
  const uint32_t* rcode;  // delta form: 8 x 4-bit steps per word per lane
  const int64_t* rcoff;   // delta form: word offset per group
  const int* rstart;      // delta form: [P*C] first pixel of each ray
  const void* rlen;    // length per entry (float or 16-bit code)
  const float* ra2;    // [P*C] sum of squared lengths (SIRT's a2)
  // backward matrix, angle-major over 32-pixel tiles (pixel_tile: 16x2, 8x4
  // or 4x8 pixels): for pixel (x, y) in tile t at lane l, the pair of angle a
  // at dense_pair(ntiles, a, t, l) holds the lengths of rays (a, window_c0)
  // and (a, window_c0 + 1) through the pixel
  const void* dlen;
  const float4* wcoef; // [P4] window coefficients {-sin, cos, D, 0}
  // segments outside their pixel's two-column window (rare: the reference's
  // tracer puts a stray segment far from its ray at some near-vertical
  // angles): per pixel tile t, entries exc[exc_first[t] .. exc_first[t+1]) =
  // {lane, angle, column, length bits}; exc_first == nullptr when none
  const int* exc_first;
  const int4* exc;
  int tiles_x, ntiles;
  int tw_shift;        // backward tiles are 2^tw_shift pixels wide
  int P4;              // angles rounded up to a multiple of 4 (padding empty)
  const float* W;      // [g*g] total length through each pixel
  const float* Wh;     // [g*g] the same over half-rounded lengths (half_gathers)
  int len_kind;        // LenKind of the forward matrices
  // LenKind of the backward matrix: IEEE halves with half gathers (the
  // backprojection's mixed-precision FMAs take them as stored), else len_kind
  int dlen_kind;
  float scale, inv_scale;
};

// Tile-staged forward matrix (tg_tiles.cu): per ts x ts tile, groups of 32
// runs (consecutive segments of one ray inside the tile), lane = run. The
// tile side ts is a plan choice (32 to 96 in steps of 16; a step inside a
// tile is one signed byte dx + dy * (ts + 1), so ts + 1 <= 127).
constexpr int kTileSide = 64;

// Division by the tile side without an integer divide (the construction
// kernels take it for every segment): q = umulhi(v, m), m = ceil(2^32 / ts),
// exact for 0 <= v < 2^32 / ts, because v * (m * ts - 2^32) < 2^32 keeps
// the error of v * m / 2^32 below 1 / ts, the smallest distance from v / ts
// up to the next integer.
struct TileDiv {
  int ts;
  uint32_t m;
};
inline TileDiv make_tile_div(int ts) {
  return TileDiv{ts, 0xFFFFFFFFu / (uint32_t)(ts > 0 ? ts : 1) + 1u};
}
__device__ __forceinline__ int tdiv(int v, TileDiv d) {
  return (int)__umulhi((uint32_t)v, d.m);
}
__device__ __forceinline__ int tile_of_pixel(int ix, int iy, int tiles_x, TileDiv d) {
  return tdiv(iy, d) * tiles_x + tdiv(ix, d);
}

// A 4-bit step code holds (dx, dy) in {0,1} x {-1,0,1}. The reference's
// tracer can emit a segment far from the previous one (float rounding with
// the source a million units away, at near-vertical angles on the edge
// columns): such a step starts a new run, as a tile change does.
__device__ __forceinline__ bool unit_step(int ix, int iy, int px, int py) {
  const int dx = ix - px, dy = iy - py;
  return dx >= 0 && dx <= 1 && dy >= -1 && dy <= 1;
}
// Each run's partial sums (K floats) go to a slot fixed at construction:
// rays are taken in groups of 32 (ray r in group r / 32 at lane r % 32), and
// run k of ray r (k-th in the order its path crosses the tiles) has slot
// pbase[r / 32] + k * 32 + r % 32, so the finish kernel's warp reads one
// contiguous row of 32 slots per run ordinal while each lane adds its ray's
// runs in path order. No atomics: the forward projection is bit-reproducible.
struct TileMatrixDev {
  int tiles_x, ntiles;
  int ts;                   // tile side (pixels); shared-memory row stride ts + 1
  int bw;                   // warps per tile block (8, 16 or 32)
  const int* group_first;   // [ntiles + 1] first group of each tile
  const int* gpart;         // [groups * 32] partial-sum slot of each lane's
                            // run, -1 if the lane is empty
  const int* rnrun;         // [P*C] runs of each ray
  const int* pbase;         // [ceil(P*C / 32)] first slot of each ray group
  const uint16_t* glp;      // [groups * 32] first pixel, tile-local (y*ts + x)
  const uint16_t* glen;     // [groups * 32] run length (segments)
  const int* gsteps;        // [groups] longest run of the group
  const int64_t* gseg_off;  // [groups] entry offset of the group's lengths
  const int64_t* gcode_off; // [groups] word offset of the step codes
  const void* tlen;         // lengths, entry (group, step/8, lane, step%8)
  const uint32_t* tcode;    // 8 x 4-bit step codes per word per lane
};

// Which per-ray value the forward kernel stores.
enum FwdOut { FWD_SIRT = 0, FWD_RATIO = 1, FWD_SIM = 2 };
// What the backward kernel does with its per-pixel sums.
enum BackEpi { EPI_UPDATE = 0, EPI_REPLICA = 1 };

struct IterArgs {
  DevGeom G;
  MatrixDev M;
  int K;              // slices per pass
  int S;              // sinogram slices
  int alg;            // 0..3
  int exact;          // TG_MODE_EXACT
  int delta_index;
  // reconstruction slots: slot(true slice t) = t + vshift; layout
  // [nslots/K][g*g][K]
  int vshift;
  int fshift;         // forward source slot of sinogram slice s = s + fshift
  int nslots;
  int slice_id, num_total_slices;  // APMLR top/bottom
  PenaltyWeights pw;
  // 16-bit gather operands (fast mode, set per launch sequence):
  // half_tile - the tile-staged forward keeps its shared-memory tile as
  //             halves; half_factors - storage of the per-ray ratio
  //             factors (FACT_*)
  int half_tile;
  int half_factors;
  // compensated (Kahan) summation of the ray and pixel sums (fast mode,
  // tile-staged forward, L1 backprojection)
  int comp;
};

// Work items of the launches that serve many plans at once (tg_batch): one
// item is one plan's slice batch, `first` its first block in the launch
// (items ascending by it).
struct FwdItem {
  TileMatrixDev T;
  const float* recon;   // the batch's reconstruction slots
  float* part;          // the plan's partial-sum slots
  int g;
  float inv_scale;
  int64_t first;
};
// Storage of the per-ray ratio factors between the forward finish and the
// backprojection. FACT_HALF_M1: halves of (factor - 1), exact to a half's
// precision relative to the factor's distance from 1, so the steady state
// (factors near 1) loses least; the backprojection adds the pixel's total
// length back. FACT_HALF: halves of the factor itself, a half's relative
// precision whatever the factor, for the first iteration after a reset,
// where factors lie anywhere between 0 and their largest value.
enum { FACT_F32 = 0, FACT_HALF_M1 = 1, FACT_HALF = 2 };

__host__ __device__ inline float factor_offset(int half_factors) {
  return half_factors == FACT_HALF_M1 ? 1.f : 0.f;
}

struct FinItem {
  const int* rnrun;
  const int* pbase;
  const float* ra2;
  const float* part;
  const float* sino;    // the batch's sinogram rows
  float* out;           // per-ray factors
  int64_t nrays;
  int64_t first;        // 256 rays a block
  int out_mode;
  int fh;               // factor storage (FACT_*)
};
struct BackItem {
  IterArgs A;
  int batch;
  const float* cur;
  float* next;
  const float* upd;
  int64_t first;
};

// The item a block belongs to.
template <class Item>
__device__ __forceinline__ int item_of(const Item* items, int n, int64_t block) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (items[mid].first <= block) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// Address of (slot, pixel) in the batched reconstruction layout.
__device__ __forceinline__ int64_t slot_addr(int slot, int64_t p, int64_t g2,
                                             int K) {
  return ((int64_t)(slot / K) * g2 + p) * K + (slot % K);
}

// APMLR's axial neighbours of slice s: the first slice of the dataset has
// none above, the last none below (apmlr.cc:937-967).
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

// tg_trace.cu
// ray_nruns (optional): runs per ray of the tile-ordered forward matrix
// (a new run at each tile change and non-unit step), counted in the same pass
void launch_trace_count(const DevGeom& G, int* nseg, int* rcap,
                        unsigned* maxlen_bits, int tiles_x, int ts, int* ray_nruns,
                        cudaStream_t st);
void launch_trace_fill(const DevGeom& G, const MatrixDev& M, int* ridx,
                       uint32_t* rcode, int* rstart, void* rlen, float* ra2,
                       double* ra2d, void* dlen, unsigned long long* overflow,
                       int4* exc, int* exc_tile, int exc_cap, cudaStream_t st);

// Adds the window exceptions of the calling lane's pixel: f(l, angle,
// column) for each, after the regular angle loop.
template <typename F>
__device__ __forceinline__ void for_each_exception(const MatrixDev& M, int tile,
                                                   int lane, F&& f) {
  if (M.exc_first == nullptr) return;
  const int e1 = M.exc_first[tile + 1];
  for (int e = M.exc_first[tile]; e < e1; ++e) {
    const int4 x = M.exc[e];
    if (x.x == lane) f(__int_as_float(x.w), x.y, x.z);
  }
}
// W (and, when Wh is given, the total of the half-rounded lengths) per pixel
void launch_weights(const DevGeom& G, const MatrixDev& M, int exact, float* W,
                    float* Wh, cudaStream_t st);
void launch_trace_export(const DevGeom& G, const int64_t* offsets, int* idx,
                         float* len, float* len2, cudaStream_t st);

// tg_forward.cu
void launch_forward(const IterArgs& A, const float* recon_batch,
                    const float* sino_batch, float* out, int out_mode,
                    cudaStream_t st);
// tg_backward.cu
// per-K instances of launch_backward (tg_backward*.cu)
#define TG_BACKWARD_DECL(KK)                                                      \
  void launch_backward_k##KK(const IterArgs& A, int batch, const float* recon_cur, \
                             float* recon_next, const float* upd, float* rep_num, \
                             int epi, cudaStream_t st);                            \
  void launch_backward_multi_k##KK(const BackItem* items, int n, int64_t blocks,   \
                                   int dlen_kind, int pen, int fh, int comp,        \
                                   cudaStream_t st);
TG_BACKWARD_DECL(1)
TG_BACKWARD_DECL(2)
TG_BACKWARD_DECL(4)
TG_BACKWARD_DECL(8)
TG_BACKWARD_DECL(16)
#undef TG_BACKWARD_DECL
void launch_backward(const IterArgs& A, int batch, const float* recon_cur,
                     float* recon_next, const float* upd, float* rep_num,
                     int epi, cudaStream_t st);
// tg_backward_staged.cu (fast mode)
void launch_backward_staged(const IterArgs& A, int batch, const float* recon_cur,
                            float* recon_next, const float* upd, float* rep_num,
                            int epi, cudaStream_t st);
// tg_fp64.cu
void launch_forward64(const IterArgs& A, const double* ra2d, const double* recon,
                      const float* sino, double* out, int out_mode,
                      cudaStream_t st);
void launch_backward64(const IterArgs& A, int s, const double* cur,
                       double* next, const double* upd, const double* W,
                       cudaStream_t st);
void launch_weights64(const DevGeom& G, const MatrixDev& M, double* W,
                      cudaStream_t st);
void launch_convert(const float* in, double* out, int64_t n, cudaStream_t st);
void launch_narrow(const double* in, float* out, int64_t n, cudaStream_t st);
void launch_fill64(double* p, int64_t n, double v, cudaStream_t st);
// tg_tiles.cu
// Run sort key: tile | chunk-count class | ray | ordinal (RunKey).
struct RunKey {
  int ray_bits;  // bits of the ray id field
  __host__ __device__ int class_shift() const { return 8 + ray_bits; }
  __host__ __device__ int tile_shift() const { return 13 + ray_bits; }
};
// Run emission and the tile-stream fill read each ray's segments back from
// the ray-ordered forward matrix M when it is stored (M.rlen), else trace them.
void launch_runs_emit(const DevGeom& G, const MatrixDev& M, int tiles_x, int ts, RunKey rk,
                      const int64_t* ray_run_off, unsigned long long* key, int* val,
                      uint16_t* run_lp, uint16_t* run_len, cudaStream_t st);
// Construction prefix sums (tg_tiles.cu): tmp == nullptr asks for the
// temporary bytes; counts (int) to int64 offsets, or int64 to int64.
cudaError_t scan_counts(void* tmp, size_t* tmp_bytes, const int* in, int64_t* out, int n,
                        cudaStream_t st);
cudaError_t scan_i64(void* tmp, size_t* tmp_bytes, const int64_t* in, int64_t* out, int n,
                     cudaStream_t st);
// gslots[g] = 32 x the longest run count of ray group g (32 rays)
void launch_group_slots(const int* nruns, int64_t R, int64_t* gslots, cudaStream_t st);
// out[g] = tile-stream entries of run group g (256 per 8-step chunk)
void launch_group_entries(const int* gsteps, int groups, int64_t* out, cudaStream_t st);
// out[i] = in[i] >> shift (as int, or int64)
void launch_shift_narrow_i32(const int64_t* in, int* out, int64_t n, int shift,
                             cudaStream_t st);
void launch_shift_i64(const int64_t* in, int64_t* out, int64_t n, int shift,
                      cudaStream_t st);
// tile_first[t] = first sorted run of tile t, tile_first[ntiles] = nruns
void launch_tile_bounds(RunKey rk, const unsigned long long* skey, int64_t nruns,
                        int ntiles, int* tile_first, cudaStream_t st);
int sort_runs(unsigned long long* key_in, unsigned long long* key_out,
              int* val_in, int* val_out, int64_t n, int end_bit,
              cudaStream_t st);
void launch_runs_group(RunKey rk, const unsigned long long* skey, const int* sval,
                       int64_t nruns, const int* tile_first_run,
                       const int* group_first, const uint16_t* run_lp,
                       const uint16_t* run_len, const int64_t* ray_run_off,
                       const int* pbase, int* gpart, uint16_t* glp,
                       uint16_t* glen, int* gsteps, int* run_slot, cudaStream_t st);
void launch_runs_fill(const DevGeom& G, const MatrixDev& M, int tiles_x, int ts,
                      const int64_t* ray_run_off, const int* run_slot,
                      const int64_t* gseg_off, const int64_t* gcode_off,
                      void* tlen, uint32_t* tcode, cudaStream_t st);
// part: [runs][K] partial sums, written (not accumulated) by each launch
void launch_forward_tiled(const IterArgs& A, const TileMatrixDev& T,
                          const float* recon_batch, float* part, cudaStream_t st);
// ray sums from the partial sums (fixed order) -> per-ray values `out`
void launch_fwd_finish(const IterArgs& A, const TileMatrixDev& T, const float* part,
                       const float* sino, float* out, int out_mode, cudaStream_t st);
// the same over many plans' slice batches in one launch each (device item
// arrays; blocks = the launch's total blocks; all items of one launch share
// K, the tile side and precision and the summation; 16-bit fixed-point
// lengths)
void launch_forward_tiled_multi(const FwdItem* items, int n, int64_t blocks, int K, int ts,
                                int bw, int half_tile, int comp, cudaStream_t st);
void launch_fwd_finish_multi(const FinItem* items, int n, int64_t blocks, int K, int comp,
                             cudaStream_t st);
// plans with 16-bit fixed-point lengths (backward matrix u16, or f16 with
// half gathers); pen: PML/APMLR; fh: half factors
void launch_backward_multi(const BackItem* items, int n, int64_t blocks, int K,
                           int dlen_kind, int pen, int fh, int comp, cudaStream_t st);
// blocks (of 256 threads) a plan's backprojection launch uses
int64_t backward_blocks(const IterArgs& A);
// tg_iter.cu
void launch_fg(const IterArgs& A, const float* recon, const float* W, float* F,
               float* Gv, cudaStream_t st);
void launch_update(const IterArgs& A, float* recon, const float* W,
                   const float* F, const float* Gv, const float* rep_num,
                   cudaStream_t st);
void launch_sino_pack(const float* in, float* out, int P, int S, int C, int K,
                      int apply_abs, int clip, float clip_min, cudaStream_t st);
void launch_sino_unpack(const float* in, float* out, int P, int S, int C,
                        int K, cudaStream_t st);
void launch_recon_pack(const float* in, float* out, int nuser, int g2, int K,
                       int slot0, int nslots, cudaStream_t st);
void launch_recon_unpack(const float* in, float* out, int nuser, int g2, int K,
                         int slot0, cudaStream_t st);
void launch_fill(float* p, size_t n, float v, cudaStream_t st);
void launch_replica_interleave(const float* rep_num, const float* W,
                               float* out, int S, int g2, cudaStream_t st);

}  // namespace tg
