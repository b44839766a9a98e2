// Host side of the C ABI declared in include/trace_gb300.h: plan creation
// (geometry tables, tracing, matrix construction), state upload/download,
// and the per-iteration launch sequence.
#include <cuda.h>

#include <algorithm>
#include <functional>
#include <map>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/trace_gb300.h"
#include "tg_kernels.cuh"

using namespace tg;

struct tg_plan {
  tg_plan_desc d{};
  int C = 0, P = 0, S = 0, K = 1;
  int fts = kTileSide;  // forward tile side (forward_tiles)
  int64_t g2 = 0, R = 0;
  float mov = 0.f;
  int len_kind = 0;
  DevGeom G{};
  MatrixDev M{};
  PenaltyWeights pw_base{};
  // device allocations
  float *d_yi = nullptr, *d_sin = nullptr, *d_cos = nullptr;
  float4* d_wcoef = nullptr;
  int* d_quad = nullptr;
  int64_t *d_roff = nullptr, *d_rcoff = nullptr;
  int *d_rcap = nullptr, *d_rnseg = nullptr, *d_ridx = nullptr, *d_rstart = nullptr;
  uint32_t* d_rcode = nullptr;
  void* d_rlen = nullptr;
  float* d_ra2 = nullptr;
  void* d_dlen = nullptr;
  float* d_W = nullptr;
  float* d_Wh = nullptr;  // half_gathers: total of the half-rounded lengths
  int* d_exc_first = nullptr;  // window exceptions (CSR over the pixel tiles)
  int4* d_exc = nullptr;
  // tile-staged forward (fast mode): the tile-ordered matrix + the runs'
  // partial sums ([runs][K], one slot per run)
  bool tiles = false;
  TileMatrixDev T{};
  float* d_part = nullptr;
  // two-stream iterations (batch_streams): odd slice batches run on st2
  // with their own partial sums and factors, so one batch's forward
  // projection overlaps the previous batch's finish and backprojection
  bool two = false;
  cudaStream_t st2 = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  // tg_iterate_get_recon: the stream that downloads finished slice batches
  // during the last iteration, one event per batch, and its join event
  cudaStream_t st_dl = nullptr;
  std::vector<cudaEvent_t> ev_batch;
  cudaEvent_t ev_dl = nullptr;
  float* d_part2 = nullptr;
  float* d_upd2 = nullptr;
  // FP64 mode: double state, factors, total lengths and SIRT's a2
  bool fp64 = false;
  double *d_ra2d = nullptr, *d_W64 = nullptr;
  unsigned* d_maxlen = nullptr;
  unsigned long long* d_overflow = nullptr;
  float* d_sino = nullptr;
  float* d_recon[2] = {nullptr, nullptr};
  int cur = 0;
  // fused iterations since the reconstruction was last reset or uploaded:
  // with half_gathers the first one stores halves of the factors, later ones
  // halves of factor - 1 (factor_storage)
  int64_t iters_done = 0;
  float* d_upd = nullptr;
  float* d_rep = nullptr;
  float *d_F = nullptr, *d_G = nullptr;
  float* d_stage = nullptr;
  size_t stage_n = 0;
  // state
  bool have_sino = false;
  int layout_alg = -1;  // algorithm whose layout the reconstruction uses
  int vshift = 0, fshift = 0, nslots = 0, halo = 0;
  int nb = 0;  // sinogram batches
  std::vector<int> h_nseg;
  cudaStream_t own = nullptr, st = nullptr;
  std::string err;
  tg_plan_info info{};
  int64_t dev_bytes = 0;
  std::vector<void*> allocs;
  // CUDA graphs of one iteration, one per buffer parity, keyed by the
  // algorithm and parameters they were captured with
  bool use_graphs = false;
  struct Graph {
    bool valid = false;
    int alg = -1;
    int half_factors = -1;
    tg_params prm{};
    cudaGraphExec_t exec = nullptr;
  } graphs[2];
  // device address of the allocation-free entry point's factor array in the
  // context this plan was created in (looked up at creation), or nullptr
  float* noalloc_factors = nullptr;
  std::string noalloc_err;
  // per-kernel timers: event pairs recorded around launches while enabled
  bool timing = false;
  std::vector<cudaEvent_t> ev_pool;
  std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> ev_used;
};

namespace {

thread_local std::string g_create_error;

int fail(tg_plan* p, int code, const std::string& msg) {
  if (p)
    p->err = msg;
  else
    g_create_error = msg;
  return code;
}

#define TG_CUDA(plan, call)                                                  \
  do {                                                                       \
    cudaError_t e_ = (call);                                                 \
    if (e_ != cudaSuccess)                                                   \
      return fail(plan, TG_E_CUDA,                                           \
                  std::string(#call) + ": " + cudaGetErrorString(e_));       \
  } while (0)

#define TG_TRY(x)          \
  do {                     \
    int rc_ = (x);         \
    if (rc_ != TG_OK) return rc_; \
  } while (0)

template <class T>
int dalloc(tg_plan* p, T** out, size_t count, bool zero = false) {
  void* ptr = nullptr;
  const size_t bytes = count * sizeof(T);
  if (bytes == 0) {
    *out = nullptr;
    return TG_OK;
  }
  cudaError_t e = cudaMalloc(&ptr, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(p, TG_E_NOMEM,
                "cudaMalloc of " + std::to_string(bytes) + " bytes failed: " +
                    cudaGetErrorString(e));
  }
  p->allocs.push_back(ptr);
  p->dev_bytes += (int64_t)bytes;
  if (zero) {
    e = cudaMemsetAsync(ptr, 0, bytes, p->st);
    if (e != cudaSuccess) return fail(p, TG_E_CUDA, cudaGetErrorString(e));
  }
  *out = static_cast<T*>(ptr);
  return TG_OK;
}

void dfree(tg_plan* p, void* ptr, size_t bytes) {
  if (!ptr) return;
  for (auto& a : p->allocs)
    if (a == ptr) a = nullptr;
  cudaFree(ptr);
  p->dev_bytes -= (int64_t)bytes;
}

constexpr float kPI = 3.14159265358979f;  // trace_utils.h:8

int quadrant_of(float t) {
  return ((t >= 0 && t < kPI / 2) || (t >= kPI && t < 3 * kPI / 2)) ? 1 : 0;
}

int halo_of(int alg) { return alg == TG_APMLR ? 1 : 0; }

bool valid_alg(int alg) { return alg >= TG_SIRT && alg <= TG_APMLR; }

// Device address through which kernels read or write the `n` floats of
// caller host memory at `ptr` in place, or nullptr. Page-locked host memory
// (cudaHostAlloc / cudaMallocHost, or registered as mapped) is addressable
// by kernels across GB300's CPU-GPU link, so the layout kernels pack from
// and unpack into it directly: no device staging buffer to allocate and no
// separate copy. Both ends of the range must be page-locked and map to one
// linear device range; anything else (pageable memory) is staged.
float* mapped_host(const void* ptr, size_t n) {
  if (n == 0) return nullptr;
  const char* first = static_cast<const char*>(ptr);
  const char* last = first + (n - 1) * sizeof(float);
  cudaPointerAttributes a{}, b{};
  if (cudaPointerGetAttributes(&a, first) != cudaSuccess ||
      cudaPointerGetAttributes(&b, last) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  if (a.type != cudaMemoryTypeHost || b.type != cudaMemoryTypeHost ||
      !a.devicePointer || !b.devicePointer)
    return nullptr;
  if (static_cast<char*>(b.devicePointer) - static_cast<char*>(a.devicePointer) !=
      last - first)
    return nullptr;
  return static_cast<float*>(a.devicePointer);
}

// Whether kernels may write the host memory at `ptr` (for downloads into a
// mapped buffer): memory registered read-only (cudaHostRegisterReadOnly) is
// mapped for device reads only, and writing it from a kernel would be an
// invalid access, so such a buffer takes the staged copy instead. The
// driver's pointer attribute is reached through the runtime's entry-point
// query (no link against the driver library); if it cannot be asked, the
// answer is no.
bool device_writable(const void* ptr) {
  using GetAttr = CUresult (*)(void*, CUpointer_attribute, CUdeviceptr);
  static const GetAttr get = []() -> GetAttr {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuPointerGetAttribute", &fn, 12000,
                                         cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess) {
      cudaGetLastError();
      return nullptr;
    }
    return reinterpret_cast<GetAttr>(fn);
  }();
  if (!get) return false;
  unsigned int flags = 0;
  if (get(&flags, CU_POINTER_ATTRIBUTE_ACCESS_FLAGS, (CUdeviceptr)(uintptr_t)ptr) !=
      CUDA_SUCCESS)
    return false;
  return flags == CU_POINTER_ATTRIBUTE_ACCESS_FLAG_READWRITE;
}

// mapped_host for a buffer the kernels will write: both ends writable too.
float* mapped_host_out(void* ptr, size_t n) {
  float* m = mapped_host(ptr, n);
  if (!m) return nullptr;
  const char* last = static_cast<const char*>(ptr) + (n - 1) * sizeof(float);
  return device_writable(ptr) && device_writable(last) ? m : nullptr;
}

// Stage host data through one reusable device buffer.
int stage(tg_plan* p, size_t n) {
  if (p->stage_n >= n) return TG_OK;
  dfree(p, p->d_stage, p->stage_n * sizeof(float));
  p->d_stage = nullptr;
  p->stage_n = 0;
  TG_TRY(dalloc(p, &p->d_stage, n));
  p->stage_n = n;
  return TG_OK;
}

void fill_weights(tg_plan* p, const tg_params* prm, PenaltyWeights& w) {
  w = p->pw_base;
  if (!prm) return;
  w.beta = prm->beta;
  w.beta1 = prm->beta1;
  w.delta = prm->delta;
  w.delta1 = prm->delta1;
  // APMLR weights (apmlr.cc:40-51, 90-97, 228-233; top/bottom variants with
  // one axial neighbour, apmlr.cc:361-370): totals evaluated in double
  // and stored as float, exactly as the reference's initialisers do.
  const double base[3] = {4 + 4 / std::sqrt(2.0), 3 + 2 / std::sqrt(2.0),
                          2 + 1 / std::sqrt(2.0)};
  const float regw = prm->regw;
  for (int r = 0; r < 3; ++r)
    for (int ax = 0; ax < 2; ++ax) {
      const float total = ax == 0 ? (float)(base[r] + 2 * regw)
                                  : (float)(base[r] + regw);
      w.apmlr[r][ax][0] = 1 / total;
      w.apmlr[r][ax][1] = (float)(1 / std::sqrt(2.0) / total);
      w.apmlr[r][ax][2] = regw / total;
    }
}

IterArgs make_args(tg_plan* p, int alg, const tg_params* prm) {
  IterArgs A{};
  A.G = p->G;
  A.M = p->M;
  A.K = p->K;
  A.S = p->S;
  A.alg = alg;
  A.exact = p->d.mode == TG_MODE_EXACT;
  A.delta_index = p->d.delta_index;
  A.vshift = p->vshift;
  A.fshift = p->fshift;
  A.nslots = p->nslots;
  A.slice_id = p->d.slice_id;
  A.num_total_slices = p->d.num_total_slices;
  A.comp = p->d.compensated;
  fill_weights(p, prm, A.pw);
  return A;
}

int check_layout(tg_plan* p, int alg) {
  if (!valid_alg(alg)) return fail(p, TG_E_ARG, "unknown algorithm");
  if (p->layout_alg < 0)
    return fail(p, TG_E_STATE,
                "no reconstruction: call tg_reset_recon or tg_set_recon first");
  if (halo_of(alg) != p->halo)
    return fail(p, TG_E_STATE,
                "reconstruction layout was set up for a different algorithm "
                "family (APMLR keeps one halo slice on each side)");
  return TG_OK;
}

void drop_graphs(tg_plan* p) {
  for (auto& g : p->graphs) {
    if (g.exec) cudaGraphExecDestroy(g.exec);
    g = tg_plan::Graph();
  }
}

int establish_layout(tg_plan* p, int alg) {
  if (!valid_alg(alg)) return fail(p, TG_E_ARG, "unknown algorithm");
  drop_graphs(p);
  const int halo = halo_of(alg);
  int vshift = 0, fshift = 0;
  if (alg == TG_APMLR) {
    if (p->d.apmlr_fixed_offset) {
      vshift = p->K;  // top halo at slot K-1, forward source aligned at s + K
      fshift = p->K;
    } else {
      vshift = 1;     // top halo at slot 0 = forward source of slice 0
      fshift = 0;
    }
  }
  const int need = p->S + vshift + halo;
  const int nslots = (need + p->K - 1) / p->K * p->K;
  if (p->layout_alg < 0 || p->nslots != nslots || p->halo != halo ||
      p->vshift != vshift) {
    const size_t esz = p->fp64 ? 2 : 1;  // floats per element
    const size_t old_n = (size_t)p->nslots * p->g2 * esz;
    for (int b = 0; b < 2; ++b) {
      dfree(p, p->d_recon[b], old_n * sizeof(float));
      p->d_recon[b] = nullptr;
    }
    for (int b = 0; b < 2; ++b)
      TG_TRY(dalloc(p, &p->d_recon[b], (size_t)nslots * p->g2 * esz));
  }
  p->halo = halo;
  p->vshift = vshift;
  p->fshift = fshift;
  p->nslots = nslots;
  p->layout_alg = alg;
  p->cur = 0;
  p->iters_done = 0;
  return TG_OK;
}

// Timer bracket around one launch; kind 0 forward, 1 backward, 2 other.
struct Timed {
  tg_plan* p;
  int kind;
  cudaEvent_t b = nullptr, e = nullptr;
  cudaEvent_t take() {
    if (!p->ev_pool.empty()) {
      cudaEvent_t ev = p->ev_pool.back();
      p->ev_pool.pop_back();
      return ev;
    }
    cudaEvent_t ev;
    cudaEventCreate(&ev);
    return ev;
  }
  Timed(tg_plan* pl, int k) : p(pl), kind(k) {
    if (!p->timing) return;
    b = take();
    e = take();
    cudaEventRecord(b, p->st);
  }
  ~Timed() {
    if (!p->timing) return;
    cudaEventRecord(e, p->st);
    p->ev_used.push_back({kind, {b, e}});
  }
};

float* batch_ptr(tg_plan* p, float* base, int batch_slot) {
  return base + (int64_t)(batch_slot / p->K) * p->g2 * p->K;
}

// Tile-ordered forward matrix (tg_tiles.cu): runs of each ray inside ts x ts
// tiles, sorted by (tile, chunk-count class, ray) and packed 32 per warp group.
int build_tiles(tg_plan* p, int* d_nruns) {
  const DevGeom& G = p->G;
  const int C = p->C;
  const int tiles_x = (C + p->fts - 1) / p->fts;
  const int ntiles = tiles_x * tiles_x;
  int tile_bits = 1;
  while ((1 << tile_bits) < ntiles) ++tile_bits;
  RunKey rk{1};
  while ((int64_t(1) << rk.ray_bits) < p->R) ++rk.ray_bits;
  const int end_bit = rk.tile_shift() + tile_bits;
  if (end_bit > 64) return fail(p, TG_E_GEOMETRY, "tile run keys exceed 64 bits");
  // temporaries of the construction, freed at the end
  std::vector<std::pair<void*, size_t>> tmp;
  auto talloc = [&](auto** ptr, size_t n, bool zero) -> int {
    int rc = dalloc(p, ptr, n, zero);
    if (rc == TG_OK) tmp.push_back({(void*)*ptr, n * sizeof(**ptr)});
    return rc;
  };
  auto release = [&]() {
    for (auto& t : tmp) dfree(p, t.first, t.second);
    tmp.clear();
  };
  int rc = TG_OK;
  // Offsets on the device (prefix sums, no round trip through the host):
  // each ray's first run, each 32-ray group's first partial-sum slot (32
  // per run ordinal up to the group's longest run count); only the totals
  // come back, to size the buffers.
  const int64_t rgroups = (p->R + 31) / 32;
  int64_t *d_run_off, *d_gslots, *d_pbase64;
  if ((rc = talloc(&d_run_off, (size_t)p->R, false)) ||
      (rc = talloc(&d_gslots, (size_t)rgroups, false)) ||
      (rc = talloc(&d_pbase64, (size_t)rgroups, false)))
    return release(), rc;
  char* scan_tmp = nullptr;
  size_t scan_bytes = 0;
  // temporary storage for one prefix sum (CUB), grown as needed
  auto scan_space = [&](size_t need) -> int {
    if (need <= scan_bytes) return TG_OK;
    int r2 = talloc(&scan_tmp, need, false);
    if (r2 == TG_OK) scan_bytes = need;
    return r2;
  };
  {
    size_t b1 = 0, b2 = 0;
    if (scan_counts(nullptr, &b1, d_nruns, d_run_off, (int)p->R, p->st) != cudaSuccess ||
        scan_i64(nullptr, &b2, d_gslots, d_pbase64, (int)rgroups, p->st) != cudaSuccess)
      return release(), fail(p, TG_E_CUDA, "prefix-sum setup failed");
    if ((rc = scan_space(std::max(b1, b2)))) return release(), rc;
    b1 = b2 = scan_bytes;
    launch_group_slots(d_nruns, p->R, d_gslots, p->st);
    if (scan_counts(scan_tmp, &b1, d_nruns, d_run_off, (int)p->R, p->st) != cudaSuccess ||
        scan_i64(scan_tmp, &b2, d_gslots, d_pbase64, (int)rgroups, p->st) != cudaSuccess)
      return release(), fail(p, TG_E_CUDA, "prefix sums failed");
  }
  int64_t last_off = 0, last_base = 0, last_slots = 0;
  int last_runs = 0;
  cudaMemcpyAsync(&last_off, d_run_off + p->R - 1, 8, cudaMemcpyDeviceToHost, p->st);
  cudaMemcpyAsync(&last_runs, d_nruns + p->R - 1, 4, cudaMemcpyDeviceToHost, p->st);
  cudaMemcpyAsync(&last_base, d_pbase64 + rgroups - 1, 8, cudaMemcpyDeviceToHost, p->st);
  cudaMemcpyAsync(&last_slots, d_gslots + rgroups - 1, 8, cudaMemcpyDeviceToHost, p->st);
  if (cudaStreamSynchronize(p->st) != cudaSuccess)
    return release(), fail(p, TG_E_CUDA, "run counting failed");
  const int64_t NR = last_off + last_runs;
  const int64_t nslots = last_base + last_slots;
  if (NR > 0x7fffffff) return release(), fail(p, TG_E_GEOMETRY, "too many tile runs");
  if (nslots > 0x7fffffff)
    return release(), fail(p, TG_E_GEOMETRY, "too many partial-sum slots");
  unsigned long long *key, *key2;
  int *val, *val2, *run_slot, *d_tile_first;
  uint16_t *run_lp, *run_len;
  if ((rc = talloc(&key, (size_t)NR, false)) ||
      (rc = talloc(&key2, (size_t)NR, false)) || (rc = talloc(&val, (size_t)NR, false)) ||
      (rc = talloc(&val2, (size_t)NR, false)) || (rc = talloc(&run_lp, (size_t)NR, false)) ||
      (rc = talloc(&run_len, (size_t)NR, false)) || (rc = talloc(&run_slot, (size_t)NR, false)) ||
      (rc = talloc(&d_tile_first, (size_t)ntiles + 1, false)))
    return release(), rc;
  launch_runs_emit(G, p->M, tiles_x, p->fts, rk, d_run_off, key, val, run_lp, run_len, p->st);
  if (sort_runs(key, key2, val, val2, NR, end_bit, p->st))
    return release(), fail(p, TG_E_CUDA, "sorting the tile runs failed");
  // each tile's first run in the sorted order, from the sorted keys
  launch_tile_bounds(rk, key2, NR, ntiles, d_tile_first, p->st);
  std::vector<int> tile_first(ntiles + 1), group_first(ntiles + 1);
  cudaMemcpyAsync(tile_first.data(), d_tile_first, (ntiles + 1) * 4, cudaMemcpyDeviceToHost,
                  p->st);
  if (cudaStreamSynchronize(p->st) != cudaSuccess) return release(), fail(p, TG_E_CUDA, "run emit failed");
  int groups = 0;
  for (int t = 0; t < ntiles; ++t) {
    group_first[t] = groups;
    groups += (tile_first[t + 1] - tile_first[t] + 31) / 32;
  }
  group_first[ntiles] = groups;
  int *d_group_first, *gpart, *gsteps, *pbase;
  uint16_t *glp, *glen;
  if ((rc = dalloc(p, &d_group_first, (size_t)ntiles + 1)) ||
      (rc = dalloc(p, &gpart, (size_t)groups * 32)) ||
      (rc = dalloc(p, &pbase, (size_t)rgroups)) ||
      (rc = dalloc(p, &glp, (size_t)groups * 32, true)) ||
      (rc = dalloc(p, &glen, (size_t)groups * 32, true)) ||
      (rc = dalloc(p, &gsteps, (size_t)groups, true)))
    return release(), rc;
  cudaMemsetAsync(gpart, 0xff, (size_t)groups * 32 * 4, p->st);  // empty lanes: -1
  cudaMemcpyAsync(d_group_first, group_first.data(), (ntiles + 1) * 4, cudaMemcpyHostToDevice, p->st);
  launch_shift_narrow_i32(d_pbase64, pbase, rgroups, 0, p->st);  // checked above
  launch_runs_group(rk, key2, val2, NR, d_tile_first, d_group_first, run_lp, run_len,
                    d_run_off, pbase, gpart, glp, glen, gsteps, run_slot, p->st);
  // the groups' tile-stream offsets: 256 entries (and 64 step words) per
  // chunk of 8 steps of the group's longest run
  int64_t *d_seg_off, *d_code_off, *d_gentries;
  if ((rc = dalloc(p, &d_seg_off, (size_t)groups)) ||
      (rc = dalloc(p, &d_code_off, (size_t)groups)) ||
      (rc = talloc(&d_gentries, (size_t)groups, false)))
    return release(), rc;
  int64_t entries = 0;
  if (groups > 0) {
    size_t b3 = 0;
    if (scan_i64(nullptr, &b3, d_gentries, d_seg_off, groups, p->st) != cudaSuccess)
      return release(), fail(p, TG_E_CUDA, "prefix-sum setup failed");
    if ((rc = scan_space(b3))) return release(), rc;
    b3 = scan_bytes;
    launch_group_entries(gsteps, groups, d_gentries, p->st);
    if (scan_i64(scan_tmp, &b3, d_gentries, d_seg_off, groups, p->st) != cudaSuccess)
      return release(), fail(p, TG_E_CUDA, "prefix sums failed");
    launch_shift_i64(d_seg_off, d_code_off, groups, 2, p->st);  // 64 words per 256 entries
    int64_t last_seg = 0, last_entries = 0;
    cudaMemcpyAsync(&last_seg, d_seg_off + groups - 1, 8, cudaMemcpyDeviceToHost, p->st);
    cudaMemcpyAsync(&last_entries, d_gentries + groups - 1, 8, cudaMemcpyDeviceToHost, p->st);
    if (cudaStreamSynchronize(p->st) != cudaSuccess)
      return release(), fail(p, TG_E_CUDA, "run grouping failed");
    entries = last_seg + last_entries;
  }
  const int64_t words = entries / 4;
  const bool l16 = p->len_kind != TG_LEN_F32;
  uint32_t* tcode;
  void* tlen = nullptr;
  // unused steps keep the "stay" step 0 (tg_tiles.cu)
  if ((rc = dalloc(p, &tcode, (size_t)words, true))) return release(), rc;
  if (l16) {
    uint16_t* t;
    if ((rc = dalloc(p, &t, (size_t)entries, true))) return release(), rc;
    tlen = t;
  } else {
    float* t;
    if ((rc = dalloc(p, &t, (size_t)entries, true))) return release(), rc;
    tlen = t;
  }
  launch_runs_fill(G, p->M, tiles_x, p->fts, d_run_off, run_slot, d_seg_off, d_code_off, tlen,
                   tcode, p->st);
  if (cudaStreamSynchronize(p->st) != cudaSuccess) return release(), fail(p, TG_E_CUDA, "run fill failed");
  release();
  if ((rc = dalloc(p, &p->d_part, (size_t)nslots * p->K))) return rc;
  TileMatrixDev& T = p->T;
  T.tiles_x = tiles_x;
  T.ntiles = ntiles;
  T.ts = p->fts;
  T.bw = p->d.forward_block_warps ? p->d.forward_block_warps : 32;
  T.group_first = d_group_first;
  T.gpart = gpart;
  T.rnrun = d_nruns;
  T.pbase = pbase;
  T.glp = glp;
  T.glen = glen;
  T.gsteps = gsteps;
  T.gseg_off = d_seg_off;
  T.gcode_off = d_code_off;
  T.tlen = tlen;
  T.tcode = tcode;
  p->tiles = true;
  p->info.tile_runs = NR;
  p->info.partial_slots = nslots;
  p->info.tile_bytes = entries * (l16 ? 2 : 4) + words * 4 + (int64_t)groups * (32 * 8 + 20);
  return TG_OK;
}

int ensure_upd(tg_plan* p) {
  if (!p->d_upd) TG_TRY(dalloc(p, &p->d_upd, (size_t)p->R * p->K * (p->fp64 ? 2 : 1)));
  if (p->two && !p->d_upd2) TG_TRY(dalloc(p, &p->d_upd2, (size_t)p->R * p->K));
  return TG_OK;
}

int fp32_only(tg_plan* p) {
  if (p->fp64)
    return fail(p, TG_E_STATE,
                "FP64 plans support tg_iterate and reconstruction upload/"
                "download only");
  return TG_OK;
}

double* as_f64(float* p) { return reinterpret_cast<double*>(p); }

}  // namespace

// tg_reduce_slice_noalloc's factor array, looked up for each new plan
static void resolve_noalloc_factors(tg_plan* p);

extern "C" {

int tg_abi_version(void) { return TG_ABI_VERSION; }

const char* tg_last_error(const tg_plan* plan) {
  return plan ? plan->err.c_str() : g_create_error.c_str();
}

int tg_degree_to_radian(float* theta, int n) {
  if (!theta || n < 0) return TG_E_ARG;
  for (int i = 0; i < n; ++i) theta[i] = theta[i] * kPI / 180.0;  // trace_utils.cc:20
  return TG_OK;
}

int tg_host_alloc(size_t bytes, void** out) {
  if (!out) return fail(nullptr, TG_E_ARG, "null output");
  *out = nullptr;
  if (bytes == 0) return TG_OK;
  // portable: page-locked for every device's context, as plans on several
  // devices in one process may share the buffer
  const cudaError_t e = cudaHostAlloc(out, bytes, cudaHostAllocPortable);
  if (e != cudaSuccess) {
    cudaGetLastError();
    *out = nullptr;
    return fail(nullptr, TG_E_NOMEM, "cudaHostAlloc of " + std::to_string(bytes) +
                                         " bytes failed: " + cudaGetErrorString(e));
  }
  return TG_OK;
}

int tg_host_free(void* ptr) {
  if (!ptr) return TG_OK;
  const cudaError_t e = cudaFreeHost(ptr);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(nullptr, TG_E_CUDA, std::string("cudaFreeHost failed: ") +
                                        cudaGetErrorString(e));
  }
  return TG_OK;
}

int tg_plan_create(const tg_plan_desc* desc, const float* theta,
                   const float* sin_tab, const float* cos_tab, tg_plan** out) {
  if (!desc || !theta || !out) return fail(nullptr, TG_E_ARG, "null argument");
  *out = nullptr;
  const tg_plan_desc& d = *desc;
  if (d.num_projs < 1 || d.num_slices < 1 || d.num_cols < 2)
    return fail(nullptr, TG_E_ARG, "need num_projs >= 1, num_slices >= 1, num_cols >= 2");
  if (d.num_cols > 32768)
    return fail(nullptr, TG_E_ARG, "num_cols above 32768 is not supported");
  if (!(d.slices_per_pass == 1 || d.slices_per_pass == 2 ||
        d.slices_per_pass == 4 || d.slices_per_pass == 8 || d.slices_per_pass == 16))
    return fail(nullptr, TG_E_ARG, "slices_per_pass must be 1, 2, 4, 8 or 16");
  if (d.slices_per_pass == 16 && d.forward_tiles && !d.half_gathers)
    return fail(nullptr, TG_E_ARG,
                "16 slices per pass with forward_tiles needs half_gathers (shared-memory tile)");
  if (d.len_storage < TG_LEN_F32 || d.len_storage > TG_LEN_U16)
    return fail(nullptr, TG_E_ARG, "unknown len_storage");
  if (d.mode != TG_MODE_EXACT && d.mode != TG_MODE_FAST && d.mode != TG_MODE_FP64)
    return fail(nullptr, TG_E_ARG, "unknown mode");
  if ((d.forward_tiles || d.backward_staged) && d.mode != TG_MODE_FAST)
    return fail(nullptr, TG_E_ARG, "forward_tiles and backward_staged need fast mode");
  if (d.forward_on_the_fly && d.mode == TG_MODE_FP64)
    return fail(nullptr, TG_E_ARG, "forward_on_the_fly is not available in FP64 mode");
  if (d.half_gathers && (d.mode != TG_MODE_FAST || !d.forward_tiles || d.backward_staged))
    return fail(nullptr, TG_E_ARG,
                "half_gathers needs fast mode, forward_tiles and the L1 backprojection");
  if (d.mode == TG_MODE_FP64 &&
      (d.len_storage != TG_LEN_F32 || d.slices_per_pass != 1 || d.delta_index))
    return fail(nullptr, TG_E_ARG,
                "FP64 mode needs f32 lengths, explicit indices and one slice per pass");
  if (d.compensated && (d.mode != TG_MODE_FAST || !d.forward_tiles || d.backward_staged ||
                        d.slices_per_pass > 8))
    return fail(nullptr, TG_E_ARG,
                "compensated needs fast mode, forward_tiles, the L1 backprojection and "
                "at most 8 slices per pass");
  // tile sides: multiples of 16 up to 96 (a step's shared-memory index
  // change dx + dy * (side + 1) must fit a signed byte)
  if (d.forward_tile_side != 0 &&
      (d.forward_tile_side < 32 || d.forward_tile_side > 96 || d.forward_tile_side % 16))
    return fail(nullptr, TG_E_ARG, "forward_tile_side must be 0, 32, 48, 64, 80 or 96");
  if (d.forward_tiles) {
    // the shared-memory tile: side x (side + 1) pixels of slices_per_pass
    // values, halves with half_gathers (and always at 16 slices per pass)
    const int64_t ts = d.forward_tile_side ? d.forward_tile_side : kTileSide;
    const int64_t bytes = ts * (ts + 1) * d.slices_per_pass *
                          ((d.half_gathers || d.slices_per_pass == 16) ? 2 : 4);
    if (bytes > 232448)
      return fail(nullptr, TG_E_ARG,
                  "the forward tile (" + std::to_string(bytes) +
                      " bytes) does not fit shared memory; use a smaller "
                      "forward_tile_side, fewer slices per pass or half_gathers");
  }
  if (d.forward_block_warps != 0 && d.forward_block_warps != 8 &&
      d.forward_block_warps != 16 && d.forward_block_warps != 32)
    return fail(nullptr, TG_E_ARG, "forward_block_warps must be 0, 8, 16 or 32");
  if (d.batch_streams < 0 || d.batch_streams > 2)
    return fail(nullptr, TG_E_ARG, "batch_streams must be 0, 1 or 2");
  if (d.backward_tile_width != 0 && d.backward_tile_width != 4 &&
      d.backward_tile_width != 8 && d.backward_tile_width != 16)
    return fail(nullptr, TG_E_ARG, "backward_tile_width must be 0, 4, 8 or 16");
  if (d.backward_staged && d.backward_tile_width != 0 && d.backward_tile_width != 8)
    return fail(nullptr, TG_E_ARG, "backward_staged uses 8x4 pixel tiles");
  if ((sin_tab == nullptr) != (cos_tab == nullptr))
    return fail(nullptr, TG_E_ARG, "give both sin_tab and cos_tab or neither");

  tg_plan* p = new (std::nothrow) tg_plan();
  if (!p) return fail(nullptr, TG_E_NOMEM, "host allocation failed");
  p->d = d;
  if (p->d.num_total_slices <= 0) p->d.num_total_slices = d.num_slices;
  p->C = d.num_cols;
  p->P = d.num_projs;
  p->S = d.num_slices;
  p->K = d.slices_per_pass;
  p->g2 = (int64_t)p->C * p->C;
  p->R = (int64_t)p->P * p->C;
  p->len_kind = d.len_storage;
  p->nb = (p->S + p->K - 1) / p->K;
  p->fp64 = d.mode == TG_MODE_FP64;
  if (d.forward_tile_side) p->fts = d.forward_tile_side;

  auto bail = [&](int rc) {
    g_create_error = p->err;
    tg_plan_destroy(p);
    return rc;
  };
  if (cudaStreamCreateWithFlags(&p->own, cudaStreamNonBlocking) != cudaSuccess) {
    cudaGetLastError();
    p->err = "cudaStreamCreate failed (no CUDA device?)";
    return bail(TG_E_CUDA);
  }
  p->st = p->own;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0, p->st);

  // geometry tables (trace_data.h:96-108, sirt.cc:117-129)
  const int C = p->C, P = p->P;
  const float center = (d.center <= 0.) ? static_cast<float>(C) / 2. + 1. : d.center;
  float mov = static_cast<float>(C) / 2. - center;
  if (mov - std::ceil(mov) < 1e-6) mov += 1e-6;
  p->mov = mov;
  std::vector<float> yi(C), sn(P), cs(P);
  std::vector<int> qd(P);
  for (int c = 0; c < C; ++c) yi[c] = (1 - C) / 2. + c + mov;
  for (int a = 0; a < P; ++a) {
    sn[a] = sin_tab ? sin_tab[a] : sinf(theta[a]);
    cs[a] = cos_tab ? cos_tab[a] : cosf(theta[a]);
    qd[a] = quadrant_of(theta[a]);
  }
  int rc;
  if ((rc = dalloc(p, &p->d_yi, C)) || (rc = dalloc(p, &p->d_sin, P)) ||
      (rc = dalloc(p, &p->d_cos, P)) || (rc = dalloc(p, &p->d_quad, P)))
    return bail(rc);
  cudaMemcpyAsync(p->d_yi, yi.data(), C * 4, cudaMemcpyHostToDevice, p->st);
  cudaMemcpyAsync(p->d_sin, sn.data(), P * 4, cudaMemcpyHostToDevice, p->st);
  cudaMemcpyAsync(p->d_cos, cs.data(), P * 4, cudaMemcpyHostToDevice, p->st);
  cudaMemcpyAsync(p->d_quad, qd.data(), P * 4, cudaMemcpyHostToDevice, p->st);

  DevGeom& G = p->G;
  G.C = C;
  G.P = P;
  G.gpa = (C + 31) / 32;
  G.gpr = (C + 31) / 32;
  G.halfg = 0.5f * (float)C;
  G.mgrids = C / 2.;
  G.off = (float)((1.0 - C) / 2.0 + (double)mov);
  G.yi = p->d_yi;
  G.sinq = p->d_sin;
  G.cosq = p->d_cos;
  G.quad = p->d_quad;

  // window coefficients of the backward matrix: c0 = round(-s*x + c*y + D)
  // (tg::window_c0), D from the pixel-centre offset, half the footprint, a
  // quarter-column margin and the +1/2 of the rounding
  const int P4 = (P + 3) / 4 * 4;  // backward matrix: angles in fours
  std::vector<float4> wc(P4, make_float4(0.f, 0.f, 0.f, 0.f));
  const double off = (1.0 - C) / 2.0 + (double)mov;
  for (int a = 0; a < P; ++a) {
    const double sd = sn[a], cd = cs[a];
    const double D = (C / 2.0 - 0.5) * (sd - cd) -
                     0.5 * (std::fabs(sd) + std::fabs(cd)) - 0.25 - off + 0.5;
    wc[a] = make_float4(-sn[a], cs[a], (float)D, 0.f);
  }
  if ((rc = dalloc(p, &p->d_wcoef, P4))) return bail(rc);
  cudaMemcpyAsync(p->d_wcoef, wc.data(), P4 * sizeof(float4),
                  cudaMemcpyHostToDevice, p->st);
  // backward pixel tiles: 2^tw_shift x 2^(5 - tw_shift)
  const int tw = d.backward_tile_width ? d.backward_tile_width : 8;
  const int tw_shift = tw == 16 ? 4 : tw == 4 ? 2 : 3;
  const int tiles_x = (C + tw - 1) / tw, tiles_y = (C + (32 / tw) - 1) / (32 / tw);

  // pass 1: segment counts, per-group capacity, longest segment
  const int ngroups = P * G.gpa;
  if ((rc = dalloc(p, &p->d_rnseg, (size_t)p->R)) ||
      (rc = dalloc(p, &p->d_rcap, (size_t)ngroups)) ||
      (rc = dalloc(p, &p->d_maxlen, 1, true)) ||
      (rc = dalloc(p, &p->d_overflow, 3, true)))
    return bail(rc);
  // runs per ray of the tile-ordered forward matrix, counted in the same pass
  // (kept on the device: the tile build's offsets and the finish kernel's
  // per-ray run counts)
  int* d_nruns = nullptr;
  if (d.forward_tiles) {
    if ((rc = dalloc(p, &d_nruns, (size_t)p->R))) return bail(rc);
  }
  launch_trace_count(G, p->d_rnseg, p->d_rcap, p->d_maxlen, (C + p->fts - 1) / p->fts,
                     p->fts, d_nruns, p->st);
  std::vector<int> rcap(ngroups);
  unsigned maxbits = 0;
  p->h_nseg.resize(p->R);
  cudaMemcpyAsync(rcap.data(), p->d_rcap, ngroups * 4, cudaMemcpyDeviceToHost, p->st);
  cudaMemcpyAsync(&maxbits, p->d_maxlen, 4, cudaMemcpyDeviceToHost, p->st);
  cudaMemcpyAsync(p->h_nseg.data(), p->d_rnseg, p->R * 4, cudaMemcpyDeviceToHost, p->st);
  const cudaError_t traced = cudaStreamSynchronize(p->st);
  if (traced != cudaSuccess) {
    p->err = std::string("tracing failed: ") + cudaGetErrorString(cudaGetLastError());
    return bail(TG_E_CUDA);
  }
  float maxlen;
  std::memcpy(&maxlen, &maxbits, 4);
  int64_t nseg_total = 0;
  for (int v : p->h_nseg) nseg_total += v;

  // layout of the forward matrix: exclusive scans of the group capacities
  std::vector<int64_t> roff(ngroups), rcoff(ngroups);
  int64_t entries = 0, words = 0;
  for (int i = 0; i < ngroups; ++i) {
    roff[i] = entries;
    rcoff[i] = words;
    entries += (int64_t)rcap[i] * 32;
    words += (int64_t)((rcap[i] + 7) / 8) * 32;
  }
  const bool l16 = p->len_kind != TG_LEN_F32;
  const size_t lbytes = l16 ? 2 : 4;
  if ((rc = dalloc(p, &p->d_roff, (size_t)ngroups)) ||
      (rc = dalloc(p, &p->d_ra2, (size_t)p->R)))
    return bail(rc);
  cudaMemcpyAsync(p->d_roff, roff.data(), ngroups * 8, cudaMemcpyHostToDevice, p->st);
  const bool otf = d.forward_on_the_fly != 0;
  if (otf) {
    // traced during each forward projection (k_forward_otf)
  } else if (d.delta_index) {
    if ((rc = dalloc(p, &p->d_rcoff, (size_t)ngroups)) ||
        (rc = dalloc(p, &p->d_rcode, (size_t)words, true)) ||
        (rc = dalloc(p, &p->d_rstart, (size_t)p->R, true)))
      return bail(rc);
    cudaMemcpyAsync(p->d_rcoff, rcoff.data(), ngroups * 8, cudaMemcpyHostToDevice, p->st);
  } else {
    if ((rc = dalloc(p, &p->d_ridx, (size_t)entries, true))) return bail(rc);
  }
  if (otf) {
  } else if (l16) {
    uint16_t* t;
    if ((rc = dalloc(p, &t, (size_t)entries, true))) return bail(rc);
    p->d_rlen = t;
  } else {
    float* t;
    if ((rc = dalloc(p, &t, (size_t)entries, true))) return bail(rc);
    p->d_rlen = t;
  }
  const size_t dense_n = (size_t)P4 * tiles_x * tiles_y * 32 * 2;
  if (l16) {
    uint16_t* t;
    if ((rc = dalloc(p, &t, dense_n, true))) return bail(rc);
    p->d_dlen = t;
  } else {
    float* t;
    if ((rc = dalloc(p, &t, dense_n, true))) return bail(rc);
    p->d_dlen = t;
  }
  if ((rc = dalloc(p, &p->d_W, (size_t)p->g2))) return bail(rc);
  if (d.half_gathers && (rc = dalloc(p, &p->d_Wh, (size_t)p->g2))) return bail(rc);
  if (p->fp64 && ((rc = dalloc(p, &p->d_ra2d, (size_t)p->R)) ||
                  (rc = dalloc(p, &p->d_W64, (size_t)p->g2))))
    return bail(rc);

  MatrixDev& M = p->M;
  M.roff = p->d_roff;
  M.rcap = p->d_rcap;
  M.rnseg = p->d_rnseg;
  M.ridx = p->d_ridx;
  M.rcode = p->d_rcode;
  M.rcoff = p->d_rcoff;
  M.rstart = p->d_rstart;
  M.rlen = p->d_rlen;
  M.ra2 = p->d_ra2;
  M.dlen = p->d_dlen;
  M.wcoef = p->d_wcoef;
  M.tiles_x = tiles_x;
  M.ntiles = tiles_x * tiles_y;
  M.tw_shift = tw_shift;
  M.P4 = P4;
  M.W = p->d_W;
  M.Wh = p->d_Wh;
  M.len_kind = p->len_kind;
  // half gathers: the backward matrix holds IEEE halves (same size as the
  // 16-bit codes), the operands of the backprojection's mixed FMAs
  M.dlen_kind = (d.half_gathers && l16) ? (int)LK_F16 : p->len_kind;
  M.scale = maxlen > 0 ? 65535.f / maxlen : 1.f;
  M.inv_scale = maxlen > 0 ? maxlen / 65535.f : 1.f;

  // pass 2: fill both matrices; pass 3: total length per pixel
  constexpr int kExcCap = 1 << 16;  // window exceptions a plan accepts
  int4* d_exc_tmp = nullptr;
  int* d_exc_tile_tmp = nullptr;
  if ((rc = dalloc(p, &d_exc_tmp, (size_t)kExcCap)) ||
      (rc = dalloc(p, &d_exc_tile_tmp, (size_t)kExcCap)))
    return bail(rc);
  cudaMemsetAsync(p->d_overflow + 1, 0xff, sizeof(unsigned long long), p->st);
  launch_trace_fill(G, M, p->d_ridx, p->d_rcode, p->d_rstart, p->d_rlen,
                    p->d_ra2, p->d_ra2d, p->d_dlen, p->d_overflow, d_exc_tmp,
                    d_exc_tile_tmp, kExcCap, p->st);
  unsigned long long counters[3] = {0, 0, 0};  // bad steps, first bad ray, exceptions
  cudaMemcpyAsync(counters, p->d_overflow, sizeof(counters), cudaMemcpyDeviceToHost, p->st);
  if (cudaStreamSynchronize(p->st) != cudaSuccess) {
    p->err = std::string("matrix construction failed: ") +
             cudaGetErrorString(cudaGetLastError());
    return bail(TG_E_CUDA);
  }
  const unsigned long long nexc = counters[2];
  if (nexc > (unsigned long long)kExcCap) {
    p->err = std::to_string(nexc) +
             " segments fall outside their pixel's two-column window (more than " +
             std::to_string(kExcCap) + "); geometry not supported by this layout";
    return bail(TG_E_GEOMETRY);
  }
  if (nexc > 0) {
    // window exceptions as a CSR list over the pixel tiles
    std::vector<int4> ex(nexc);
    std::vector<int> et(nexc);
    cudaMemcpy(ex.data(), d_exc_tmp, nexc * sizeof(int4), cudaMemcpyDeviceToHost);
    cudaMemcpy(et.data(), d_exc_tile_tmp, nexc * sizeof(int), cudaMemcpyDeviceToHost);
    std::vector<size_t> order(nexc);
    for (size_t i = 0; i < nexc; ++i) order[i] = i;
    std::sort(order.begin(), order.end(), [&](size_t u, size_t v) {
      if (et[u] != et[v]) return et[u] < et[v];
      if (ex[u].x != ex[v].x) return ex[u].x < ex[v].x;
      if (ex[u].y != ex[v].y) return ex[u].y < ex[v].y;
      return ex[u].z < ex[v].z;
    });
    std::vector<int> first(M.ntiles + 1, 0);
    std::vector<int4> sorted(nexc);
    for (size_t i = 0; i < nexc; ++i) {
      sorted[i] = ex[order[i]];
      ++first[et[order[i]] + 1];
    }
    for (int t = 0; t < M.ntiles; ++t) first[t + 1] += first[t];
    if ((rc = dalloc(p, &p->d_exc_first, (size_t)M.ntiles + 1)) ||
        (rc = dalloc(p, &p->d_exc, (size_t)nexc)))
      return bail(rc);
    cudaMemcpyAsync(p->d_exc_first, first.data(), (M.ntiles + 1) * sizeof(int),
                    cudaMemcpyHostToDevice, p->st);
    cudaMemcpyAsync(p->d_exc, sorted.data(), nexc * sizeof(int4), cudaMemcpyHostToDevice,
                    p->st);
    M.exc_first = p->d_exc_first;
    M.exc = p->d_exc;
  }
  dfree(p, d_exc_tmp, (size_t)kExcCap * sizeof(int4));
  dfree(p, d_exc_tile_tmp, (size_t)kExcCap * sizeof(int));
  if (counters[0] && d.delta_index && !otf) {
    // a stray segment's step does not fit the 4-bit code: this plan's
    // ray-ordered forward projection traces its rays on the fly instead
    dfree(p, p->d_rcode, (size_t)words * sizeof(uint32_t));
    dfree(p, p->d_rstart, (size_t)p->R * sizeof(int));
    dfree(p, p->d_rlen, (size_t)entries * lbytes);
    p->d_rcode = nullptr;
    p->d_rstart = nullptr;
    p->d_rlen = nullptr;
    M.rcode = nullptr;
    M.rstart = nullptr;
    M.rlen = nullptr;
    p->info.forward_traced = 1;
  }
  launch_weights(G, M, d.mode == TG_MODE_EXACT, p->d_W, p->d_Wh, p->st);
  if (p->fp64) launch_weights64(G, M, p->d_W64, p->st);
  p->info.window_exceptions = (int64_t)nexc;
  (void)counters[1];
  if (d.forward_tiles && (rc = build_tiles(p, d_nruns))) {
    if (p->err.empty()) p->err = "building the tile-ordered forward matrix failed";
    return bail(rc);
  }
  // two-stream iterations: tile-staged plans with two or more slice batches
  if (p->tiles && p->nb >= 2 && d.batch_streams != 1) {
    if (cudaStreamCreateWithFlags(&p->st2, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&p->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&p->ev_join, cudaEventDisableTiming) != cudaSuccess) {
      cudaGetLastError();
      p->err = "creating the second stream failed";
      return bail(TG_E_CUDA);
    }
    if ((rc = dalloc(p, &p->d_part2, (size_t)p->info.partial_slots * p->K))) return bail(rc);
    p->two = true;
  }
  cudaEventRecord(e1, p->st);
  cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);

  // PML weights (pml.h:22-29), double literals narrowed to float
  PenaltyWeights& pw = p->pw_base;
  pw.pml[0][0] = (float)0.1464466094;
  pw.pml[0][1] = (float)0.10355339059;
  pw.pml[1][0] = (float)0.226540919667;
  pw.pml[1][1] = (float)0.1601886205;
  pw.pml[2][0] = (float)0.36939806251;
  pw.pml[2][1] = (float)0.26120387496;

  tg_plan_info& I = p->info;
  I.num_segments = nseg_total;
  if (otf) I.forward_traced = 1;
  I.forward_bytes = (otf || p->info.forward_traced) ? 0
                        : entries * (int64_t)lbytes +
                              (d.delta_index ? words * 4 + p->R * 4 : entries * 4);
  I.backward_bytes = (int64_t)dense_n * (int64_t)lbytes;
  I.max_segment_length = maxlen;
  I.setup_ms = ms;
  resolve_noalloc_factors(p);
  *out = p;
  return TG_OK;
}

int tg_plan_set_timing(tg_plan* p, int enable) {
  if (!p) return TG_E_ARG;
  if (p->st) cudaStreamSynchronize(p->st);
  for (auto& u : p->ev_used) {
    p->ev_pool.push_back(u.second.first);
    p->ev_pool.push_back(u.second.second);
  }
  p->ev_used.clear();
  p->timing = enable != 0;
  return TG_OK;
}

int tg_plan_get_timing(tg_plan* p, tg_timing* out) {
  if (!p || !out) return TG_E_ARG;
  TG_CUDA(p, cudaStreamSynchronize(p->st));
  std::memset(out, 0, sizeof(*out));
  for (auto& u : p->ev_used) {
    float ms = 0.f;
    TG_CUDA(p, cudaEventElapsedTime(&ms, u.second.first, u.second.second));
    if (u.first == 0) {
      out->forward_ms += ms;
      out->forward_launches++;
    } else if (u.first == 1) {
      out->backward_ms += ms;
      out->backward_launches++;
    } else {
      out->other_ms += ms;
      out->other_launches++;
    }
  }
  return TG_OK;
}

int tg_plan_destroy(tg_plan* p) {
  if (!p) return TG_OK;
  if (p->st) cudaStreamSynchronize(p->st);
  drop_graphs(p);
  for (auto& u : p->ev_used) {
    cudaEventDestroy(u.second.first);
    cudaEventDestroy(u.second.second);
  }
  for (auto ev : p->ev_pool) cudaEventDestroy(ev);
  for (void* a : p->allocs)
    if (a) cudaFree(a);
  if (p->st2) cudaStreamSynchronize(p->st2);
  if (p->ev_fork) cudaEventDestroy(p->ev_fork);
  if (p->ev_join) cudaEventDestroy(p->ev_join);
  if (p->st2) cudaStreamDestroy(p->st2);
  if (p->st_dl) cudaStreamSynchronize(p->st_dl);
  for (auto ev : p->ev_batch) cudaEventDestroy(ev);
  if (p->ev_dl) cudaEventDestroy(p->ev_dl);
  if (p->st_dl) cudaStreamDestroy(p->st_dl);
  if (p->own) cudaStreamDestroy(p->own);
  delete p;
  return TG_OK;
}

int tg_plan_get_info(const tg_plan* p, tg_plan_info* info) {
  if (!p || !info) return TG_E_ARG;
  *info = p->info;
  info->device_bytes = p->dev_bytes;
  info->batches = p->nb;
  return TG_OK;
}

int tg_plan_set_stream(tg_plan* p, void* stream) {
  if (!p) return TG_E_ARG;
  p->st = stream ? static_cast<cudaStream_t>(stream) : p->own;
  return TG_OK;
}

int tg_synchronize(tg_plan* p) {
  if (!p) return TG_E_ARG;
  TG_CUDA(p, cudaStreamSynchronize(p->st));
  TG_CUDA(p, cudaGetLastError());
  return TG_OK;
}

static int set_sinogram(tg_plan* p, const float* sino, int on_device,
                        int apply_abs, int clip, float clip_min) {
  if (!p || !sino) return p ? fail(p, TG_E_ARG, "null sinogram") : TG_E_ARG;
  const size_t n = (size_t)p->P * p->S * p->C;
  if (!p->d_sino) TG_TRY(dalloc(p, &p->d_sino, (size_t)p->nb * p->R * p->K));
  TG_CUDA(p, cudaMemsetAsync(p->d_sino, 0,
                             (size_t)p->nb * p->R * p->K * sizeof(float), p->st));
  const float* src = sino;
  if (!on_device && !(src = mapped_host(sino, n))) {
    TG_TRY(stage(p, n));
    TG_CUDA(p, cudaMemcpyAsync(p->d_stage, sino, n * sizeof(float),
                               cudaMemcpyHostToDevice, p->st));
    src = p->d_stage;
  }
  launch_sino_pack(src, p->d_sino, p->P, p->S, p->C, p->K, apply_abs, clip, clip_min,
                   p->st);
  TG_CUDA(p, cudaGetLastError());
  // a host sinogram has been read when the call returns
  if (!on_device) TG_CUDA(p, cudaStreamSynchronize(p->st));
  p->have_sino = true;
  return TG_OK;
}

int tg_set_sinogram(tg_plan* p, const float* sino, int on_device, int apply_abs) {
  return set_sinogram(p, sino, on_device, apply_abs, 0, 0.f);
}

int tg_set_sinogram_clip(tg_plan* p, const float* sino, int on_device, int apply_abs,
                         float clip_min) {
  if (p && std::isnan(clip_min)) return fail(p, TG_E_ARG, "clip_min is NaN");
  return set_sinogram(p, sino, on_device, apply_abs, 1, clip_min);
}

int tg_reset_recon(tg_plan* p, int alg) {
  if (!p) return TG_E_ARG;
  TG_TRY(establish_layout(p, alg));
  const float init = alg == TG_SIRT ? 0.f : 1.f;
  for (int b = 0; b < 2; ++b) {
    if (p->fp64)
      launch_fill64(as_f64(p->d_recon[b]), (int64_t)p->nslots * p->g2, init, p->st);
    else
      launch_fill(p->d_recon[b], (size_t)p->nslots * p->g2, init, p->st);
  }
  TG_CUDA(p, cudaGetLastError());
  return TG_OK;
}

int tg_set_recon(tg_plan* p, int alg, const float* recon, int on_device) {
  if (!p || !recon) return p ? fail(p, TG_E_ARG, "null reconstruction") : TG_E_ARG;
  TG_TRY(tg_reset_recon(p, alg));
  const int nuser = p->S + 2 * p->halo;
  const size_t n = (size_t)nuser * p->g2;
  const float* src = recon;
  if (!on_device && !(src = mapped_host(recon, n))) {
    TG_TRY(stage(p, n));
    TG_CUDA(p, cudaMemcpyAsync(p->d_stage, recon, n * sizeof(float),
                               cudaMemcpyHostToDevice, p->st));
    src = p->d_stage;
  }
  // the source is read once; the second buffer is a device copy of the first
  if (p->fp64)
    launch_convert(src, as_f64(p->d_recon[0]) + (int64_t)(p->vshift - p->halo) * p->g2,
                   (int64_t)n, p->st);
  else
    launch_recon_pack(src, p->d_recon[0], nuser, (int)p->g2, p->K,
                      p->vshift - p->halo, p->nslots, p->st);
  TG_CUDA(p, cudaGetLastError());
  TG_CUDA(p, cudaMemcpyAsync(p->d_recon[1], p->d_recon[0],
                             (size_t)p->nslots * p->g2 * (p->fp64 ? 8 : 4),
                             cudaMemcpyDeviceToDevice, p->st));
  // a host reconstruction has been read when the call returns
  if (!on_device) TG_CUDA(p, cudaStreamSynchronize(p->st));
  return TG_OK;
}

int tg_get_recon(tg_plan* p, int alg, float* recon, int on_device) {
  if (!p || !recon) return p ? fail(p, TG_E_ARG, "null output") : TG_E_ARG;
  TG_TRY(check_layout(p, alg));
  const int nuser = p->S + 2 * p->halo;
  const size_t n = (size_t)nuser * p->g2;
  float* dst = recon;
  float* mapped = on_device ? nullptr : mapped_host_out(recon, n);
  if (!on_device) {
    if (mapped) {
      dst = mapped;
    } else {
      TG_TRY(stage(p, n));
      dst = p->d_stage;
    }
  }
  if (p->fp64)
    launch_narrow(as_f64(p->d_recon[p->cur]) + (int64_t)(p->vshift - p->halo) * p->g2,
                  dst, (int64_t)n, p->st);
  else
    launch_recon_unpack(p->d_recon[p->cur], dst, nuser, (int)p->g2, p->K,
                        p->vshift - p->halo, p->st);
  TG_CUDA(p, cudaGetLastError());
  if (mapped) {
    TG_CUDA(p, cudaStreamSynchronize(p->st));
  } else if (!on_device) {
    TG_CUDA(p, cudaMemcpyAsync(recon, p->d_stage, n * sizeof(float),
                               cudaMemcpyDeviceToHost, p->st));
    TG_CUDA(p, cudaStreamSynchronize(p->st));
  }
  return TG_OK;
}

// Forward projection of batch b into per-ray values `out` (FP32): the
// tile-ordered kernel (per-run partial sums, added per ray in path order by
// the finish kernel) when the plan has the tile-ordered matrix, else the
// ray-ordered kernel.
static int run_forward(tg_plan* p, const IterArgs& A0, int b, int out_mode,
                       float* out) {
  const float* src = batch_ptr(p, p->d_recon[p->cur], b * p->K + p->fshift);
  if (p->tiles) {
    IterArgs A = A0;
    A.half_tile = p->d.half_gathers;
    A.half_factors = 0;
    {
      Timed t(p, 0);
      launch_forward_tiled(A, p->T, src, p->d_part, p->st);
    }
    Timed t(p, 2);
    launch_fwd_finish(A, p->T, p->d_part,
                      p->d_sino ? p->d_sino + (int64_t)b * p->R * p->K : nullptr, out,
                      out_mode, p->st);
    return TG_OK;
  }
  const IterArgs& A = A0;
  Timed t(p, 0);
  launch_forward(A, src, p->d_sino + (int64_t)b * p->R * p->K, out, out_mode,
                 p->st);
  return TG_OK;
}

// Storage of the ratio factors of a fused iteration on a plan that has run
// `done` iterations since its reset (FACT_*): on half_gathers plans halves
// of the factor in the first iteration, of (factor - 1) from the second on.
static int factor_storage(const tg_plan* p, int mode, int64_t done) {
  if (!(p->tiles && p->d.half_gathers && mode == FWD_RATIO)) return FACT_F32;
  return done >= 1 ? FACT_HALF_M1 : FACT_HALF;
}

static int half_factors_next(const tg_plan* p, int mode) {
  return factor_storage(p, mode, p->iters_done);
}

// Launches of one fused iteration on the plan's stream (buffers by p->cur;
// the caller flips p->cur and counts the iteration).
// two_streams: the plan's odd slice batches go to its second stream (forked
// from and joined back into p->st), except while the per-kernel timers run.
// after_batch(b, s): called once batch b's backprojection is issued on s.
static void issue_iteration(tg_plan* p, const IterArgs& A0, int mode, bool two_streams,
                            const std::function<void(int, cudaStream_t)>& after_batch = {}) {
  IterArgs A = A0;
  if (p->tiles && p->d.half_gathers) {
    A.half_tile = 1;
    A.half_factors = half_factors_next(p, mode);
  }
  const bool two = two_streams && p->two && !p->timing;
  if (two) {
    cudaEventRecord(p->ev_fork, p->st);
    cudaStreamWaitEvent(p->st2, p->ev_fork, 0);
  }
  for (int b = 0; b < p->nb; ++b) {
    const bool odd = two && (b & 1);
    const cudaStream_t s = odd ? p->st2 : p->st;
    float* upd = odd ? p->d_upd2 : p->d_upd;
    if (p->tiles) {
      float* part = odd ? p->d_part2 : p->d_part;
      const float* src = batch_ptr(p, p->d_recon[p->cur], b * p->K + p->fshift);
      {
        Timed t(p, 0);
        launch_forward_tiled(A, p->T, src, part, s);
      }
      Timed t(p, 2);
      launch_fwd_finish(A, p->T, part, p->d_sino + (int64_t)b * p->R * p->K, upd, mode, s);
    } else {
      run_forward(p, A, b, mode, upd);
    }
    Timed t(p, 1);
    if (!p->d.backward_staged)
      launch_backward(A, b, p->d_recon[p->cur], p->d_recon[p->cur ^ 1], upd, nullptr,
                      EPI_UPDATE, s);
    else
      launch_backward_staged(A, b, p->d_recon[p->cur], p->d_recon[p->cur ^ 1], upd,
                             nullptr, EPI_UPDATE, s);
    if (after_batch) after_batch(b, s);
  }
  if (two) {
    cudaEventRecord(p->ev_join, p->st2);
    cudaStreamWaitEvent(p->st, p->ev_join, 0);
  }
}

// Checks shared by tg_iterate and tg_batch_iterate.
static int iterate_ready(tg_plan* p, int alg, const tg_params* prm) {
  TG_TRY(check_layout(p, alg));
  if (!p->have_sino) return fail(p, TG_E_STATE, "no sinogram uploaded");
  if (alg >= TG_PML && !prm) return fail(p, TG_E_ARG, "penalised algorithms need params");
  return ensure_upd(p);
}

static bool same_params(const tg_params& a, const tg_params* b) {
  const tg_params z{};
  return std::memcmp(&a, b ? b : &z, sizeof(tg_params)) == 0;
}

int tg_plan_set_graphs(tg_plan* p, int enable) {
  if (!p) return TG_E_ARG;
  TG_CUDA(p, cudaStreamSynchronize(p->st));
  drop_graphs(p);
  p->use_graphs = enable != 0;
  return TG_OK;
}

int tg_iterate(tg_plan* p, int alg, const tg_params* prm, int n_iter) {
  if (!p || n_iter < 0) return p ? fail(p, TG_E_ARG, "bad n_iter") : TG_E_ARG;
  TG_TRY(iterate_ready(p, alg, prm));
  const IterArgs A = make_args(p, alg, prm);
  const int mode = alg == TG_SIRT ? FWD_SIRT : FWD_RATIO;
  if (p->fp64) {
    for (int it = 0; it < n_iter; ++it) {
      const double* cur = as_f64(p->d_recon[p->cur]);
      double* next = as_f64(p->d_recon[p->cur ^ 1]);
      double* upd = as_f64(p->d_upd);
      for (int s = 0; s < p->S; ++s) {
        {
          Timed t(p, 0);
          launch_forward64(A, p->d_ra2d, cur + (int64_t)(s + p->fshift) * p->g2,
                           p->d_sino + (int64_t)s * p->R, upd, mode, p->st);
        }
        Timed t(p, 1);
        launch_backward64(A, s, cur, next, upd, p->d_W64, p->st);
      }
      p->cur ^= 1;
    }
    TG_CUDA(p, cudaGetLastError());
    return TG_OK;
  }
  // graphs need a capturable stream and no per-launch timers
  const bool graphs = p->use_graphs && !p->timing && p->st != nullptr;
  for (int it = 0; it < n_iter; ++it) {
    if (graphs) {
      tg_plan::Graph& g = p->graphs[p->cur];
      const int hf = half_factors_next(p, mode);
      if (!g.valid || g.alg != alg || g.half_factors != hf || !same_params(g.prm, prm)) {
        if (g.exec) cudaGraphExecDestroy(g.exec);
        g = tg_plan::Graph();
        cudaGraph_t graph;
        TG_CUDA(p, cudaStreamBeginCapture(p->st, cudaStreamCaptureModeThreadLocal));
        issue_iteration(p, A, mode, true);
        TG_CUDA(p, cudaStreamEndCapture(p->st, &graph));
        const cudaError_t e = cudaGraphInstantiate(&g.exec, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) return fail(p, TG_E_CUDA, cudaGetErrorString(e));
        g.valid = true;
        g.alg = alg;
        g.half_factors = hf;
        g.prm = prm ? *prm : tg_params{};
      }
      TG_CUDA(p, cudaGraphLaunch(g.exec, p->st));
    } else {
      issue_iteration(p, A, mode, true);
    }
    p->cur ^= 1;
    ++p->iters_done;
  }
  TG_CUDA(p, cudaGetLastError());
  return TG_OK;
}

int tg_iterate_get_recon(tg_plan* p, int alg, const tg_params* prm, int n_iter,
                         float* recon, int on_device) {
  if (!p || !recon || n_iter < 0)
    return p ? fail(p, TG_E_ARG, "null output or bad n_iter") : TG_E_ARG;
  TG_TRY(iterate_ready(p, alg, prm));
  const int nuser = p->S + 2 * p->halo;
  const size_t n = (size_t)nuser * p->g2;
  float* dst = on_device ? recon : mapped_host_out(recon, n);
  // Overlapped when the output is device or mapped host memory, the plan
  // runs FP32 without halo slices and without per-kernel timers; else
  // iterate, then download.
  if (n_iter == 0 || !dst || p->halo || p->fp64 || p->timing) {
    TG_TRY(tg_iterate(p, alg, prm, n_iter));
    return tg_get_recon(p, alg, recon, on_device);
  }
  TG_TRY(tg_iterate(p, alg, prm, n_iter - 1));
  if (!p->st_dl &&
      (cudaStreamCreateWithFlags(&p->st_dl, cudaStreamNonBlocking) != cudaSuccess ||
       cudaEventCreateWithFlags(&p->ev_dl, cudaEventDisableTiming) != cudaSuccess)) {
    cudaGetLastError();
    return fail(p, TG_E_CUDA, "creating the download stream failed");
  }
  while ((int)p->ev_batch.size() < p->nb) {
    cudaEvent_t e = nullptr;
    if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) {
      cudaGetLastError();
      return fail(p, TG_E_CUDA, "creating the batch events failed");
    }
    p->ev_batch.push_back(e);
  }
  const IterArgs A = make_args(p, alg, prm);
  const int mode = alg == TG_SIRT ? FWD_SIRT : FWD_RATIO;
  const float* next = p->d_recon[p->cur ^ 1];
  // the download stream follows everything issued so far; each batch's
  // slices go out once its backprojection (the last writer of its slots in
  // this iteration) is done, while the following batches compute
  TG_CUDA(p, cudaEventRecord(p->ev_dl, p->st));
  TG_CUDA(p, cudaStreamWaitEvent(p->st_dl, p->ev_dl, 0));
  issue_iteration(p, A, mode, true, [&](int b, cudaStream_t s) {
    const int s0 = b * p->K;
    const int cnt = std::min(p->K, p->S - s0);
    if (cnt <= 0) return;
    cudaEventRecord(p->ev_batch[b], s);
    cudaStreamWaitEvent(p->st_dl, p->ev_batch[b], 0);
    launch_recon_unpack(next, dst + (int64_t)s0 * p->g2, cnt, (int)p->g2, p->K,
                        p->vshift + s0, p->st_dl);
  });
  TG_CUDA(p, cudaEventRecord(p->ev_dl, p->st_dl));
  TG_CUDA(p, cudaStreamWaitEvent(p->st, p->ev_dl, 0));
  p->cur ^= 1;
  ++p->iters_done;
  TG_CUDA(p, cudaGetLastError());
  // a host reconstruction has been written when the call returns
  if (!on_device) TG_CUDA(p, cudaStreamSynchronize(p->st));
  return TG_OK;
}

// ---- batches of plans: one graph launch per iteration for all of them ------
struct tg_batch {
  std::vector<tg_plan*> plans;
  std::vector<cudaStream_t> streams;  // branch streams of the captured graph
  cudaStream_t main = nullptr;
  cudaEvent_t fork = nullptr;
  std::vector<cudaEvent_t> joins;
  struct Graph {
    bool valid = false;
    std::vector<int> algs;
    std::vector<int> half_factors;  // per plan, as issue_iteration decides
    std::vector<tg_params> prms;
    int cur0 = -1;  // plan 0's buffer parity the graph was captured in
    cudaGraphExec_t exec = nullptr;
  } graphs[2];
  std::string err;
  // Multi-plan launches (every plan fast mode, tile-staged forward, L1
  // backprojection, 16-bit fixed-point lengths): one iteration of all plans
  // is, per slice batch round, one launch per kernel variant whose blocks
  // walk the work items of every plan. Each iteration state (the plans'
  // buffer parities and factor precisions) has its device work items and a
  // CUDA graph of its launches.
  bool multi = false;
  int last_launches = 0;  // kernel launches per iteration, last tg_batch_iterate
  struct State {
    std::string key;
    void* d_items = nullptr;
    cudaGraphExec_t exec = nullptr;
    int launches = 0;
  };
  std::vector<State> states;
};

namespace {

bool multi_eligible(const tg_plan* p) {
  return !p->fp64 && p->tiles && !p->d.backward_staged && p->d.mode == TG_MODE_FAST &&
         p->len_kind == TG_LEN_U16;
}

void drop_states(tg_batch* b) {
  for (auto& s : b->states) {
    if (s.exec) cudaGraphExecDestroy(s.exec);
    if (s.d_items) cudaFree(s.d_items);
  }
  b->states.clear();
}

// A launch of the multi-plan kernels: kind 0 forward, 1 finish, 2 backward;
// its items start at byte `off` of the state's item buffer.
struct MultiLaunch {
  int kind, branch, K, ts, bw, half_tile, comp, dlen, pen, fh;
  size_t off;
  int n;
  int64_t blocks;
};

// Key of iteration `it` (counted from now) of the batch: algorithms,
// parameters, every plan's buffer parity and factor precision then, and the
// addresses of its reconstruction buffers (reallocated when a plan's layout
// changes, which the captured work items must follow).
std::string multi_key(const tg_batch* b, const int* algs, const tg_params* params, int it) {
  std::string k;
  for (size_t i = 0; i < b->plans.size(); ++i) {
    const tg_plan* p = b->plans[i];
    const int mode = algs[i] == TG_SIRT ? FWD_SIRT : FWD_RATIO;
    const int cur = p->cur ^ (it & 1);
    const int hf = factor_storage(p, mode, p->iters_done + it);
    const tg_params prm = params ? params[i] : tg_params{};
    k.append(reinterpret_cast<const char*>(&algs[i]), sizeof(int));
    k.append(reinterpret_cast<const char*>(&prm), sizeof(prm));
    k.append(reinterpret_cast<const char*>(p->d_recon), sizeof(p->d_recon));
    k.push_back((char)(cur | (hf << 1)));
  }
  return k;
}

// Work items and launches of one iteration state. Plans are split into
// branches by the forward kernel they take (slices per pass, tile side and
// precision, summation); a branch's launches form one chain - per round of
// slice batches a forward launch, a finish launch and one backprojection
// launch per (penalty, factor precision) - and branches share no plan, so
// they run concurrently.
void multi_build(const tg_batch* b, const int* algs, const tg_params* params, int it,
                 std::vector<char>& bytes, std::vector<MultiLaunch>& launches) {
  auto put = [&](const void* src, size_t n) {
    const size_t off = (bytes.size() + 15) / 16 * 16;
    bytes.resize(off + n);
    std::memcpy(bytes.data() + off, src, n);
    return off;
  };
  std::map<std::vector<int>, std::vector<int>> branches;  // key -> plan indices
  for (size_t i = 0; i < b->plans.size(); ++i) {
    const tg_plan* p = b->plans[i];
    const int half_tile = p->K == 16 || p->d.half_gathers;
    branches[{p->K, p->T.ts, p->T.bw, half_tile, p->d.compensated}].push_back((int)i);
  }
  int branch = 0;
  for (auto& br : branches) {
    const std::vector<int>& key = br.first;
    int rounds = 0;
    for (int i : br.second) rounds = std::max(rounds, b->plans[i]->nb);
    for (int r = 0; r < rounds; ++r) {
      std::vector<FwdItem> fwd;
      std::vector<FinItem> fin;
      std::map<std::vector<int>, std::vector<BackItem>> back;
      for (int i : br.second) {
        tg_plan* p = b->plans[i];
        if (r >= p->nb) continue;
        const int mode = algs[i] == TG_SIRT ? FWD_SIRT : FWD_RATIO;
        const int cur = p->cur ^ (it & 1);
        const int hf = factor_storage(p, mode, p->iters_done + it);
        IterArgs A = make_args(p, algs[i], params ? &params[i] : nullptr);
        A.half_tile = p->d.half_gathers;
        A.half_factors = hf;
        FwdItem f{};
        f.T = p->T;
        f.recon = batch_ptr(p, p->d_recon[cur], r * p->K + p->fshift);
        f.part = p->d_part;
        f.g = p->C;
        f.inv_scale = A.M.inv_scale;
        f.first = p->T.ntiles;  // block count; turned into offsets below
        fwd.push_back(f);
        FinItem n{};
        n.rnrun = p->T.rnrun;
        n.pbase = p->T.pbase;
        n.ra2 = A.M.ra2;
        n.part = p->d_part;
        n.sino = p->d_sino + (int64_t)r * p->R * p->K;
        n.out = p->d_upd;
        n.nrays = p->R;
        n.first = (p->R + 255) / 256;
        n.out_mode = mode;
        n.fh = hf;
        fin.push_back(n);
        BackItem k{};
        k.A = A;
        k.batch = r;
        k.cur = p->d_recon[cur];
        k.next = p->d_recon[cur ^ 1];
        k.upd = p->d_upd;
        k.first = backward_blocks(A);
        // both half storages share one kernel (each item carries its own)
        back[{A.M.dlen_kind, algs[i] >= TG_PML, hf != FACT_F32}].push_back(k);
      }
      auto emit = [&](int kind, auto& items, int dlen, int pen, int fh) {
        int64_t total = 0;
        for (auto& x : items) {
          const int64_t nb = x.first;
          x.first = total;
          total += nb;
        }
        MultiLaunch l{};
        l.kind = kind;
        l.branch = branch;
        l.K = key[0];
        l.ts = key[1];
        l.bw = key[2];
        l.half_tile = key[3];
        l.comp = key[4];
        l.dlen = dlen;
        l.pen = pen;
        l.fh = fh;
        l.off = put(items.data(), items.size() * sizeof(items[0]));
        l.n = (int)items.size();
        l.blocks = total;
        launches.push_back(l);
      };
      emit(0, fwd, 0, 0, 0);
      emit(1, fin, 0, 0, 0);
      for (auto& c : back) emit(2, c.second, c.first[0], c.first[1], c.first[2]);
    }
    ++branch;
  }
}

// Issues the launches, branch k on stream branch_st[k % n] (forked from and
// joined back into `st` by the caller).
void multi_issue(const std::vector<MultiLaunch>& launches, const char* d_items,
                 const std::vector<cudaStream_t>& branch_st) {
  for (const MultiLaunch& l : launches) {
    const void* items = d_items + l.off;
    const cudaStream_t st = branch_st[l.branch % branch_st.size()];
    if (l.kind == 0)
      launch_forward_tiled_multi(static_cast<const FwdItem*>(items), l.n, l.blocks, l.K,
                                 l.ts, l.bw, l.half_tile, l.comp, st);
    else if (l.kind == 1)
      launch_fwd_finish_multi(static_cast<const FinItem*>(items), l.n, l.blocks, l.K, l.comp,
                              st);
    else
      launch_backward_multi(static_cast<const BackItem*>(items), l.n, l.blocks, l.K, l.dlen,
                            l.pen, l.fh, l.comp, st);
  }
}

// The state of iteration `it`, built (items uploaded, launches captured)
// when it is new. Keeps the most recent few.
int multi_state(tg_batch* b, const int* algs, const tg_params* params, int it,
                tg_batch::State** out) {
  const std::string key = multi_key(b, algs, params, it);
  for (auto& s : b->states)
    if (s.key == key) {
      *out = &s;
      return TG_OK;
    }
  if (b->states.size() >= 6) {
    cudaStreamSynchronize(b->main);
    if (b->states.front().exec) cudaGraphExecDestroy(b->states.front().exec);
    if (b->states.front().d_items) cudaFree(b->states.front().d_items);
    b->states.erase(b->states.begin());
  }
  std::vector<char> bytes;
  std::vector<MultiLaunch> launches;
  multi_build(b, algs, params, it, bytes, launches);
  tg_batch::State s;
  s.key = key;
  s.launches = (int)launches.size();
  cudaError_t e = cudaMalloc(&s.d_items, std::max<size_t>(bytes.size(), 16));
  if (e == cudaSuccess)
    e = cudaMemcpy(s.d_items, bytes.data(), bytes.size(), cudaMemcpyHostToDevice);
  cudaGraph_t graph = nullptr;
  if (e == cudaSuccess) e = cudaStreamBeginCapture(b->main, cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess) {
    // fork the branch streams from `main`, issue, join them back
    int nbranch = 0;
    for (const MultiLaunch& l : launches) nbranch = std::max(nbranch, l.branch + 1);
    const int ns = std::min<int>(nbranch, (int)b->streams.size());
    std::vector<cudaStream_t> bst(b->streams.begin(), b->streams.begin() + std::max(ns, 1));
    cudaError_t ef = cudaEventRecord(b->fork, b->main);
    for (int k = 0; ef == cudaSuccess && k < ns; ++k)
      ef = cudaStreamWaitEvent(bst[k], b->fork, 0);
    if (ef == cudaSuccess) multi_issue(launches, static_cast<const char*>(s.d_items), bst);
    for (int k = 0; ef == cudaSuccess && k < ns; ++k) {
      ef = cudaEventRecord(b->joins[k], bst[k]);
      if (ef == cudaSuccess) ef = cudaStreamWaitEvent(b->main, b->joins[k], 0);
    }
    const cudaError_t e1 = ef != cudaSuccess ? ef : cudaGetLastError();
    const cudaError_t e2 = cudaStreamEndCapture(b->main, &graph);
    e = e1 != cudaSuccess ? e1 : e2;
  }
  if (e == cudaSuccess) e = cudaGraphInstantiate(&s.exec, graph, 0);
  if (graph) cudaGraphDestroy(graph);
  if (e != cudaSuccess) {
    if (s.d_items) cudaFree(s.d_items);
    b->err = std::string("multi-plan iteration setup failed: ") + cudaGetErrorString(e);
    return TG_E_CUDA;
  }
  b->states.push_back(s);
  *out = &b->states.back();
  return TG_OK;
}

}  // namespace

extern "C" int tg_batch_create(tg_plan* const* plans, int n, tg_batch** out) {
  if (!plans || n < 1 || !out) return fail(nullptr, TG_E_ARG, "need plans");
  *out = nullptr;
  for (int i = 0; i < n; ++i)
    if (!plans[i] || plans[i]->fp64)
      return fail(nullptr, TG_E_ARG, "batch plans must be FP32 plans");
  tg_batch* b = new (std::nothrow) tg_batch();
  if (!b) return fail(nullptr, TG_E_NOMEM, "host allocation failed");
  b->plans.assign(plans, plans + n);
  b->multi = true;
  for (int i = 0; i < n; ++i) b->multi = b->multi && multi_eligible(plans[i]);
  const int nstreams = n < 16 ? n : 16;
  bool ok = cudaStreamCreateWithFlags(&b->main, cudaStreamNonBlocking) == cudaSuccess &&
            cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) == cudaSuccess;
  for (int i = 0; ok && i < nstreams; ++i) {
    cudaStream_t s;
    cudaEvent_t e;
    ok = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) == cudaSuccess &&
         cudaEventCreateWithFlags(&e, cudaEventDisableTiming) == cudaSuccess;
    if (ok) {
      b->streams.push_back(s);
      b->joins.push_back(e);
    }
  }
  if (!ok) {
    g_create_error = "stream/event creation failed";
    tg_batch_destroy(b);
    return TG_E_CUDA;
  }
  *out = b;
  return TG_OK;
}

extern "C" int tg_batch_destroy(tg_batch* b) {
  if (!b) return TG_OK;
  if (b->main) cudaStreamSynchronize(b->main);
  drop_states(b);
  for (auto& g : b->graphs)
    if (g.exec) cudaGraphExecDestroy(g.exec);
  for (auto s : b->streams) cudaStreamDestroy(s);
  for (auto e : b->joins) cudaEventDestroy(e);
  if (b->fork) cudaEventDestroy(b->fork);
  if (b->main) cudaStreamDestroy(b->main);
  delete b;
  return TG_OK;
}

extern "C" int tg_batch_get_info(const tg_batch* b, int* multi, int* launches) {
  if (!b) return TG_E_ARG;
  if (multi) *multi = b->multi ? 1 : 0;
  if (launches) *launches = b->last_launches;
  return TG_OK;
}

extern "C" const char* tg_batch_last_error(const tg_batch* b) {
  return b ? b->err.c_str() : g_create_error.c_str();
}

extern "C" int tg_batch_synchronize(tg_batch* b) {
  if (!b) return TG_E_ARG;
  const cudaError_t e = cudaStreamSynchronize(b->main);
  if (e != cudaSuccess) {
    b->err = cudaGetErrorString(e);
    return TG_E_CUDA;
  }
  return TG_OK;
}

extern "C" int tg_batch_iterate(tg_batch* b, const int* algs, const tg_params* params,
                                int n_iter) {
  if (!b || !algs || n_iter < 0) return TG_E_ARG;
  const int n = (int)b->plans.size();
  for (int i = 0; i < n; ++i) {
    tg_plan* p = b->plans[i];
    const int rc = iterate_ready(p, algs[i], params ? &params[i] : nullptr);
    if (rc) {
      b->err = "plan " + std::to_string(i) + ": " + p->err;
      return rc;
    }
    if (p->timing) {
      b->err = "plan " + std::to_string(i) + " has per-kernel timers on";
      return TG_E_STATE;
    }
  }
  // plans' own streams must be done before the graph (on `main`) reads their data
  for (tg_plan* p : b->plans) cudaStreamSynchronize(p->st);
  if (b->multi) {
    for (int it = 0; it < n_iter; ++it) {
      tg_batch::State* s = nullptr;
      const int rc = multi_state(b, algs, params, 0, &s);
      if (rc) return rc;
      b->last_launches = s->launches;
      const cudaError_t e = cudaGraphLaunch(s->exec, b->main);
      if (e != cudaSuccess) {
        b->err = cudaGetErrorString(e);
        return TG_E_CUDA;
      }
      for (tg_plan* p : b->plans) {
        p->cur ^= 1;
        ++p->iters_done;
      }
    }
    const cudaError_t e = cudaStreamSynchronize(b->main);
    if (e != cudaSuccess) {
      b->err = cudaGetErrorString(e);
      return TG_E_CUDA;
    }
    return TG_OK;
  }
  b->last_launches = 0;
  for (tg_plan* p : b->plans) b->last_launches += p->nb * (p->tiles ? 3 : 2);
  for (int it = 0; it < n_iter; ++it) {
    const int parity = b->plans[0]->cur;
    tg_batch::Graph& g = b->graphs[parity];
    std::vector<int> hf(n);
    for (int i = 0; i < n; ++i)
      hf[i] = half_factors_next(b->plans[i], algs[i] == TG_SIRT ? FWD_SIRT : FWD_RATIO);
    bool match = g.valid && g.cur0 == parity && g.half_factors == hf;
    for (int i = 0; match && i < n; ++i)
      match = g.algs[i] == algs[i] &&
              same_params(g.prms[i], params ? &params[i] : nullptr);
    if (!match) {
      if (g.exec) cudaGraphExecDestroy(g.exec);
      g = tg_batch::Graph();
      cudaGraph_t graph;
      cudaError_t e = cudaStreamBeginCapture(b->main, cudaStreamCaptureModeThreadLocal);
      if (e == cudaSuccess) e = cudaEventRecord(b->fork, b->main);
      const int ns = (int)b->streams.size();
      for (int s = 0; e == cudaSuccess && s < ns; ++s)
        e = cudaStreamWaitEvent(b->streams[s], b->fork, 0);
      for (int i = 0; e == cudaSuccess && i < n; ++i) {
        tg_plan* p = b->plans[i];
        const cudaStream_t keep = p->st;
        p->st = b->streams[i % ns];
        const IterArgs A = make_args(p, algs[i], params ? &params[i] : nullptr);
        issue_iteration(p, A, algs[i] == TG_SIRT ? FWD_SIRT : FWD_RATIO, false);
        p->st = keep;
      }
      for (int s = 0; e == cudaSuccess && s < ns; ++s) {
        e = cudaEventRecord(b->joins[s], b->streams[s]);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(b->main, b->joins[s], 0);
      }
      const cudaError_t e2 = cudaStreamEndCapture(b->main, &graph);
      if (e == cudaSuccess) e = e2;
      if (e == cudaSuccess) {
        e = cudaGraphInstantiate(&g.exec, graph, 0);
        cudaGraphDestroy(graph);
      }
      if (e != cudaSuccess) {
        b->err = std::string("graph capture failed: ") + cudaGetErrorString(e);
        return TG_E_CUDA;
      }
      g.valid = true;
      g.cur0 = parity;
      g.half_factors = hf;
      g.algs.assign(algs, algs + n);
      for (int i = 0; i < n; ++i) g.prms.push_back(params ? params[i] : tg_params{});
    }
    const cudaError_t e = cudaGraphLaunch(g.exec, b->main);
    if (e != cudaSuccess) {
      b->err = cudaGetErrorString(e);
      return TG_E_CUDA;
    }
    for (tg_plan* p : b->plans) {
      p->cur ^= 1;
      ++p->iters_done;
    }
  }
  // later calls on the plans' own streams see the batch's results
  const cudaError_t e = cudaStreamSynchronize(b->main);
  if (e != cudaSuccess) {
    b->err = cudaGetErrorString(e);
    return TG_E_CUDA;
  }
  return TG_OK;
}

int tg_reduce(tg_plan* p, int alg, const tg_params* prm) {
  if (!p) return TG_E_ARG;
  TG_TRY(fp32_only(p));
  TG_TRY(check_layout(p, alg));
  if (!p->have_sino) return fail(p, TG_E_STATE, "no sinogram uploaded");
  TG_TRY(ensure_upd(p));
  if (!p->d_rep) TG_TRY(dalloc(p, &p->d_rep, (size_t)p->S * p->g2, true));
  const IterArgs A = make_args(p, alg, prm);
  const int mode = alg == TG_SIRT ? FWD_SIRT : FWD_RATIO;
  for (int b = 0; b < p->nb; ++b) {
    run_forward(p, A, b, mode, p->d_upd);
    Timed t(p, 1);
    if (!p->d.backward_staged)
      launch_backward(A, b, p->d_recon[p->cur], nullptr, p->d_upd, p->d_rep,
                      EPI_REPLICA, p->st);
    else
      launch_backward_staged(A, b, p->d_recon[p->cur], nullptr, p->d_upd,
                             p->d_rep, EPI_REPLICA, p->st);
  }
  TG_CUDA(p, cudaGetLastError());
  return TG_OK;
}

int tg_get_replica(tg_plan* p, int alg, float* replica, int on_device) {
  if (!p || !replica) return p ? fail(p, TG_E_ARG, "null output") : TG_E_ARG;
  TG_TRY(check_layout(p, alg));
  if (!p->d_rep) return fail(p, TG_E_STATE, "no replica: call tg_reduce first");
  const size_t n = (size_t)p->S * p->g2 * 2;
  float* dst = replica;
  float* mapped = on_device ? nullptr : mapped_host_out(replica, n);
  if (!on_device) {
    if (mapped) {
      dst = mapped;
    } else {
      TG_TRY(stage(p, n));
      dst = p->d_stage;
    }
  }
  launch_replica_interleave(p->d_rep, p->d_W, dst, p->S, (int)p->g2, p->st);
  TG_CUDA(p, cudaGetLastError());
  if (mapped) {
    TG_CUDA(p, cudaStreamSynchronize(p->st));
  } else if (!on_device) {
    TG_CUDA(p, cudaMemcpyAsync(replica, p->d_stage, n * sizeof(float),
                               cudaMemcpyDeviceToHost, p->st));
    TG_CUDA(p, cudaStreamSynchronize(p->st));
  }
  return TG_OK;
}

int tg_reset_replica(tg_plan* p) {
  if (!p) return TG_E_ARG;
  if (p->d_rep)
    TG_CUDA(p, cudaMemsetAsync(p->d_rep, 0, (size_t)p->S * p->g2 * sizeof(float), p->st));
  return TG_OK;
}

int tg_calculate_fg(tg_plan* p, int alg, const tg_params* prm) {
  if (!p) return TG_E_ARG;
  TG_TRY(fp32_only(p));
  TG_TRY(check_layout(p, alg));
  if (alg < TG_PML) return fail(p, TG_E_ARG, "CalculateFG exists for PML and APMLR only");
  if (!prm) return fail(p, TG_E_ARG, "null params");
  if (!p->d_F) {
    TG_TRY(dalloc(p, &p->d_F, (size_t)p->S * p->g2));
    TG_TRY(dalloc(p, &p->d_G, (size_t)p->S * p->g2));
  }
  const IterArgs A = make_args(p, alg, prm);
  Timed t(p, 2);
  launch_fg(A, p->d_recon[p->cur], p->d_W, p->d_F, p->d_G, p->st);
  TG_CUDA(p, cudaGetLastError());
  return TG_OK;
}

int tg_get_fg(tg_plan* p, float* F, float* G, int on_device) {
  if (!p || !F || !G) return p ? fail(p, TG_E_ARG, "null output") : TG_E_ARG;
  if (!p->d_F) return fail(p, TG_E_STATE, "no F/G: call tg_calculate_fg first");
  const size_t bytes = (size_t)p->S * p->g2 * sizeof(float);
  const cudaMemcpyKind kind = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
  TG_CUDA(p, cudaMemcpyAsync(F, p->d_F, bytes, kind, p->st));
  TG_CUDA(p, cudaMemcpyAsync(G, p->d_G, bytes, kind, p->st));
  TG_CUDA(p, cudaStreamSynchronize(p->st));
  return TG_OK;
}

int tg_update_recon(tg_plan* p, int alg, const tg_params* prm) {
  if (!p) return TG_E_ARG;
  TG_TRY(fp32_only(p));
  TG_TRY(check_layout(p, alg));
  if (!p->d_rep) return fail(p, TG_E_STATE, "no replica: call tg_reduce first");
  if (alg >= TG_PML && !p->d_F)
    return fail(p, TG_E_STATE, "call tg_calculate_fg before tg_update_recon");
  const IterArgs A = make_args(p, alg, prm);
  float* cur = p->d_recon[p->cur];
  Timed t(p, 2);
  launch_update(A, cur, p->d_W, p->d_F, p->d_G, p->d_rep, p->st);
  // keep the other buffer's copy identical so fused and operator calls mix
  TG_CUDA(p, cudaMemcpyAsync(p->d_recon[p->cur ^ 1], cur,
                             (size_t)p->nslots * p->g2 * sizeof(float),
                             cudaMemcpyDeviceToDevice, p->st));
  TG_CUDA(p, cudaGetLastError());
  return TG_OK;
}

int tg_forward_project(tg_plan* p, int alg, const tg_params* prm, float* sim,
                       int on_device) {
  if (!p || !sim) return p ? fail(p, TG_E_ARG, "null output") : TG_E_ARG;
  TG_TRY(fp32_only(p));
  TG_TRY(check_layout(p, alg));
  const size_t packed = (size_t)p->nb * p->R * p->K;
  const size_t n = (size_t)p->P * p->S * p->C;
  float* mapped = on_device ? nullptr : mapped_host_out(sim, n);
  const bool staged = !on_device && !mapped;
  TG_TRY(stage(p, packed + (staged ? n : 0)));
  const IterArgs A = make_args(p, alg, prm);
  for (int b = 0; b < p->nb; ++b)
    run_forward(p, A, b, FWD_SIM, p->d_stage + (int64_t)b * p->R * p->K);
  float* dst = on_device ? sim : mapped ? mapped : p->d_stage + packed;
  launch_sino_unpack(p->d_stage, dst, p->P, p->S, p->C, p->K, p->st);
  TG_CUDA(p, cudaGetLastError());
  if (staged)
    TG_CUDA(p, cudaMemcpyAsync(sim, dst, n * sizeof(float), cudaMemcpyDeviceToHost, p->st));
  TG_CUDA(p, cudaStreamSynchronize(p->st));
  return TG_OK;
}

int tg_trace_rays(tg_plan* p, int32_t* counts, const int64_t* offsets,
                  int32_t* idx, float* len, float* len2) {
  if (!p || !counts) return p ? fail(p, TG_E_ARG, "null counts") : TG_E_ARG;
  std::memcpy(counts, p->h_nseg.data(), p->R * sizeof(int32_t));
  if (!idx) return TG_OK;
  if (!offsets || !len) return fail(p, TG_E_ARG, "offsets and len are required with idx");
  const int64_t total = offsets[p->R];
  int64_t* d_off = nullptr;
  int* d_idx = nullptr;
  float *d_len = nullptr, *d_len2 = nullptr;
  int rc;
  if ((rc = dalloc(p, &d_off, (size_t)p->R + 1)) || (rc = dalloc(p, &d_idx, (size_t)total)) ||
      (rc = dalloc(p, &d_len, (size_t)total)) ||
      (len2 && (rc = dalloc(p, &d_len2, (size_t)total))))
    return rc;
  TG_CUDA(p, cudaMemcpyAsync(d_off, offsets, (p->R + 1) * 8, cudaMemcpyHostToDevice, p->st));
  launch_trace_export(p->G, d_off, d_idx, d_len, d_len2, p->st);
  TG_CUDA(p, cudaMemcpyAsync(idx, d_idx, total * 4, cudaMemcpyDeviceToHost, p->st));
  TG_CUDA(p, cudaMemcpyAsync(len, d_len, total * 4, cudaMemcpyDeviceToHost, p->st));
  if (len2) TG_CUDA(p, cudaMemcpyAsync(len2, d_len2, total * 4, cudaMemcpyDeviceToHost, p->st));
  TG_CUDA(p, cudaStreamSynchronize(p->st));
  dfree(p, d_off, (p->R + 1) * 8);
  dfree(p, d_idx, total * 4);
  dfree(p, d_len, total * 4);
  dfree(p, d_len2, len2 ? total * 4 : 0);
  return TG_OK;
}

}  // extern "C"

// ---- allocation-free single-slice reduce ------------------------------------
// For callers that may not allocate device memory while they run (see the
// declaration in trace_gb300.h): the per-ray factors the forward pass hands
// to the backprojection go to this fixed array instead of the plan's buffer.
namespace {

constexpr int64_t kNoAllocMaxRays = int64_t(1) << 22;  // 4,194,304 floats
static __device__ __align__(256) float g_noalloc_factors[kNoAllocMaxRays];

}  // namespace

// Device address of the array in the current context, stored in the plan at
// its creation (the plan's device is current then; in host code the array's
// name is only a host-side stand-in, never a device address). A plan lives
// in one context, so the address cannot go stale under it; looking it up
// here also loads the array on the device before any allocation-free call.
static void resolve_noalloc_factors(tg_plan* p) {
  void* addr = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&addr, g_noalloc_factors);
  if (e != cudaSuccess || !addr) {
    cudaGetLastError();
    p->noalloc_err = std::string("cudaGetSymbolAddress of the factor array: ") +
                     cudaGetErrorString(e);
    return;
  }
  p->noalloc_factors = static_cast<float*>(addr);
}

extern "C" int tg_reduce_slice_noalloc(tg_plan* p, int alg,
                                       const tg_params* prm, const float* recon,
                                       const float* sino, float* num) {
  if (!p) return TG_E_ARG;
  if (!recon || !sino || !num) return fail(p, TG_E_ARG, "null device buffer");
  if (!valid_alg(alg)) return fail(p, TG_E_ARG, "unknown algorithm");
  TG_TRY(fp32_only(p));
  if (p->R > kNoAllocMaxRays)
    return fail(p, TG_E_LIMIT,
                "P*C = " + std::to_string(p->R) +
                    " rays exceeds the 4,194,304-ray factor array of "
                    "tg_reduce_slice_noalloc");
  if (!p->noalloc_factors) return fail(p, TG_E_CUDA, p->noalloc_err);
  float* factors = p->noalloc_factors;
  IterArgs A = make_args(p, alg, prm);
  A.K = 1;  // one slice: plain [C*C] / [P*C] layouts
  A.S = 1;
  A.vshift = 0;
  A.fshift = 0;
  A.nslots = 1;
  launch_forward(A, recon, sino, factors, alg == TG_SIRT ? FWD_SIRT : FWD_RATIO,
                 p->st);
  launch_backward(A, 0, recon, nullptr, factors, num, EPI_REPLICA, p->st);
  TG_CUDA(p, cudaGetLastError());
  return TG_OK;
}
