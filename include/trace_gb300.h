/* trace_gb300 — GB300 (sm_103a) implementation of Trace's iterative
 * reconstruction hot path behind a plain C ABI.
 *
 * One plan holds one parallel-beam geometry (num_projs angles x num_cols
 * detector columns, grid = num_cols), the sinogram of num_slices slices, the
 * reconstruction, and the device-resident system matrix traced once from the
 * geometry. Calls replace, for that path, the reference's operator surface:
 *
 *   reference (file:line in tekinbicer/Trace)          replaced by
 *   ------------------------------------------------   --------------------------
 *   TraceMetadata ctor, src/common/trace_data.h:53-109  tg_plan_create
 *   DataRegionBase over the sinogram,
 *     src/common/DISP/core/data_region_base.h:48-51    tg_set_sinogram
 *   trace_utils::Absolute, src/common/trace_utils.cc:4-8  tg_set_sinogram(abs=1)
 *   (no counterpart: sinogram floor before MLEM's ratio)  tg_set_sinogram_clip
 *   trace_utils::DegreeToRadian, trace_utils.cc:10-24   tg_degree_to_radian
 *   trace_utils::Calculate* tracer chain,
 *     src/common/trace_utils.cc:41-216                  tg_trace_rays (export)
 *   DISPEngineReduction::RunParallelReduction +
 *     XReconSpace::Reduce (sirt.cc:97-186, mlem.cc:92-181,
 *     pml.cc:276-366, apmlr.cc:1057-1147)               tg_reduce
 *   ParInPlaceLocalSynchWrapper,
 *     disp_engine_reduction.h:132-167                   (no-op: one device replica)
 *   XReconSpace::reduction_objects(),
 *     reduction_space_a.h:40-42                         tg_get_replica
 *   PMLReconSpace::CalculateFG pml.cc:25-201 /
 *     APMLRReconSpace::CalculateFG apmlr.cc:919-982     tg_calculate_fg
 *   XReconSpace::UpdateRecon sirt.cc:21-33, mlem.cc:21-34,
 *     pml.cc:3-23, apmlr.cc:3-26                        tg_update_recon
 *   ResetReductionSpaces, disp_engine_reduction.h:188-202  tg_reset_replica
 *   the drivers' iteration loop, e.g.
 *     src/sirt/sirt_main.cc:177-202                     tg_iterate (fused)
 *   TraceMetadata::recon(), trace_data.h:169            tg_get_recon / tg_set_recon
 *
 * Conventions: every function returns 0 on success or a TG_E* code; the
 * message of the last failure on a plan is tg_last_error(plan) (or
 * tg_last_error(NULL) for a failed tg_plan_create). No call throws. The
 * library owns device memory; callers own host buffers. Each plan issues its
 * work on one CUDA stream (its own, or one given with tg_plan_set_stream);
 * tg_iterate may fork part of an iteration onto the plan's own second stream
 * (batch_streams) and joins it back into that stream before returning, so
 * callers see stream order as if one stream did all the work. Calls on one
 * plan are not thread-safe; distinct plans are independent.
 *
 * Host buffers (on_device = 0): a page-locked buffer (cudaHostAlloc,
 * cudaMallocHost, or cudaHostRegister'ed and mapped) is read or written in
 * place by the kernels that convert between the reference layout and the
 * device layout, across the CPU-GPU link, with no device staging copy; a
 * pageable buffer, and a download into memory registered read-only
 * (cudaHostRegisterReadOnly), go through a device staging buffer. Either
 * way a call that takes a host buffer returns after it has read (uploads)
 * or written (downloads) it.
 */
#ifndef TRACE_GB300_H
#define TRACE_GB300_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TG_ABI_VERSION 1

enum tg_status {
  TG_OK = 0,
  TG_E_ARG = 1,      /* invalid argument (null pointer, bad size, bad enum) */
  TG_E_CUDA = 2,     /* a CUDA runtime call failed */
  TG_E_NOMEM = 3,    /* device allocation failed */
  TG_E_STATE = 4,    /* call out of order (e.g. no sinogram uploaded) */
  TG_E_GEOMETRY = 5, /* geometry outside what the plan's layout supports */
  TG_E_LIMIT = 6     /* request exceeds a fixed limit of the entry point */
};

enum tg_alg { TG_SIRT = 0, TG_MLEM = 1, TG_PML = 2, TG_APMLR = 3 };

/* Storage of the traced segment lengths in the device system matrix.
 * Arithmetic is FP32 in every case. */
enum tg_len_storage {
  TG_LEN_F32 = 0,  /* float32 lengths */
  TG_LEN_BF16 = 1, /* bfloat16 */
  TG_LEN_F16 = 2,  /* IEEE half */
  TG_LEN_U16 = 3   /* 16-bit fixed point, scale = longest segment / 65535 */
};

/* Arithmetic mode of the iteration kernels. */
enum tg_mode {
  TG_MODE_EXACT = 0, /* reference operation order, IEEE-rounded mul/add/div:
                        forward ray sums are bit-identical to the reference */
  TG_MODE_FAST = 1,  /* fused multiply-add accumulation */
  TG_MODE_FP64 = 2   /* reconstruction, factors, sums and updates in double
                        (f32 lengths, one slice per pass, tg_iterate only):
                        the FP64 run errors are measured against */
};

typedef struct {
  int num_projs;          /* P: angles */
  int num_slices;         /* S: sinogram slices held by this plan */
  int num_cols;           /* C: detector columns; the grid is C x C */
  float center;           /* rotation centre; <= 0 selects C/2 + 1 */
  int slice_id;           /* global index of this plan's first slice */
  int num_total_slices;   /* slices in the whole dataset (APMLR top/bottom) */
  int len_storage;        /* tg_len_storage */
  int slices_per_pass;    /* k in {1,2,4,8,16}: slices served per matrix read
                             (16 with forward_tiles needs half_gathers) */
  int mode;               /* tg_mode */
  int delta_index;        /* 1 = forward pixel indices delta-coded (4 bits) */
  int apmlr_fixed_offset; /* APMLR only. 0 = reference behaviour: the forward
                             projection of slice s reads reconstruction slice
                             s-1 (apmlr.cc:1083-1084); 1 = reads slice s */
  int forward_tiles;      /* fast mode only: tg_iterate runs the forward
                             projection through square reconstruction tiles
                             (forward_tile_side) staged in shared memory (an
                             extra tile-ordered copy of the forward matrix
                             is built) */
  int backward_staged;    /* fast mode only: the backprojection stages each
                             16x16-pixel block's detector windows in shared
                             memory instead of gathering through L1 */
  int half_gathers;       /* fast mode with forward_tiles, L1 backprojection:
                             tg_iterate keeps the gathered operands as IEEE
                             halves with FP32 arithmetic - the forward
                             projection's shared-memory reconstruction tile,
                             and (MLEM/PML/APMLR) the per-ray factors as
                             factor - 1 - halving the bytes of both gathers;
                             the backward matrix then stores its lengths as
                             halves (16-bit storages). The first iteration
                             after tg_reset_recon / tg_set_recon stores
                             halves of the factors themselves (they start
                             anywhere between 0 and their largest value,
                             where a half of factor - 1 loses the small
                             ones). tg_reduce keeps FP32 factors (half
                             tile) */
  int forward_on_the_fly; /* not with FP64 mode: no ray-ordered forward matrix
                             is stored; the forward projections that would
                             read it (tg_iterate, tg_reduce and
                             tg_forward_project on plans without
                             forward_tiles) trace each ray while projecting
                             it. Saves the matrix's memory (segments x
                             (L + 4) bytes) for tracing work; results equal
                             the stored f32 form's. With forward_tiles the
                             projections use the tile-ordered matrix and the
                             option only saves memory (the tile build traces
                             instead of reading the ray-ordered matrix) */
  int compensated;        /* fast mode with forward_tiles, the L1
                             backprojection and at most 8 slices per pass:
                             compensated (Kahan) summation -
                             each ray's sum in blocks of 8 segments within a
                             tile run and across its runs, each pixel's
                             backprojection sum in blocks of 4 angles; the
                             blocks themselves are FMA chains */
  int backward_tile_width; /* pixels per warp row of the backward matrix and
                              backprojection: 8 (8x4 tiles; 0 selects it),
                              16 (16x2) or 4 (4x8); backward_staged needs 8 */
  int forward_tile_side;   /* forward_tiles: side of the shared-memory
                              reconstruction tiles, 32, 48, 64 (0 selects
                              it), 80 or 96; the tile of slices_per_pass
                              slices must fit
                              shared memory (96 needs half_gathers and at
                              most 8 slices per pass) */
  int batch_streams;       /* forward_tiles with two or more slice batches:
                              2 (0 selects it) - tg_iterate runs odd batches
                              on a second stream with their own partial sums
                              and factors (one more partial-sum buffer), so
                              one batch's forward projection overlaps the
                              previous batch's finish and backprojection;
                              1 - every batch on the plan's stream. Results
                              are the same bits either way */
  int forward_block_warps; /* forward_tiles: warps of each tile's block, i.e.
                              runs (one per lane) in flight per tile: 32 (0
                              selects it), 16 or 8; same results */
} tg_plan_desc;

typedef struct {
  float beta;    /* PML beta; APMLR in-plane beta0 */
  float beta1;   /* APMLR axial beta */
  float delta;   /* APMLR in-plane delta0 */
  float delta1;  /* APMLR axial delta */
  float regw;    /* APMLR axial weight */
} tg_params;

typedef struct {
  int64_t num_segments;       /* traced ray-pixel segments (one slice) */
  int64_t forward_bytes;      /* bytes of the forward (ray-major) matrix */
  int64_t backward_bytes;     /* bytes of the backward (pixel-major) matrix */
  int64_t device_bytes;       /* all device memory held by the plan */
  float max_segment_length;
  double setup_ms;            /* time spent tracing and building matrices */
  int batches;                /* ceil(stored slices / slices_per_pass) */
  int64_t tile_bytes;         /* bytes of the tile-ordered forward matrix */
  int64_t tile_runs;          /* runs (ray pieces inside one tile) */
  int64_t window_exceptions;  /* segments kept apart from the backward matrix:
                                 the reference's tracer can place a stray
                                 segment far from its ray (near-vertical
                                 angles, edge columns); they are added to
                                 their pixels from a short per-tile list */
  int forward_traced;         /* 1: the ray-ordered forward projection traces
                                 its rays on the fly - requested, or a stray
                                 segment's step did not fit the 4-bit code */
  int64_t partial_slots;      /* tile-staged forward: slots of the runs'
                                 partial sums (slices_per_pass floats each),
                                 written by every forward launch and summed
                                 per ray in a fixed order */
} tg_plan_info;

typedef struct {
  double forward_ms;          /* summed device time of forward launches */
  double backward_ms;         /* backprojection (+ fused update) launches */
  double other_ms;            /* operator-level penalty/update launches */
  int64_t forward_launches, backward_launches, other_launches;
} tg_timing;

typedef struct tg_plan tg_plan;

int tg_abi_version(void);

/* Create a plan: traces every ray of the geometry on the device and builds
 * the forward and backward matrices. theta (P floats, radians) is required.
 * sin_tab / cos_tab (P floats each, both or neither) replace the host
 * C library's sinf/cosf values the reference uses (sirt.cc:119-120). */
int tg_plan_create(const tg_plan_desc* desc, const float* theta,
                   const float* sin_tab, const float* cos_tab, tg_plan** out);
int tg_plan_destroy(tg_plan* plan);
int tg_plan_get_info(const tg_plan* plan, tg_plan_info* info);
/* Use `stream` (a cudaStream_t) for all later work of this plan; NULL
 * returns to the plan's own stream. */
int tg_plan_set_stream(tg_plan* plan, void* stream);
int tg_synchronize(tg_plan* plan);
const char* tg_last_error(const tg_plan* plan);

/* Per-kernel device timers (CUDA events around each launch on the plan's
 * stream), the counterpart of the reference drivers' -DTIMERON phase timers
 * (sirt_main.cc:174-223). tg_plan_set_timing(plan, 1) clears and starts;
 * tg_plan_get_timing synchronizes the stream and returns the sums. */
int tg_plan_set_timing(tg_plan* plan, int enable);
int tg_plan_get_timing(tg_plan* plan, tg_timing* out);

/* In-place degrees -> radians with the reference's float constant. Host. */
int tg_degree_to_radian(float* theta, int n);

/* Page-locked host memory for sinograms and reconstructions (so that the
 * transfers read and write it in place; see the conventions above), for
 * hosts that do not call the CUDA runtime themselves. tg_host_alloc stores
 * the address in *out (NULL for bytes == 0) or returns TG_E_NOMEM;
 * tg_host_free(NULL) does nothing. No plan is involved: tg_last_error(NULL)
 * holds the message of a failure. */
int tg_host_alloc(size_t bytes, void** out);
int tg_host_free(void* ptr);

/* Sinogram in the reference layout [P][S][C] float32. `on_device` != 0 means
 * `sino` is a device pointer. apply_abs != 0 applies |x| (trace_utils::Absolute)
 * during the upload. */
int tg_set_sinogram(tg_plan* plan, const float* sino, int on_device,
                    int apply_abs);

/* tg_set_sinogram, then every value below clip_min (after |x| when
 * apply_abs) is raised to clip_min; NaN stays NaN. No counterpart in the
 * reference, whose MLEM driver divides by whatever the sinogram holds
 * (mlem.cc:50-52): a floor such as 1e-6 keeps the ratio step's factors
 * positive for noisy, log-converted data with zero-count rays. */
int tg_set_sinogram_clip(tg_plan* plan, const float* sino, int on_device,
                         int apply_abs, float clip_min);

/* Reconstruction in the reference layout: (S + 2*halo) x C x C float32 where
 * halo = 1 for APMLR (TraceMetadata with num_neighbor_recon_slices = 1) and 0
 * otherwise. tg_reset_recon fills it with the algorithm's initial value
 * (0 for SIRT, 1 otherwise; trace_data.h:91-94 with the drivers' init). */
int tg_reset_recon(tg_plan* plan, int alg);
int tg_set_recon(tg_plan* plan, int alg, const float* recon, int on_device);
int tg_get_recon(tg_plan* plan, int alg, float* recon, int on_device);

/* Operator-level surface (one call per reference engine step). */
int tg_reduce(tg_plan* plan, int alg, const tg_params* params);
int tg_get_replica(tg_plan* plan, int alg, float* replica /* S x 2*C*C */,
                   int on_device);
int tg_calculate_fg(tg_plan* plan, int alg, const tg_params* params);
int tg_get_fg(tg_plan* plan, float* F, float* G /* S x C x C each */,
              int on_device);
int tg_update_recon(tg_plan* plan, int alg, const tg_params* params);
int tg_reset_replica(tg_plan* plan);

/* Fused iterations: forward projection + backprojection + (penalty) update
 * per slice batch, n_iter times. */
int tg_iterate(tg_plan* plan, int alg, const tg_params* params, int n_iter);

/* tg_iterate, then tg_get_recon into `recon`, the same bits: the
 * reconstruction of a whole run (the drivers' loop, then WriteRecon). For a
 * device or mapped host buffer, an FP32 plan without halo slices (not
 * APMLR) and no per-kernel timers, the last iteration's slice batches are
 * written out as each one finishes, on a stream of the plan's own, while
 * the following batches still compute; otherwise the two calls run one
 * after the other. No counterpart in the reference. */
int tg_iterate_get_recon(tg_plan* plan, int alg, const tg_params* params, int n_iter,
                         float* recon, int on_device);

/* Capture each fused iteration of tg_iterate in a CUDA graph (one per
 * reconstruction-buffer parity, re-captured when the algorithm or its
 * parameters change) and replay it. Needs the plan's own stream or a
 * user stream other than the legacy default stream; ignored while the
 * per-kernel timers are on. */
int tg_plan_set_graphs(tg_plan* plan, int enable);

/* A batch of independent plans (any geometries and slice counts) iterated
 * together - the counterpart of running many drivers (or MPI ranks over
 * disjoint slice blocks, trace_h5io.cc:7-22) side by side. Plans must be
 * ready to iterate (layout, sinogram) and stay owned by the caller.
 * When every plan is fast mode with forward_tiles, the L1 backprojection
 * and TG_LEN_U16 lengths, one iteration of all plans is, per round of slice
 * batches, one launch of each kernel variant (tile-staged forward, finish,
 * fused backprojection + update; variants by slices per pass, gather
 * precision, penalty, summation) whose blocks walk a work list spanning
 * every plan's tiles and rays; otherwise each plan's own launches are
 * branches of one graph over up to 16 streams. Either way each iteration
 * replays a captured CUDA graph, and results equal tg_iterate's bit for
 * bit. tg_batch_iterate returns after the work has finished. */
typedef struct tg_batch tg_batch;
int tg_batch_create(tg_plan* const* plans, int n, tg_batch** out);
int tg_batch_iterate(tg_batch* batch, const int* algs, const tg_params* params,
                     int n_iter);
int tg_batch_synchronize(tg_batch* batch);
int tg_batch_destroy(tg_batch* batch);
const char* tg_batch_last_error(const tg_batch* batch);
/* *multi: 1 when iterations use the multi-plan launches above;
 * *launches: kernel launches per iteration of the last tg_batch_iterate
 * (0 before the first). Either pointer may be NULL. */
int tg_batch_get_info(const tg_batch* batch, int* multi, int* launches);

/* Forward projection of the current reconstruction: sim [P][S][C]. */
int tg_forward_project(tg_plan* plan, int alg, const tg_params* params,
                       float* sim, int on_device);

/* Traced segment lists in the reference's order, ray r = p*C + c.
 * counts: P*C ints. With idx == NULL only counts are written; otherwise
 * offsets (P*C+1, exclusive scan of counts) must be given and idx/len
 * (and len2, nullable) receive the segments. Host buffers. */
int tg_trace_rays(tg_plan* plan, int32_t* counts, const int64_t* offsets,
                  int32_t* idx, float* len, float* len2);

/* One slice's reduction (forward projection + backprojection) into caller
 * buffers, allocating no device memory. No counterpart in the reference: it
 * exists for callers that must not allocate on the GPU while they run -
 * hosts that hand the library a fixed memory budget up front and treat any
 * later allocation as a failure, or latency-sensitive pipelines where a
 * cudaMalloc/cudaFree (which may synchronize the device) would stall work on
 * their other streams. The plan itself is created beforehand, as usual.
 *
 *   recon: device, C x C floats - the reconstruction the forward projection
 *          reads (for APMLR's reference behaviour, slice s-1).
 *   sino:  device, P x C floats - this slice's sinogram rows, used as they
 *          are: the caller applies |x| where the driver applies it
 *          (trace_utils::Absolute) and any floor it wants (what
 *          tg_set_sinogram_clip applies on upload is not applied here).
 *   num:   device, C x C floats - receives replica[2p] for every pixel, the
 *          values tg_get_replica returns at even positions.
 * The per-ray factors between the two passes live in one file-scope device
 * array of 4,194,304 floats (16 MiB, held by every GPU that loads the
 * library until the process exits); plans with P*C above that return
 * TG_E_LIMIT. tg_plan_create looks the array's device address up
 * (cudaGetSymbolAddress, in the plan's context) and keeps it in the plan, so
 * calls look nothing up and the address is valid for the plan's lifetime.
 * Every call shares the array: calls whose work overlaps on the GPU
 * (different streams, or different plans on one device) race on it; the
 * array needs no clearing, since each call writes every factor it reads.
 * The forward projection is always the ray-ordered one (or the on-the-fly
 * tracer when the plan keeps no ray-ordered matrix) and the backprojection
 * the L1 one with FP32 factors, whatever the plan's forward_tiles /
 * backward_staged / half_gathers options, so on such plans the numerators
 * agree with tg_reduce's to the rounding of those options' operands.
 * Work is issued on the plan's stream; the device that was current when the
 * plan was created must be current. */
int tg_reduce_slice_noalloc(tg_plan* plan, int alg, const tg_params* params,
                            const float* recon, const float* sino, float* num);

#ifdef __cplusplus
}
#endif
#endif /* TRACE_GB300_H */
