// Test infrastructure only: a C-callable harness around the reference's OWN
// tracer, operators and DISP engine (compiled unmodified from the reference
// tree by oracle/Makefile into oracle/_ref/). It is the checker the oracle
// restatement and the golden fixtures are pinned against; nothing in the
// product links it.
//
// The harness replays the drivers' call sequence:
//   - tracing: the per-ray call chain of SIRTReconSpace::Reduce
//     (src/sirt/sirt.cc:117-160): CalculateQuadrant, sinf/cosf,
//     CalculateCoordinates, MergeTrimCoordinates, SortIntersectionPoints,
//     CalculateDistanceLengths (the leng2 overload, src/common/trace_utils.cc:160-187);
//   - reconstruction: the iteration loop of src/sirt/sirt_main.cc:177-202,
//     src/mlem/mlem_main.cc (same loop), src/pml/pml_main.cc:178-193 and
//     src/apmlr/apmlr_main.cc:209-244, with a size-1 communicator standing in
//     for DISPCommMPI (the halo exchange returns early at size 1,
//     src/common/trace_comm.cc:23).
//
// Compile once per algorithm with -DREF_ALG_SIRT / _MLEM / _PML / _APMLR
// (mlem.h and apmlr.h share one include guard, so they cannot share a TU),
// and once with -DREF_TRACE for the tracer entry points.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include "disp_comm_base.h"
#include "disp_engine_reduction.h"
#include "data_region_base.h"
#include "trace_data.h"
#include "trace_utils.h"

namespace {
class SizeOneComm : public DISPCommBase<float> {
 public:
  SizeOneComm() { rank_ = 0; size_ = 1; }
  void GlobalInPlaceCombination(DataRegion2DBareBase<float>&) override {}
};

float* copy_new(const float* src, size_t n) {
  float* p = new float[n];
  std::memcpy(p, src, n * sizeof(float));
  return p;
}
}  // namespace

#if defined(REF_TRACE)
// Per-ray segment lists of the reference tracer. Two-call protocol:
// with idx == nullptr only counts[r] = max(len-1, 0) are written; otherwise
// the caller passes offsets (exclusive scan of counts) and buffers sized to
// the total, and gets pixel indices, lengths and squared lengths. sin_out /
// cos_out / quad_out (nullable) receive the per-angle values the tracer used.
extern "C" int ref_trace(int num_cols, int num_projs, const float* theta,
                         float center, int32_t* counts, const int64_t* offsets,
                         int32_t* idx, float* len, float* len2,
                         float* sin_out, float* cos_out, int32_t* quad_out) {
  const int g = num_cols;
  TraceMetadata md(copy_new(theta, num_projs), 0, 0, 0, 1, num_projs, 1,
                   num_cols, num_cols, center, 0, 0.f);
  const float* gridx = md.gridx();
  const float* gridy = md.gridy();
  const float mov = md.mov();
  std::vector<float> coordx(g + 1), coordy(g + 1), ax(g + 1), ay(g + 1),
      bx(g + 1), by(g + 1), coorx(2 * g + 2), coory(2 * g + 2),
      lg(2 * g + 2), lg2(2 * g + 2);
  std::vector<int> ind(2 * g + 2);
  for (int p = 0; p < num_projs; ++p) {
    float theta_q = theta[p];
    int quadrant = trace_utils::CalculateQuadrant(theta_q);
    float sinq = sinf(theta_q);
    float cosq = cosf(theta_q);
    if (sin_out) sin_out[p] = sinq;
    if (cos_out) cos_out[p] = cosq;
    if (quad_out) quad_out[p] = quadrant;
    for (int c = 0; c < num_cols; ++c) {
      float xi = -1e6;
      float yi = (1 - num_cols) / 2. + c + mov;
      trace_utils::CalculateCoordinates(g, xi, yi, sinq, cosq, gridx, gridy,
                                        coordx.data(), coordy.data());
      int alen, blen;
      trace_utils::MergeTrimCoordinates(g, coordx.data(), coordy.data(), gridx,
                                        gridy, &alen, &blen, ax.data(),
                                        ay.data(), bx.data(), by.data());
      trace_utils::SortIntersectionPoints(quadrant, alen, blen, ax.data(),
                                          ay.data(), bx.data(), by.data(),
                                          coorx.data(), coory.data());
      int n = alen + blen;
      trace_utils::CalculateDistanceLengths(n, g, coorx.data(), coory.data(),
                                            lg.data(), lg2.data(), ind.data());
      int nseg = n > 1 ? n - 1 : 0;
      int64_t r = (int64_t)p * num_cols + c;
      if (idx == nullptr) {
        counts[r] = nseg;
        continue;
      }
      int64_t o = offsets[r];
      for (int i = 0; i < nseg; ++i) {
        idx[o + i] = ind[i];
        len[o + i] = lg[i];
        len2[o + i] = lg2[i];
      }
    }
  }
  return 0;
}

// TraceMetadata's derived geometry (mov, grid lines) for a detector width.
extern "C" int ref_geometry(int num_cols, float center, float* mov_out,
                            float* gridx_out) {
  float th = 0.f;
  TraceMetadata md(copy_new(&th, 1), 0, 0, 0, 1, 1, 1, num_cols, num_cols,
                   center, 0, 0.f);
  *mov_out = md.mov();
  for (int i = 0; i <= num_cols; ++i) gridx_out[i] = md.gridx()[i];
  return 0;
}
#else

#if defined(REF_ALG_SIRT)
#include "sirt.h"
typedef SIRTReconSpace Space;
typedef DataRegionBase<float, TraceMetadata> Region;
#define REF_ENTRY ref_run_sirt
#define REF_HALO 0
#define REF_INIT 0.f
#define REF_ABS 0
#elif defined(REF_ALG_MLEM)
#include "mlem.h"
typedef MLEMReconSpace Space;
typedef DataRegionBase<float, TraceMetadata> Region;
#define REF_ENTRY ref_run_mlem
#define REF_HALO 0
#define REF_INIT 1.f
#define REF_ABS 1
#elif defined(REF_ALG_PML)
#include "pml.h"
typedef PMLReconSpace Space;
typedef PMLDataRegion Region;
#define REF_ENTRY ref_run_pml
#define REF_HALO 0
#define REF_INIT 1.f
#define REF_ABS 1
#elif defined(REF_ALG_APMLR)
#include "apmlr.h"
typedef APMLRReconSpace Space;
typedef APMLRDataRegion Region;
#define REF_ENTRY ref_run_apmlr
#define REF_HALO 1
#define REF_INIT 1.f
#define REF_ABS 1
#else
#error "define one of REF_TRACE, REF_ALG_SIRT, REF_ALG_MLEM, REF_ALG_PML, REF_ALG_APMLR"
#endif

// One reconstruction run through the reference's engine.
//   sino: [P][S][C] float32, as the drivers hold it after ReadSlices.
//   params: {beta, beta1, delta, delta1, regw} (PML reads beta only).
//   recon_out: (S + 2*halo) * C * C floats (halo = 1 for APMLR, else 0).
//   iters_out (nullable): n_iter snapshots of the same size.
//   replica_out (nullable): S * 2*C*C floats, the combined reduction
//     objects of the LAST iteration, taken before UpdateRecon.
//   apply_abs: apply trace_utils::Absolute to the sinogram first, as the
//     MLEM/PML/APMLR drivers do (-1 = the driver's own choice).
extern "C" int REF_ENTRY(int num_projs, int num_slices, int num_cols,
                         const float* theta, const float* sino, float center,
                         int n_iter, int threads, const float* params,
                         int slice_id, int num_total_slices, int apply_abs,
                         float* recon_out, float* iters_out,
                         float* replica_out) {
  const int g = num_cols;
  const size_t count = (size_t)num_projs * num_slices * num_cols;
  TraceMetadata md(copy_new(theta, num_projs), 0, slice_id, 0,
                   num_total_slices, num_projs, num_slices, num_cols, num_cols,
                   center, REF_HALO, REF_INIT);
  float* data = copy_new(sino, count);
  if (apply_abs < 0 ? REF_ABS : apply_abs) trace_utils::Absolute(data, count);
  Region* slices = new Region(data, count, &md);
  Space* space = new Space(num_slices, 2 * g * g);
  space->Initialize(g);
  auto& replica = space->reduction_objects();
  float init_val = 0.;
  replica.ResetAllItems(init_val);
  SizeOneComm comm;
  DISPEngineBase<Space, float>* engine =
      new DISPEngineReduction<Space, float>(&comm, space, threads);
  const size_t recon_count = (size_t)(num_slices + 2 * REF_HALO) * g * g;
  for (int it = 0; it < n_iter; ++it) {
    engine->RunParallelReduction(*slices, num_cols);
    engine->ParInPlaceLocalSynchWrapper();
    if (replica_out && it == n_iter - 1) {
      for (int s = 0; s < num_slices; ++s)
        std::memcpy(replica_out + (size_t)s * 2 * g * g, &replica[s][0],
                    sizeof(float) * 2 * g * g);
    }
#if defined(REF_ALG_SIRT) || defined(REF_ALG_MLEM)
    space->UpdateRecon(md.recon(), replica);
#elif defined(REF_ALG_PML)
    slices->SetFG(0.);
    space->CalculateFG(*slices, params[0]);
    space->UpdateRecon(*slices, replica);
#else
    slices->SetFG(0.);
    space->CalculateFG(*slices, params[0], params[1], params[2], params[3],
                       params[4]);
    space->UpdateRecon(*slices, replica);
#endif
    engine->ResetReductionSpaces(init_val);
    slices->ResetMirroredRegionIter();
    if (iters_out)
      std::memcpy(iters_out + (size_t)it * recon_count, &md.recon()[0],
                  sizeof(float) * recon_count);
  }
  std::memcpy(recon_out, &md.recon()[0], sizeof(float) * recon_count);
  delete slices;  // owns and frees `data`
  delete engine;  // owns and frees `space` and its clones
  return 0;
}
#endif
