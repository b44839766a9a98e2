// C++ drop-in for the reference's operator surface on top of the C ABI.
//
// The classes mirror the reference types a driver touches, with the same
// constructor arguments and member calls, so a driver's iteration loop
// (e.g. src/sirt/sirt_main.cc:177-202, src/pml/pml_main.cc:178-193,
// src/apmlr/apmlr_main.cc:209-244) compiles against them unchanged apart
// from the type names:
//
//   reference                                   here
//   TraceMetadata        (trace_data.h:25-192)  trace_gb300::GpuTraceMetadata
//   DataRegionBase<float, TraceMetadata>,
//   PMLDataRegion / APMLRDataRegion (pml.h:16-61, apmlr.h:16-53)
//                                               trace_gb300::GpuDataRegion
//   SIRT/MLEM/PML/APMLRReconSpace (sirt.h:16-71 ...)
//                                               trace_gb300::Gpu*ReconSpace
//   DISPEngineReduction<RST, float> (disp_engine_reduction.h:147-350)
//                                               trace_gb300::GpuDISPEngine<RST>
//
// Like the reference, failures throw (std::runtime_error with the library's
// message). Header-only; link libtrace_gb300.so.
#pragma once
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#include "../../include/trace_gb300.h"

namespace trace_gb300 {

inline void check(int rc, const tg_plan* plan) {
  if (rc != TG_OK)
    throw std::runtime_error(std::string("trace_gb300: ") + tg_last_error(plan));
}

// How the plan stores and streams the system matrix (not part of the
// reference, which re-traces every ray each iteration).
struct Options {
  int len_storage = TG_LEN_F32;
  int slices_per_pass = 1;
  int mode = TG_MODE_EXACT;
  int delta_index = 0;
  int apmlr_fixed_offset = 0;
  int forward_tiles = 0;    // fast mode: tile-staged forward projection
  int backward_staged = 0;  // fast mode: shared-memory detector windows
  int half_gathers = 0;     // fast mode + forward_tiles: 16-bit gather operands
  int forward_on_the_fly = 0;  // trace rays during the forward projection
  int compensated = 0;      // fast mode + forward_tiles: Kahan ray/pixel sums
  int backward_tile_width = 0;  // 8 (default), 16 or 4 pixels per tile row
  int forward_tile_side = 0;    // 64 (default); 32 to 96 in steps of 16
  int batch_streams = 0;        // 2 (default): odd slice batches on a 2nd stream
  int forward_block_warps = 0;  // 32 (default), 16 or 8 warps per forward tile
};

// Geometry + reconstruction (TraceMetadata). theta is copied, not owned.
class GpuTraceMetadata {
 public:
  GpuTraceMetadata(const float* theta, int proj_id, int slice_id, int col_id,
                   int num_total_slices, int num_projs, int num_slices,
                   int num_cols, int num_grids, float center,
                   int num_neighbor_recon_slices, float recon_init_val,
                   Options opt = Options())
      : proj_id_(proj_id), slice_id_(slice_id), col_id_(col_id),
        num_total_slices_(num_total_slices), num_projs_(num_projs),
        num_slices_(num_slices), num_cols_(num_cols), num_grids_(num_grids),
        halo_(num_neighbor_recon_slices), recon_init_(recon_init_val) {
    if (theta == nullptr) throw std::invalid_argument("theta ptr is null");
    if (num_grids != num_cols)
      throw std::invalid_argument("the grid size equals the column count");
    if (halo_ != 0 && halo_ != 1)
      throw std::invalid_argument("num_neighbor_recon_slices must be 0 or 1");
    tg_plan_desc d{};
    d.num_projs = num_projs;
    d.num_slices = num_slices;
    d.num_cols = num_cols;
    d.center = center;
    d.slice_id = slice_id;
    d.num_total_slices = num_total_slices;
    d.len_storage = opt.len_storage;
    d.slices_per_pass = opt.slices_per_pass;
    d.mode = opt.mode;
    d.delta_index = opt.delta_index;
    d.apmlr_fixed_offset = opt.apmlr_fixed_offset;
    d.forward_tiles = opt.forward_tiles;
    d.backward_staged = opt.backward_staged;
    d.half_gathers = opt.half_gathers;
    d.forward_on_the_fly = opt.forward_on_the_fly;
    d.compensated = opt.compensated;
    d.backward_tile_width = opt.backward_tile_width;
    d.forward_tile_side = opt.forward_tile_side;
    d.batch_streams = opt.batch_streams;
    d.forward_block_warps = opt.forward_block_warps;
    tg_plan* p = nullptr;
    check(tg_plan_create(&d, theta, nullptr, nullptr, &p), nullptr);
    plan_.reset(p);
    center_ = (center <= 0.) ? static_cast<float>(num_cols) / 2. + 1. : center;
  }

  tg_plan* plan() const { return plan_.get(); }
  int slice_id() const { return slice_id_; }
  int proj_id() const { return proj_id_; }
  int col_id() const { return col_id_; }
  int num_total_slices() const { return num_total_slices_; }
  int num_projs() const { return num_projs_; }
  int num_slices() const { return num_slices_; }
  int num_cols() const { return num_cols_; }
  int num_grids() const { return num_grids_; }
  float center() const { return center_; }
  size_t count() const { return (size_t)num_projs_ * num_slices_ * num_cols_; }
  int num_neighbor_recon_slices() const { return halo_; }
  float recon_init_val() const { return recon_init_; }

  // The reconstruction, (num_slices + 2*halo) x grid x grid, on the host.
  std::vector<float> recon(int alg) const {
    std::vector<float> out(recon_count());
    check(tg_get_recon(plan_.get(), alg, out.data(), 0), plan_.get());
    return out;
  }
  // Into a caller's host buffer of recon_count() floats (page-locked memory,
  // e.g. from tg_host_alloc, is written in place).
  void recon_into(int alg, float* out) const {
    check(tg_get_recon(plan_.get(), alg, out, 0), plan_.get());
  }
  size_t recon_count() const {
    return (size_t)(num_slices_ + 2 * halo_) * num_grids_ * num_grids_;
  }

 private:
  struct Del {
    void operator()(tg_plan* p) const { tg_plan_destroy(p); }
  };
  std::unique_ptr<tg_plan, Del> plan_;
  int proj_id_, slice_id_, col_id_, num_total_slices_, num_projs_,
      num_slices_, num_cols_, num_grids_, halo_;
  float recon_init_, center_ = 0.f;
};

// The sinogram as the reduction input (DataRegionBase / PMLDataRegion /
// APMLRDataRegion): uploads [P][S][C] floats. F and G live on the device.
class GpuDataRegion {
 public:
  GpuDataRegion(const float* data, size_t count, GpuTraceMetadata* md,
                bool apply_abs = false)
      : md_(md) {
    if (!md) throw std::invalid_argument("metadata is null");
    if (count != md->count()) throw std::out_of_range("sinogram size mismatch");
    check(tg_set_sinogram(md->plan(), data, 0, apply_abs ? 1 : 0), md->plan());
  }
  GpuTraceMetadata& metadata() const { return *md_; }
  void SetFG(float) {}                 // F and G are recomputed by CalculateFG
  void ResetMirroredRegionIter() {}    // work is not handed out in chunks

 private:
  GpuTraceMetadata* md_;
};

// The combined replica, downloaded on demand (reduction_objects()).
class GpuReplica {
 public:
  GpuReplica(tg_plan* plan, int alg, int rows, int cols)
      : plan_(plan), alg_(alg), rows_(rows), cols_(cols) {}
  size_t rows() const { return rows_; }
  size_t cols() const { return cols_; }
  std::vector<float> download() const {
    std::vector<float> out((size_t)rows_ * cols_);
    check(tg_get_replica(plan_, alg_, out.data(), 0), plan_);
    return out;
  }

 private:
  tg_plan* plan_;
  int alg_, rows_, cols_;
};

// XReconSpace: Initialize / UpdateRecon / CalculateFG / reduction_objects.
template <int ALG>
class GpuReconSpace {
 public:
  GpuReconSpace(int rows, int cols) : rows_(rows), cols_(cols) {}
  void Initialize(int n_grids) { n_grids_ = n_grids; }
  void Bind(GpuTraceMetadata& md) {
    md_ = &md;
    check(tg_reset_recon(md.plan(), ALG), md.plan());
  }
  GpuReplica reduction_objects() {
    return GpuReplica(md_->plan(), ALG, rows_, cols_);
  }
  // SIRT / MLEM form (sirt.cc:21-33, mlem.cc:21-34)
  void UpdateRecon(GpuTraceMetadata&, const GpuReplica&) { update(); }
  // PML / APMLR form (pml.cc:3-23, apmlr.cc:3-26)
  void UpdateRecon(GpuDataRegion&, const GpuReplica&) { update(); }
  void CalculateFG(GpuDataRegion& slices, float beta) {
    CalculateFG(slices, beta, 1.f, 1.f, 1.f, 1.f);
  }
  void CalculateFG(GpuDataRegion& slices, float beta, float beta1, float delta,
                   float delta1, float regw) {
    prm_ = tg_params{beta, beta1, delta, delta1, regw};
    check(tg_calculate_fg(slices.metadata().plan(), ALG, &prm_),
          slices.metadata().plan());
  }
  GpuTraceMetadata* metadata() const { return md_; }
  const tg_params& params() const { return prm_; }

 private:
  void update() { check(tg_update_recon(md_->plan(), ALG, &prm_), md_->plan()); }
  int rows_, cols_, n_grids_ = 0;
  GpuTraceMetadata* md_ = nullptr;
  tg_params prm_{10.f, 1.f, 1.f, 1.f, 1.f};
};

using GpuSIRTReconSpace = GpuReconSpace<TG_SIRT>;
using GpuMLEMReconSpace = GpuReconSpace<TG_MLEM>;
using GpuPMLReconSpace = GpuReconSpace<TG_PML>;
using GpuAPMLRReconSpace = GpuReconSpace<TG_APMLR>;

// DISPEngineReduction: the reduction runs on the device into one replica,
// so the local combination is a no-op and the thread count is ignored.
template <class RS>
class GpuDISPEngine {
 public:
  template <class Comm>
  GpuDISPEngine(Comm*, RS* space, int /*num_reduction_threads*/)
      : space_(space) {}
  GpuDISPEngine(RS* space) : space_(space) {}
  void RunParallelReduction(GpuDataRegion& input, int /*req_units*/) {
    tg_plan* p = input.metadata().plan();
    check(tg_reduce(p, alg_of(), &space_->params()), p);
  }
  void SeqInPlaceLocalSynchWrapper() {}
  void ParInPlaceLocalSynchWrapper() {}
  void DistInPlaceGlobalSynchWrapper() {}
  void ResetReductionSpaces(float) {
    if (space_->metadata()) {
      tg_plan* p = space_->metadata()->plan();
      check(tg_reset_replica(p), p);
    }
  }

 private:
  static constexpr int alg_of() {
    return std::is_same<RS, GpuSIRTReconSpace>::value   ? TG_SIRT
           : std::is_same<RS, GpuMLEMReconSpace>::value ? TG_MLEM
           : std::is_same<RS, GpuPMLReconSpace>::value  ? TG_PML
                                                        : TG_APMLR;
  }
  RS* space_;
};

}  // namespace trace_gb300
