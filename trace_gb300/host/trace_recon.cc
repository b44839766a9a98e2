// Reconstruction driver on the C++ drop-in classes (trace_gb300.hpp).
//
// The iteration loop is the reference drivers' loop - src/sirt/sirt_main.cc:
// 177-202 (SIRT, MLEM), src/pml/pml_main.cc:178-193 (PML) and
// src/apmlr/apmlr_main.cc:209-244 (APMLR) - with the reference types swapped
// for their GPU counterparts. Inputs are raw little-endian float32 files
// (the reference reads HDF5, which this build does not link):
//
//   trace_recon -r pml -f sino.f32 -t theta.f32 -o recon.f32 -P 180 -S 8 -C 256
//               [-i iters] [-c center] [-j beta] [-k beta1] [-l delta]
//               [-m delta1] [-w regw] [--degrees] [--fused]
//               [--len u16|f16|bf16|f32] [--slices-per-pass K] [--fast]
//               [--delta-index] [--apmlr-fixed-offset] [--tiles] [--half]
//               [--compensated]
//               [--on-the-fly]
//
// sino is [P][S][C] (the /exchange/data order), theta holds P angles in
// radians (--degrees converts with the reference's DegreeToRadian). The
// output is the reconstruction [S(+2 halo for APMLR)][C][C].
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

#include "trace_gb300.hpp"

using namespace trace_gb300;

namespace {

struct Config {
  std::string alg = "sirt", sino, theta, out;
  int P = 0, S = 0, C = 0, iters = 10, spp = 1;
  float center = 0.f, beta = 10.f, beta1 = 1.f, delta = 1.f, delta1 = 1.f,
        regw = 1.f;
  bool degrees = false, fused = false, fast = false, delta_index = false,
       fixed = false, tiles = false, half = false, otf = false, comp = false;
  int len = TG_LEN_F32;
};

std::vector<float> read_f32(const std::string& path, size_t n) {
  std::vector<float> v(n);
  std::ifstream f(path, std::ios::binary);
  if (!f) throw std::runtime_error("cannot open " + path);
  f.read(reinterpret_cast<char*>(v.data()), n * sizeof(float));
  if ((size_t)f.gcount() != n * sizeof(float))
    throw std::runtime_error(path + ": expected " + std::to_string(n) + " floats");
  return v;
}

Config parse(int argc, char** argv) {
  Config c;
  for (int i = 1; i < argc; ++i) {
    std::string a = argv[i];
    auto next = [&]() -> std::string {
      if (i + 1 >= argc) throw std::runtime_error("missing value for " + a);
      return argv[++i];
    };
    if (a == "-r") c.alg = next();
    else if (a == "-f") c.sino = next();
    else if (a == "-t") c.theta = next();
    else if (a == "-o") c.out = next();
    else if (a == "-P") c.P = std::stoi(next());
    else if (a == "-S") c.S = std::stoi(next());
    else if (a == "-C") c.C = std::stoi(next());
    else if (a == "-i") c.iters = std::stoi(next());
    else if (a == "-c") c.center = std::stof(next());
    else if (a == "-j") c.beta = std::stof(next());
    else if (a == "-k") c.beta1 = std::stof(next());
    else if (a == "-l") c.delta = std::stof(next());
    else if (a == "-m") c.delta1 = std::stof(next());
    else if (a == "-w") c.regw = std::stof(next());
    else if (a == "--degrees") c.degrees = true;
    else if (a == "--fused") c.fused = true;
    else if (a == "--fast") c.fast = true;
    else if (a == "--delta-index") c.delta_index = true;
    else if (a == "--apmlr-fixed-offset") c.fixed = true;
    else if (a == "--tiles") c.tiles = true;
    else if (a == "--half") c.half = true;
    else if (a == "--on-the-fly") c.otf = true;
    else if (a == "--compensated") c.comp = true;
    else if (a == "--slices-per-pass") c.spp = std::stoi(next());
    else if (a == "--len") {
      const std::string v = next();
      c.len = v == "u16" ? TG_LEN_U16 : v == "f16" ? TG_LEN_F16
            : v == "bf16" ? TG_LEN_BF16 : TG_LEN_F32;
    } else {
      throw std::runtime_error("unknown flag " + a);
    }
  }
  if (c.sino.empty() || c.theta.empty() || c.out.empty() || c.P < 1 ||
      c.S < 1 || c.C < 2)
    throw std::runtime_error("need -f -t -o -P -S -C");
  return c;
}

template <class Space>
void run(const Config& cfg, int alg, std::vector<float>& theta,
         std::vector<float>& sino) {
  const bool pen = alg == TG_PML || alg == TG_APMLR;
  Options opt;
  opt.len_storage = cfg.len;
  opt.slices_per_pass = cfg.spp;
  opt.mode = cfg.fast ? TG_MODE_FAST : TG_MODE_EXACT;
  opt.delta_index = cfg.delta_index;
  opt.apmlr_fixed_offset = cfg.fixed;
  opt.forward_tiles = cfg.tiles;
  opt.half_gathers = cfg.half;
  opt.forward_on_the_fly = cfg.otf;
  opt.compensated = cfg.comp;
  // MLEM/PML/APMLR drivers apply Absolute and start from 1 (mlem_main.cc:115,
  // 134); APMLR keeps one neighbour slice on each side (apmlr_main.cc:170).
  GpuTraceMetadata trace_metadata(theta.data(), 0, 0, 0, cfg.S, cfg.P, cfg.S,
                                  cfg.C, cfg.C, cfg.center,
                                  alg == TG_APMLR ? 1 : 0,
                                  alg == TG_SIRT ? 0.f : 1.f, opt);
  GpuDataRegion slices(sino.data(), sino.size(), &trace_metadata, alg != TG_SIRT);
  auto main_recon_space = new Space(cfg.S, 2 * cfg.C * cfg.C);
  main_recon_space->Initialize(trace_metadata.num_grids());
  main_recon_space->Bind(trace_metadata);
  auto main_recon_replica = main_recon_space->reduction_objects();
  float init_val = 0.;
  GpuDISPEngine<Space> engine(main_recon_space);
  const auto t0 = std::chrono::steady_clock::now();
  if (cfg.fused) {
    tg_params prm{cfg.beta, cfg.beta1, cfg.delta, cfg.delta1, cfg.regw};
    check(tg_iterate(trace_metadata.plan(), alg, &prm, cfg.iters),
          trace_metadata.plan());
  } else {
    for (int i = 0; i < cfg.iters; ++i) {
      engine.RunParallelReduction(slices, cfg.C);  /// Reconstruction
      engine.ParInPlaceLocalSynchWrapper();        /// Local combination
      if (pen) {
        slices.SetFG(0.);
        if (alg == TG_PML)
          main_recon_space->CalculateFG(slices, cfg.beta);
        else
          main_recon_space->CalculateFG(slices, cfg.beta, cfg.beta1, cfg.delta,
                                        cfg.delta1, cfg.regw);
        main_recon_space->UpdateRecon(slices, main_recon_replica);
      } else {
        main_recon_space->UpdateRecon(trace_metadata, main_recon_replica);
      }
      engine.ResetReductionSpaces(init_val);
      slices.ResetMirroredRegionIter();
    }
  }
  const std::vector<float> recon = trace_metadata.recon(alg);
  const double secs = std::chrono::duration<double>(
                          std::chrono::steady_clock::now() - t0).count();
  std::ofstream f(cfg.out, std::ios::binary);
  f.write(reinterpret_cast<const char*>(recon.data()), recon.size() * sizeof(float));
  std::cout << "Reconstruction time=" << secs << " s, slice-iter/s="
            << cfg.S * cfg.iters / secs << std::endl;
  delete main_recon_space;
}

}  // namespace

int main(int argc, char** argv) {
  try {
    Config cfg = parse(argc, argv);
    std::vector<float> theta = read_f32(cfg.theta, cfg.P);
    std::vector<float> sino = read_f32(cfg.sino, (size_t)cfg.P * cfg.S * cfg.C);
    if (cfg.degrees) check(tg_degree_to_radian(theta.data(), cfg.P), nullptr);
    if (cfg.alg == "sirt") run<GpuSIRTReconSpace>(cfg, TG_SIRT, theta, sino);
    else if (cfg.alg == "mlem") run<GpuMLEMReconSpace>(cfg, TG_MLEM, theta, sino);
    else if (cfg.alg == "pml") run<GpuPMLReconSpace>(cfg, TG_PML, theta, sino);
    else if (cfg.alg == "apmlr") run<GpuAPMLRReconSpace>(cfg, TG_APMLR, theta, sino);
    else throw std::runtime_error("unknown algorithm " + cfg.alg);
  } catch (const std::exception& e) {
    std::cerr << e.what() << std::endl;
    return 1;
  }
  return 0;
}
