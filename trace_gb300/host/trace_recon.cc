// Reconstruction driver on the C++ drop-in classes (trace_gb300.hpp).
//
// The iteration loop is the reference drivers' loop - src/sirt/sirt_main.cc:
// 177-202 (SIRT, MLEM), src/pml/pml_main.cc:178-193 (PML) and
// src/apmlr/apmlr_main.cc:209-244 (APMLR) - with the reference types swapped
// for their GPU counterparts. The reference reads HDF5 (/exchange/data,
// /exchange/theta) and writes /data, which this build does not link; files
// here are NumPy .npy (little-endian float32, C order; the shapes then come
// from the files) or raw little-endian float32 (shapes from -P -S -C):
//
//   trace_recon -r pml -f sino.npy -t theta.npy -o recon.npy
//   trace_recon -r pml -f sino.f32 -t theta.f32 -o recon.f32 -P 180 -S 8 -C 256
//               [-i iters] [-c center] [-j beta] [-k beta1] [-l delta]
//               [-m delta1] [-w regw] [--degrees] [--fused]
//               [--len u16|f16|bf16|f32] [--slices-per-pass K] [--fast]
//               [--delta-index] [--apmlr-fixed-offset] [--tiles] [--half]
//               [--compensated] [--on-the-fly] [--staged]
//               [--tile-side N] [--backward-tile-width N]
//               [--batch-streams N] [--block-warps N]
//
// sino is [P][S][C] (the /exchange/data order), theta holds P angles in
// radians (--degrees converts with the reference's DegreeToRadian). The
// output is the reconstruction [S(+2 halo for APMLR)][C][C]. The sinogram
// and the reconstruction live in page-locked host memory (tg_host_alloc),
// so the upload and download kernels read and write them in place.
#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <memory>
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
       fixed = false, tiles = false, half = false, otf = false, comp = false,
       staged = false;
  int len = TG_LEN_F32, tile_side = 0, btw = 0, streams = 0, warps = 0;
};

// A float buffer in page-locked host memory, or in ordinary memory when
// page-locked memory cannot be had (the transfers then stage it).
class HostFloats {
 public:
  explicit HostFloats(size_t n) : n_(n) {
    void* p = nullptr;
    if (n && tg_host_alloc(n * sizeof(float), &p) == TG_OK) {
      locked_ = static_cast<float*>(p);
    } else {
      plain_.resize(n);
    }
  }
  ~HostFloats() {
    if (locked_) tg_host_free(locked_);
  }
  HostFloats(const HostFloats&) = delete;
  HostFloats& operator=(const HostFloats&) = delete;
  float* data() { return locked_ ? locked_ : plain_.data(); }
  size_t size() const { return n_; }

 private:
  size_t n_;
  float* locked_ = nullptr;
  std::vector<float> plain_;
};

bool is_npy(const std::string& path) {
  return path.size() > 4 && path.compare(path.size() - 4, 4, ".npy") == 0;
}

// Value text of `key` in a .npy header dictionary (up to the next top-level
// comma; a parenthesised tuple whole).
std::string npy_field(const std::string& h, const std::string& key,
                      const std::string& path) {
  const size_t k = h.find("'" + key + "'");
  if (k == std::string::npos) throw std::runtime_error(path + ": .npy header lacks " + key);
  size_t i = h.find(':', k);
  if (i == std::string::npos) throw std::runtime_error(path + ": bad .npy header");
  ++i;
  while (i < h.size() && h[i] == ' ') ++i;
  if (i < h.size() && h[i] == '(') {
    const size_t e = h.find(')', i);
    if (e == std::string::npos) throw std::runtime_error(path + ": bad .npy shape");
    return h.substr(i, e - i + 1);
  }
  size_t e = i;
  while (e < h.size() && h[e] != ',' && h[e] != '}') ++e;
  return h.substr(i, e - i);
}

// Opens a .npy file of little-endian float32 in C order, positioned at its
// data; returns the shape.
std::vector<int64_t> npy_open(std::ifstream& f, const std::string& path) {
  char magic[6];
  f.read(magic, 6);
  if (!f || std::memcmp(magic, "\x93NUMPY", 6) != 0)
    throw std::runtime_error(path + ": not a .npy file");
  unsigned char ver[2];
  f.read(reinterpret_cast<char*>(ver), 2);
  uint32_t hlen = 0;
  if (ver[0] == 1) {
    unsigned char b[2];
    f.read(reinterpret_cast<char*>(b), 2);
    hlen = b[0] | (uint32_t)b[1] << 8;
  } else if (ver[0] == 2 || ver[0] == 3) {
    unsigned char b[4];
    f.read(reinterpret_cast<char*>(b), 4);
    hlen = b[0] | (uint32_t)b[1] << 8 | (uint32_t)b[2] << 16 | (uint32_t)b[3] << 24;
  } else {
    throw std::runtime_error(path + ": unsupported .npy version");
  }
  if (!f || hlen > (1u << 20)) throw std::runtime_error(path + ": bad .npy header");
  std::string h(hlen, ' ');
  f.read(&h[0], hlen);
  if (!f) throw std::runtime_error(path + ": truncated .npy header");
  std::string descr = npy_field(h, "descr", path);
  if (descr.find("<f4") == std::string::npos && descr.find("|f4") == std::string::npos)
    throw std::runtime_error(path + ": expects little-endian float32 ('<f4'), found " + descr);
  if (npy_field(h, "fortran_order", path).find("False") == std::string::npos)
    throw std::runtime_error(path + ": expects C order (fortran_order False)");
  const std::string t = npy_field(h, "shape", path);
  std::vector<int64_t> shape;
  size_t i = 1;
  while (i < t.size()) {
    while (i < t.size() && (t[i] == ' ' || t[i] == ',')) ++i;
    if (i >= t.size() || t[i] == ')') break;
    size_t used = 0;
    shape.push_back(std::stoll(t.substr(i), &used));
    i += used;
  }
  return shape;
}

void read_into(std::ifstream& f, float* dst, size_t n, const std::string& path) {
  f.read(reinterpret_cast<char*>(dst), (std::streamsize)(n * sizeof(float)));
  if ((size_t)f.gcount() != n * sizeof(float))
    throw std::runtime_error(path + ": expected " + std::to_string(n) + " floats");
}

// A float32 input: `dims` (P, or P S C) checked against - or, where zero,
// taken from - a .npy file's shape; raw files need every dimension given.
std::unique_ptr<HostFloats> read_input(const std::string& path, std::vector<int*> dims) {
  std::ifstream f(path, std::ios::binary);
  if (!f) throw std::runtime_error("cannot open " + path);
  if (is_npy(path)) {
    const std::vector<int64_t> shape = npy_open(f, path);
    if (shape.size() != dims.size())
      throw std::runtime_error(path + ": expects a " + std::to_string(dims.size()) +
                               "-dimensional array");
    for (size_t k = 0; k < dims.size(); ++k) {
      if (shape[k] < 1 || shape[k] > (1 << 30))
        throw std::runtime_error(path + ": bad dimension " + std::to_string(shape[k]));
      if (*dims[k] == 0) *dims[k] = (int)shape[k];
      else if (*dims[k] != shape[k])
        throw std::runtime_error(path + ": shape does not match -P/-S/-C");
    }
  }
  size_t n = 1;
  for (int* d : dims) {
    if (*d < 1) throw std::runtime_error("need -P -S -C for raw input " + path);
    n *= (size_t)*d;
  }
  auto buf = std::make_unique<HostFloats>(n);
  read_into(f, buf->data(), n, path);
  return buf;
}

// Raw float32, or .npy (format 1.0) with the given shape.
void write_output(const std::string& path, const float* data, std::vector<int64_t> shape) {
  std::ofstream f(path, std::ios::binary);
  if (!f) throw std::runtime_error("cannot write " + path);
  size_t n = 1;
  for (int64_t d : shape) n *= (size_t)d;
  if (is_npy(path)) {
    std::string dims;  // "a, b, c", or "a," for one dimension
    for (size_t k = 0; k < shape.size(); ++k)
      dims += (k ? ", " : "") + std::to_string(shape[k]);
    if (shape.size() == 1) dims += ",";
    std::string h = "{'descr': '<f4', 'fortran_order': False, 'shape': (" + dims + "), }";
    // pad so that magic + version + length + header is a multiple of 64
    while ((10 + h.size() + 1) % 64) h += ' ';
    h += '\n';
    const uint16_t hl = (uint16_t)h.size();
    const unsigned char pre[10] = {0x93, 'N', 'U', 'M', 'P', 'Y', 1, 0,
                                   (unsigned char)(hl & 255), (unsigned char)(hl >> 8)};
    f.write(reinterpret_cast<const char*>(pre), 10);
    f.write(h.data(), (std::streamsize)h.size());
  }
  f.write(reinterpret_cast<const char*>(data), (std::streamsize)(n * sizeof(float)));
  if (!f) throw std::runtime_error("writing " + path + " failed");
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
    else if (a == "--staged") c.staged = true;
    else if (a == "--slices-per-pass") c.spp = std::stoi(next());
    else if (a == "--tile-side") c.tile_side = std::stoi(next());
    else if (a == "--backward-tile-width") c.btw = std::stoi(next());
    else if (a == "--batch-streams") c.streams = std::stoi(next());
    else if (a == "--block-warps") c.warps = std::stoi(next());
    else if (a == "--len") {
      const std::string v = next();
      c.len = v == "u16" ? TG_LEN_U16 : v == "f16" ? TG_LEN_F16
            : v == "bf16" ? TG_LEN_BF16 : TG_LEN_F32;
    } else {
      throw std::runtime_error("unknown flag " + a);
    }
  }
  if (c.sino.empty() || c.theta.empty() || c.out.empty())
    throw std::runtime_error("need -f -t -o (and -P -S -C for raw files)");
  return c;
}

template <class Space>
void run(const Config& cfg, int alg, float* theta, const float* sino, size_t sino_n) {
  const bool pen = alg == TG_PML || alg == TG_APMLR;
  Options opt;
  opt.len_storage = cfg.len;
  opt.slices_per_pass = cfg.spp;
  opt.mode = cfg.fast ? TG_MODE_FAST : TG_MODE_EXACT;
  opt.delta_index = cfg.delta_index;
  opt.apmlr_fixed_offset = cfg.fixed;
  opt.forward_tiles = cfg.tiles;
  opt.backward_staged = cfg.staged;
  opt.half_gathers = cfg.half;
  opt.forward_on_the_fly = cfg.otf;
  opt.compensated = cfg.comp;
  opt.forward_tile_side = cfg.tile_side;
  opt.backward_tile_width = cfg.btw;
  opt.batch_streams = cfg.streams;
  opt.forward_block_warps = cfg.warps;
  // MLEM/PML/APMLR drivers apply Absolute and start from 1 (mlem_main.cc:115,
  // 134); APMLR keeps one neighbour slice on each side (apmlr_main.cc:170).
  GpuTraceMetadata trace_metadata(theta, 0, 0, 0, cfg.S, cfg.P, cfg.S,
                                  cfg.C, cfg.C, cfg.center,
                                  alg == TG_APMLR ? 1 : 0,
                                  alg == TG_SIRT ? 0.f : 1.f, opt);
  GpuDataRegion slices(sino, sino_n, &trace_metadata, alg != TG_SIRT);
  auto main_recon_space = new Space(cfg.S, 2 * cfg.C * cfg.C);
  main_recon_space->Initialize(trace_metadata.num_grids());
  main_recon_space->Bind(trace_metadata);
  auto main_recon_replica = main_recon_space->reduction_objects();
  float init_val = 0.;
  GpuDISPEngine<Space> engine(main_recon_space);
  HostFloats recon(trace_metadata.recon_count());
  const auto t0 = std::chrono::steady_clock::now();
  if (cfg.fused) {
    // iterations and download in one call (the last iteration's slice
    // batches leave as each one finishes)
    tg_params prm{cfg.beta, cfg.beta1, cfg.delta, cfg.delta1, cfg.regw};
    check(tg_iterate_get_recon(trace_metadata.plan(), alg, &prm, cfg.iters, recon.data(), 0),
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
    trace_metadata.recon_into(alg, recon.data());
  }
  const double secs = std::chrono::duration<double>(
                          std::chrono::steady_clock::now() - t0).count();
  const int halo = alg == TG_APMLR ? 1 : 0;
  write_output(cfg.out, recon.data(), {cfg.S + 2 * halo, cfg.C, cfg.C});
  std::cout << "Reconstruction time=" << secs << " s, slice-iter/s="
            << cfg.S * cfg.iters / secs << std::endl;
  delete main_recon_space;
}

}  // namespace

int main(int argc, char** argv) {
  try {
    Config cfg = parse(argc, argv);
    // the sinogram first: a .npy sinogram gives P, S and C
    std::unique_ptr<HostFloats> sino = read_input(cfg.sino, {&cfg.P, &cfg.S, &cfg.C});
    std::unique_ptr<HostFloats> theta = read_input(cfg.theta, {&cfg.P});
    if (cfg.C < 2) throw std::runtime_error("need at least 2 detector columns");
    if (cfg.degrees) check(tg_degree_to_radian(theta->data(), cfg.P), nullptr);
    float* th = theta->data();
    const float* sn = sino->data();
    const size_t n = sino->size();
    if (cfg.alg == "sirt") run<GpuSIRTReconSpace>(cfg, TG_SIRT, th, sn, n);
    else if (cfg.alg == "mlem") run<GpuMLEMReconSpace>(cfg, TG_MLEM, th, sn, n);
    else if (cfg.alg == "pml") run<GpuPMLReconSpace>(cfg, TG_PML, th, sn, n);
    else if (cfg.alg == "apmlr") run<GpuAPMLRReconSpace>(cfg, TG_APMLR, th, sn, n);
    else throw std::runtime_error("unknown algorithm " + cfg.alg);
  } catch (const std::exception& e) {
    std::cerr << e.what() << std::endl;
    return 1;
  }
  return 0;
}
