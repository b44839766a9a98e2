// Test infrastructure only: CPU restatement of Trace's reconstruction hot
// path, used as the checker by tests/, __graft_entry__.smoke() and the CPU
// baseline leg of bench.py. Must be compiled with -ffp-contract=off (see
// oracle/Makefile): every float expression below is meant as a sequence of
// individually rounded IEEE single operations, as in the reference.
//
// Reference correspondence (file:line within the reference project):
//   angle table      src/sirt/sirt.cc:117-121, src/common/trace_utils.cc:41-46
//   geometry         src/common/trace_data.h:96-108
//   ray tracing      src/common/trace_utils.cc:48-216 (coordinates, trim,
//                    merge, lengths/indices), driven as in src/sirt/sirt.cc:126-160
//   forward / scatter src/sirt/sirt.cc:4-64, src/mlem/mlem.cc:4-61,
//                    src/pml/pml.cc:204-246, src/apmlr/apmlr.cc:985-1027
//   UpdateRecon      src/sirt/sirt.cc:21-33, src/mlem/mlem.cc:21-34,
//                    src/pml/pml.cc:3-23, src/apmlr/apmlr.cc:3-26
//   penalty F/G      src/pml/pml.cc:25-201 (+ weights src/pml/pml.h:22-29),
//                    src/apmlr/apmlr.cc:28-982
//   engine           src/common/DISP/core/disp_engine_reduction.h:132-202
#include "trace_oracle.h"

#include <atomic>
#include <chrono>
#include <cmath>
#include <cstring>
#include <memory>
#include <thread>
#include <vector>

namespace {

constexpr float kPI = 3.14159265358979f;  // trace_utils.h:8

double g_last_loop_seconds = 0.0;

int quadrant_of(float t) {
  return ((t >= 0 && t < kPI / 2) || (t >= kPI && t < 3 * kPI / 2)) ? 1 : 0;
}

struct Geometry {
  int C = 0, P = 0;  // grid size g == C
  float mov = 0.f, mgrids = 0.f;
  std::vector<float> grid;  // g+1 lines, gridx == gridy
  std::vector<float> yi;    // per detector column
  std::vector<float> sinq, cosq;
  std::vector<int> quad;
};

void make_geometry(Geometry& G, int C, int P, float center, const float* theta,
                   const float* sinq, const float* cosq, const int32_t* quad) {
  G.C = C;
  G.P = P;
  float ctr = (center <= 0.) ? static_cast<float>(C) / 2. + 1. : center;
  float mov = static_cast<float>(C) / 2. - ctr;
  if (mov - std::ceil(mov) < 1e-6) mov += 1e-6;  // always true: mov <= ceil(mov)
  G.mov = mov;
  G.mgrids = C / 2.;
  G.grid.resize(C + 1);
  for (int i = 0; i <= C; ++i) G.grid[i] = -C / 2. + i;
  G.yi.resize(C);
  for (int c = 0; c < C; ++c) G.yi[c] = (1 - C) / 2. + c + mov;
  G.sinq.resize(P);
  G.cosq.resize(P);
  G.quad.resize(P);
  for (int p = 0; p < P; ++p) {
    if (sinq) {
      G.sinq[p] = sinq[p];
      G.cosq[p] = cosq[p];
      G.quad[p] = quad[p];
    } else {
      G.sinq[p] = sinf(theta[p]);
      G.cosq[p] = cosf(theta[p]);
      G.quad[p] = quadrant_of(theta[p]);
    }
  }
}

// One traced segment: pixel index, float length and squared length, and
// (when requested) the double-precision length of the same float points.
struct Seg {
  int idx;
  float len, len2;
  double dlen, dlen2;
};

// Per-thread scratch of the tracer: the crossing coordinates of one ray
// with every horizontal (cx) and vertical (cy) grid line.
struct TraceWs {
  std::vector<float> cx, cy;
  std::vector<Seg> segs;
  // merged crossing points and per-segment results of trace_ray_arrays
  std::vector<float> px, py, len, len2;
  std::vector<int> idx;
  explicit TraceWs(int g)
      : cx(g + 1), cy(g + 1), px(2 * g + 2), py(2 * g + 2), len(2 * g + 2),
        len2(2 * g + 2), idx(2 * g + 2) {
    segs.reserve(2 * g + 2);
  }
};

// Streams the segments of ray (p, c) to `emit` in the reference's order.
//
// The reference materialises all g+1 crossings with horizontal lines
// ("a" points, x = islope*(y_n - srcy) + srcx) and vertical lines ("b"
// points, y = slope*(x_n - srcx) + srcy), keeps those strictly inside the
// grid, and merges the a list (in n order for quadrant 1, reversed for
// quadrant 0) with the b list by x, taking b on ties. Here the two lists
// are walked by cursors that skip rejected crossings, so each output point
// is produced in the same order without the arrays.
template <bool WANT_DOUBLE = false, class Emit>
int trace_ray(const Geometry& G, int p, int c, TraceWs& ws, Emit&& emit) {
  const int g = G.C;
  const float* grid = G.grid.data();
  const float xi = -1e6f;
  const float yi = G.yi[c];
  const float s = G.sinq[p], co = G.cosq[p];
  const float srcx = xi * co - yi * s;
  const float srcy = xi * s + yi * co;
  const float detx = -1 * (xi * co + yi * s);
  const float dety = -xi * s + yi * co;
  const float slope = (srcy - dety) / (srcx - detx);
  const float islope = 1 / slope;
  const float lo = grid[0], hi = grid[g];
  // all crossings first (a vectorisable loop, as CalculateCoordinates)
  float* cx = ws.cx.data();
  float* cy = ws.cy.data();
  for (int n = 0; n <= g; ++n) {
    cx[n] = islope * (grid[n] - srcy) + srcx;
    cy[n] = slope * (grid[n] - srcx) + srcy;
  }

  const int da = G.quad[p] ? 1 : -1;
  int na = G.quad[p] ? 0 : g;
  float ax = 0.f;
  auto seek_a = [&]() {
    for (; na >= 0 && na <= g; na += da) {
      ax = cx[na];
      if (ax > lo && ax < hi) return;
    }
  };
  int nb = 0;
  float by = 0.f;
  auto seek_b = [&]() {
    for (; nb <= g; ++nb) {
      by = cy[nb];
      if (by > lo && by < hi) return;
    }
  };
  seek_a();
  seek_b();

  int nseg = 0;
  bool have_prev = false;
  float px = 0.f, py = 0.f;
  for (;;) {
    const bool va = (na >= 0 && na <= g), vb = (nb <= g);
    if (!va && !vb) break;
    const bool take_a = va && (!vb || ax < grid[nb]);
    float x, y;
    if (take_a) {
      x = ax;
      y = grid[na];
      na += da;
      seek_a();
    } else {
      x = grid[nb];
      y = by;
      ++nb;
      seek_b();
    }
    if (have_prev) {
      Seg sg;
      const float dx = x - px, dy = y - py;
      const float midx = (x + px) / 2., midy = (y + py) / 2.;
      sg.len2 = dx * dx + dy * dy;
      sg.len = std::sqrt(sg.len2);
      const int ix = midx + G.mgrids;  // truncation, as trace_utils.cc:179
      const int iy = midy + G.mgrids;
      sg.idx = ix + iy * g;
      if (WANT_DOUBLE) {
        const double ddx = (double)x - (double)px, ddy = (double)y - (double)py;
        sg.dlen2 = ddx * ddx + ddy * ddy;
        sg.dlen = std::sqrt(sg.dlen2);
      }
      // A stray segment whose cell index falls outside the grid (the
      // reference would index its arrays out of bounds: undefined) is
      // dropped; in-grid indices are kept as the reference forms them.
      if (sg.idx >= 0 && sg.idx < g * g) {
        emit(sg);
        ++nseg;
      }
    }
    px = x;
    py = y;
    have_prev = true;
  }
  return nseg;
}

// The same tracing as trace_ray in three passes over arrays (crossings,
// merge, lengths), so the first and last passes vectorise. Fills ws.idx,
// ws.len, ws.len2 and returns the segment count.
int trace_ray_arrays(const Geometry& G, int p, int c, TraceWs& ws) {
  const int g = G.C;
  const float* grid = G.grid.data();
  const float xi = -1e6f;
  const float yi = G.yi[c];
  const float s = G.sinq[p], co = G.cosq[p];
  const float srcx = xi * co - yi * s;
  const float srcy = xi * s + yi * co;
  const float detx = -1 * (xi * co + yi * s);
  const float dety = -xi * s + yi * co;
  const float slope = (srcy - dety) / (srcx - detx);
  const float islope = 1 / slope;
  const float lo = grid[0], hi = grid[g];
  float* cx = ws.cx.data();
  float* cy = ws.cy.data();
  for (int n = 0; n <= g; ++n) {
    cx[n] = islope * (grid[n] - srcy) + srcx;
    cy[n] = slope * (grid[n] - srcx) + srcy;
  }
  float* px = ws.px.data();
  float* py = ws.py.data();
  const int da = G.quad[p] ? 1 : -1;
  int na = G.quad[p] ? 0 : g, nb = 0, m = 0;
  while (na >= 0 && na <= g && !(cx[na] > lo && cx[na] < hi)) na += da;
  while (nb <= g && !(cy[nb] > lo && cy[nb] < hi)) ++nb;
  for (;;) {
    const bool va = (na >= 0 && na <= g), vb = (nb <= g);
    if (!va && !vb) break;
    if (va && (!vb || cx[na] < grid[nb])) {
      px[m] = cx[na];
      py[m] = grid[na];
      for (na += da; na >= 0 && na <= g && !(cx[na] > lo && cx[na] < hi); na += da) {
      }
    } else {
      px[m] = grid[nb];
      py[m] = cy[nb];
      for (++nb; nb <= g && !(cy[nb] > lo && cy[nb] < hi); ++nb) {
      }
    }
    ++m;
  }
  const int nseg = m > 1 ? m - 1 : 0;
  float* ln = ws.len.data();
  float* ln2 = ws.len2.data();
  int* ix = ws.idx.data();
  const float mg = G.mgrids;
  for (int i = 0; i < nseg; ++i) {
    const float dx = px[i + 1] - px[i], dy = py[i + 1] - py[i];
    const float midx = (px[i + 1] + px[i]) / 2., midy = (py[i + 1] + py[i]) / 2.;
    ln2[i] = dx * dx + dy * dy;
    ln[i] = std::sqrt(ln2[i]);
    ix[i] = (int)(midx + mg) + (int)(midy + mg) * g;
  }
  // drop stray segments outside the grid, as trace_ray does (rare)
  int kept = 0;
  for (int i = 0; i < nseg; ++i) {
    if (ix[i] < 0 || ix[i] >= g * g) continue;
    ix[kept] = ix[i];
    ln[kept] = ln[i];
    ln2[kept] = ln2[i];
    ++kept;
  }
  return kept;
}

template <class F>
void parallel_for(long n, int threads, F&& body) {
  if (threads <= 1 || n < 2) {
    for (long i = 0; i < n; ++i) body(i, 0);
    return;
  }
  std::atomic<long> next(0);
  std::vector<std::thread> pool;
  for (int t = 0; t < threads; ++t)
    pool.emplace_back([&, t]() {
      for (long i = next++; i < n; i = next++) body(i, t);
    });
  for (auto& th : pool) th.join();
}

// In-plane neighbour classes of the 8-neighbour penalty, with the
// neighbour order of the reference's region loops (pml.cc:39-192,
// apmlr.cc:57-346). kind 0 = orthogonal, 1 = diagonal.
struct NbrClass {
  int n;
  int dx[8], dy[8], kind[8];
};
const NbrClass kInterior = {8,
                            {1, -1, 0, 0, 1, -1, 1, -1},
                            {0, 0, 1, -1, 1, 1, -1, -1},
                            {0, 0, 0, 0, 1, 1, 1, 1}};
const NbrClass kTop = {5, {1, -1, 0, 1, -1}, {0, 0, 1, 1, 1}, {0, 0, 0, 1, 1}};
const NbrClass kBottom = {5, {1, -1, 0, 1, -1}, {0, 0, -1, -1, -1}, {0, 0, 0, 1, 1}};
const NbrClass kLeft = {5, {1, 0, 0, 1, 1}, {0, 1, -1, 1, -1}, {0, 0, 0, 1, 1}};
const NbrClass kRight = {5, {-1, 0, 0, -1, -1}, {0, 1, -1, 1, -1}, {0, 0, 0, 1, 1}};
const NbrClass kTL = {3, {1, 0, 1}, {0, 1, 1}, {0, 0, 1}};
const NbrClass kTR = {3, {-1, 0, -1}, {0, 1, 1}, {0, 0, 1}};
const NbrClass kBL = {3, {1, 0, 1}, {0, -1, -1}, {0, 0, 1}};
const NbrClass kBR = {3, {-1, 0, -1}, {0, -1, -1}, {0, 0, 1}};

// 0 interior, 1 edge, 2 corner
const NbrClass& class_of(int x, int y, int g, int* region) {
  const bool l = x == 0, r = x == g - 1, t = y == 0, b = y == g - 1;
  if ((l || r) && (t || b)) {
    *region = 2;
    return t ? (l ? kTL : kTR) : (l ? kBL : kBR);
  }
  if (l || r || t || b) {
    *region = 1;
    return t ? kTop : b ? kBottom : l ? kLeft : kRight;
  }
  *region = 0;
  return kInterior;
}

// PML weights (pml.h:22-29): {orthogonal, diagonal} per region.
const float kPmlW[3][2] = {{(float)0.1464466094, (float)0.10355339059},
                           {(float)0.226540919667, (float)0.1601886205},
                           {(float)0.36939806251, (float)0.26120387496}};

// APMLR weights (apmlr.cc:40-51, 90-97, 228-233 and the top/bottom
// variants): totals 4+4/sqrt(2), 3+2/sqrt(2), 2+1/sqrt(2) plus regw per
// axial neighbour, evaluated in double and stored as float.
struct ApmlrW {
  float o, d, a;
};
ApmlrW apmlr_weights(int region, int n_axial, float regw) {
  const double base[3] = {4 + 4 / std::sqrt(2.0), 3 + 2 / std::sqrt(2.0),
                          2 + 1 / std::sqrt(2.0)};
  float total = (n_axial == 2) ? (float)(base[region] + 2 * regw)
                               : (float)(base[region] + regw);
  ApmlrW w;
  w.o = 1 / total;
  w.d = (float)(1 / std::sqrt(2.0) / total);
  w.a = regw / total;
  return w;
}

template <class T>
struct Run {
  const tor_run_args& A;
  Geometry G;
  int S, g, halo;
  size_t g2;
  std::vector<T> recon;  // (S + 2*halo) * g2
  std::vector<float> sino;

  explicit Run(const tor_run_args& a) : A(a) {
    make_geometry(G, a.num_cols, a.num_projs, a.center, a.theta, a.sinq,
                  a.cosq, a.quad);
    S = a.num_slices;
    g = a.num_cols;
    g2 = (size_t)g * g;
    halo = (a.alg == TOR_APMLR) ? 1 : 0;
    recon.assign((S + 2 * halo) * g2, (T)(a.alg == TOR_SIRT ? 0.f : 1.f));
    if (a.recon_in) {
      const T* src = static_cast<const T*>(a.recon_in);
      std::copy(src, src + recon.size(), recon.begin());
    }
    const size_t n = (size_t)a.num_projs * S * g;
    sino.assign(a.sino, a.sino + n);
    if (a.apply_abs)
      for (auto& v : sino) v = std::fabs(v);
  }

  T seg_len(const Seg& s) const {
    return (A.precision == TOR_F64 && A.dlen) ? (T)s.dlen : (T)s.len;
  }
  T seg_len2(const Seg& s) const {
    return (A.precision == TOR_F64 && A.dlen) ? (T)s.dlen2 : (T)s.len2;
  }

  // Forward projection source slice for sinogram slice s.
  const T* fwd_slice(int s) const {
    int off = s;
    if (A.alg == TOR_APMLR && A.apmlr_fixed) off = s + 1;
    return recon.data() + (size_t)off * g2;
  }

  // Float path of one ray, over the tracer's arrays (the reference's loops:
  // CalculateSimdata then UpdateReconReplica).
  void reduce_ray_f32(int p, int c, const T* rc, T* row, float rayv,
                      TraceWs& ws) {
    const int n = trace_ray_arrays(G, p, c, ws);
    const int* ix = ws.idx.data();
    const float* ln = ws.len.data();
    float sim = 0.f;
    for (int i = 0; i < n; ++i) sim += (float)rc[ix[i]] * ln[i];
    if (A.alg == TOR_SIRT) {
      float a2 = 0.f;
      const float* ln2 = ws.len2.data();
      for (int i = 0; i < n; ++i) a2 += ln2[i];
      const float upd = (rayv - sim) / a2;
      for (int i = 0; i < n; ++i) {
        row[(size_t)ix[i] * 2] += ln[i] * upd;
        row[(size_t)ix[i] * 2 + 1] += ln[i];
      }
    } else if (A.alg == TOR_MLEM) {
      const float upd = rayv / sim;
      for (int i = 0; i < n; ++i) {
        row[(size_t)ix[i] * 2] += ln[i] * upd;
        row[(size_t)ix[i] * 2 + 1] += ln[i];
      }
    } else {
      const float upd = rayv / sim;
      for (int i = 0; i < n; ++i) {
        row[(size_t)ix[i] * 2] -= rc[ix[i]] * ln[i] * upd;
        row[(size_t)ix[i] * 2 + 1] += ln[i];
      }
    }
  }

  // One work unit = one (projection, slice) row of C rays, exactly the
  // chunk the reference engine hands out (sirt_main.cc:172).
  void reduce_unit(long u, std::vector<T>& rep, TraceWs& ws) {
    std::vector<Seg>& buf = ws.segs;
    const int p = (int)(u / S), s = (int)(u % S);
    const T* rc = fwd_slice(s);
    T* row = rep.data() + (size_t)s * 2 * g2;
    const float* rays = sino.data() + ((size_t)p * S + s) * g;
    for (int c = 0; c < g; ++c) {
      if (A.precision == TOR_F32) {
        reduce_ray_f32(p, c, rc, row, rays[c], ws);
        continue;
      }
      buf.clear();
      if (A.dlen)
        trace_ray<true>(G, p, c, ws, [&](const Seg& sg) { buf.push_back(sg); });
      else
        trace_ray<false>(G, p, c, ws, [&](const Seg& sg) { buf.push_back(sg); });
      T sim = 0.;
      for (const Seg& sg : buf) sim += rc[sg.idx] * seg_len(sg);
      const T ray = rays[c];
      if (A.alg == TOR_SIRT) {
        T a2 = 0.;
        for (const Seg& sg : buf) a2 += seg_len2(sg);
        const T upd = (ray - sim) / a2;
        for (const Seg& sg : buf) {
          const T l = seg_len(sg);
          row[(size_t)sg.idx * 2] += l * upd;
          row[(size_t)sg.idx * 2 + 1] += l;
        }
      } else if (A.alg == TOR_MLEM) {
        const T upd = ray / sim;
        for (const Seg& sg : buf) {
          const T l = seg_len(sg);
          row[(size_t)sg.idx * 2] += l * upd;
          row[(size_t)sg.idx * 2 + 1] += l;
        }
      } else {
        const T upd = ray / sim;
        for (const Seg& sg : buf) {
          const T l = seg_len(sg);
          row[(size_t)sg.idx * 2] -= rc[sg.idx] * l * upd;
          row[(size_t)sg.idx * 2 + 1] += l;
        }
      }
    }
  }

  // F and G of the penalised algorithms for every slice.
  void calculate_fg(const std::vector<T>& rep, std::vector<T>& F,
                    std::vector<T>& Gv) {
    F.assign(S * g2, (T)0.);
    Gv.assign(S * g2, (T)0.);
    const T* rb = recon.data() + (size_t)halo * g2;  // true slice 0
    for (int k = 0; k < S; ++k) {
      int n_axial = 0, up = 0, down = 0;
      if (A.alg == TOR_APMLR) {
        const int beg = A.slice_id, end = A.slice_id + S - 1;
        const int final_index = A.slice_id + A.num_total_slices - 1;
        const bool top = (beg == 0 && k == 0);
        const bool bottom =
            !top && (final_index == end && final_index != 0 && k == S - 1);
        up = !bottom;   // neighbour at +g2 (apmlr.cc:63, 388)
        down = !top;    // neighbour at -g2
        n_axial = up + down;
      }
      for (int y = 0; y < g; ++y)
        for (int x = 0; x < g; ++x) {
          int region;
          const NbrClass& nc = class_of(x, y, g, &region);
          const size_t i0 = (size_t)k * g2 + (size_t)y * g + x;
          const T r0 = rb[i0];
          T f = F[i0], gg = Gv[i0];
          if (A.alg == TOR_PML) {
            const T twob = (T)(2 * A.beta);
            for (int q = 0; q < nc.n; ++q) {
              const T w = (T)kPmlW[region][nc.kind[q]];
              const T rq = rb[i0 + nc.dx[q] + (long)nc.dy[q] * g];
              f += twob * w;
              gg -= twob * w * (r0 + rq);
            }
          } else {
            const ApmlrW w = apmlr_weights(region, n_axial, A.regw);
            const T twob = (T)(2 * A.beta), twob1 = (T)(2 * A.beta1);
            const T delta = (T)A.delta, delta1 = (T)A.delta1;
            for (int q = 0; q < nc.n; ++q) {
              const T wq = (T)(nc.kind[q] ? w.d : w.o);
              const T rq = rb[i0 + nc.dx[q] + (long)nc.dy[q] * g];
              const T mg = r0 + rq, rg = r0 - rq;
              const T gam = 1 / (1 + std::fabs(rg / delta));
              f += twob * wq * gam;
              gg -= twob * wq * gam * mg;
            }
            const long axial[2] = {(long)g2, -(long)g2};
            const int use[2] = {up, down};
            for (int q = 0; q < 2; ++q) {
              if (!use[q]) continue;
              const T wq = (T)w.a;
              const T rq = rb[(long)i0 + axial[q]];
              const T mg = r0 + rq, rg = r0 - rq;
              const T gam = 1 / (1 + std::fabs(rg / delta1));
              f += twob1 * wq * gam;
              gg -= twob1 * wq * gam * mg;
            }
          }
          F[i0] = f;
          Gv[i0] = gg;
        }
    }
    for (int k = 0; k < S; ++k)
      for (size_t j = 0; j < g2; ++j)
        Gv[(size_t)k * g2 + j] += rep[(size_t)k * 2 * g2 + 2 * j + 1];
  }

  void update(const std::vector<T>& rep) {
    T* rb = recon.data() + (size_t)halo * g2;
    if (A.alg == TOR_SIRT || A.alg == TOR_MLEM) {
      for (int k = 0; k < S; ++k)
        for (size_t j = 0; j < g2; ++j) {
          const T* r = rep.data() + (size_t)k * 2 * g2;
          const T q = r[2 * j] / r[2 * j + 1];
          if (A.alg == TOR_SIRT)
            rb[(size_t)k * g2 + j] += q;
          else
            rb[(size_t)k * g2 + j] *= q;
        }
      return;
    }
    std::vector<T> F, Gv;
    calculate_fg(rep, F, Gv);
    for (int k = 0; k < S; ++k)
      for (size_t j = 0; j < g2; ++j) {
        const size_t i = (size_t)k * g2 + j;
        const T num = rep[(size_t)k * 2 * g2 + 2 * j];
        rb[i] = (-Gv[i] + std::sqrt(Gv[i] * Gv[i] - 8 * num * F[i])) /
                (4 * F[i]);
      }
  }

  int run() {
    const int T_ = A.threads < 1 ? (int)std::thread::hardware_concurrency()
                                 : A.threads;
    const int nthr = T_ < 1 ? 1 : T_;
    const size_t rep_n = (size_t)S * 2 * g2;
    std::vector<std::vector<T>> reps(nthr, std::vector<T>(rep_n, (T)0.));
    // one heap-allocated workspace per thread (no shared cache lines)
    std::vector<std::unique_ptr<TraceWs>> wss;
    for (int t = 0; t < nthr; ++t) wss.emplace_back(new TraceWs(g));
    const long units = (long)A.num_projs * S;
    auto t0 = std::chrono::steady_clock::now();
    for (int it = 0; it < A.n_iter; ++it) {
      parallel_for(units, nthr,
                   [&](long u, int t) { reduce_unit(u, reps[t], *wss[t]); });
      // pairwise tree combination, as ParInPlaceLocalSynch(…, 2, …)
      for (int step = 1; step < nthr; step *= 2)
        parallel_for((nthr + 2 * step - 1) / (2 * step), nthr, [&](long i, int) {
          const int a = (int)i * 2 * step, b = a + step;
          if (b < nthr)
            for (size_t j = 0; j < rep_n; ++j) reps[a][j] += reps[b][j];
        });
      if (A.replica_out && it == A.n_iter - 1)
        std::memcpy(A.replica_out, reps[0].data(), rep_n * sizeof(T));
      update(reps[0]);
      for (auto& r : reps) std::fill(r.begin(), r.end(), (T)0.);
      if (A.iters_out)
        std::memcpy(static_cast<T*>(A.iters_out) + (size_t)it * recon.size(),
                    recon.data(), recon.size() * sizeof(T));
    }
    g_last_loop_seconds =
        std::chrono::duration<double>(std::chrono::steady_clock::now() - t0)
            .count();
    std::memcpy(A.recon_out, recon.data(), recon.size() * sizeof(T));
    return 0;
  }
};

}  // namespace

extern "C" {

int tor_angle_table(int num_projs, const float* theta, float* sinq, float* cosq,
                    int32_t* quad) {
  for (int p = 0; p < num_projs; ++p) {
    sinq[p] = sinf(theta[p]);
    cosq[p] = cosf(theta[p]);
    quad[p] = quadrant_of(theta[p]);
  }
  return 0;
}

int tor_geometry(int num_cols, float center, float* mov, float* grid) {
  if (num_cols < 2) return 1;
  Geometry G;
  float th = 0.f;
  make_geometry(G, num_cols, 1, center, &th, nullptr, nullptr, nullptr);
  *mov = G.mov;
  std::memcpy(grid, G.grid.data(), sizeof(float) * (num_cols + 1));
  return 0;
}

int tor_trace_counts(int num_cols, int num_projs, float center,
                     const float* sinq, const float* cosq, const int32_t* quad,
                     int32_t* counts, int threads) {
  if (num_cols < 2 || num_projs < 1) return 1;
  Geometry G;
  make_geometry(G, num_cols, num_projs, center, nullptr, sinq, cosq, quad);
  parallel_for((long)num_projs, threads, [&](long p, int) {
    TraceWs ws(num_cols);
    for (int c = 0; c < num_cols; ++c)
      counts[p * num_cols + c] = trace_ray(G, (int)p, c, ws, [](const Seg&) {});
  });
  return 0;
}

int tor_trace_fill(int num_cols, int num_projs, float center, const float* sinq,
                   const float* cosq, const int32_t* quad,
                   const int64_t* offsets, int32_t* idx, float* len,
                   float* len2, int threads) {
  if (num_cols < 2 || num_projs < 1) return 1;
  Geometry G;
  make_geometry(G, num_cols, num_projs, center, nullptr, sinq, cosq, quad);
  parallel_for((long)num_projs, threads, [&](long p, int) {
    TraceWs ws(num_cols);
    for (int c = 0; c < num_cols; ++c) {
      int64_t o = offsets[p * num_cols + c];
      trace_ray(G, (int)p, c, ws, [&](const Seg& s) {
        idx[o] = s.idx;
        len[o] = s.len;
        if (len2) len2[o] = s.len2;
        ++o;
      });
    }
  });
  return 0;
}

int tor_run(const tor_run_args* a) {
  if (!a || a->num_cols < 2 || a->num_projs < 1 || a->num_slices < 1 ||
      !a->sino || !a->recon_out || (!a->theta && !a->sinq))
    return 1;
  if (a->precision == TOR_F32) return Run<float>(*a).run();
  return Run<double>(*a).run();
}

int tor_forward(int num_cols, int num_projs, int num_slices, float center,
                const float* sinq, const float* cosq, const int32_t* quad,
                const float* recon, float* sim, int threads) {
  if (num_cols < 2 || num_projs < 1 || num_slices < 1) return 1;
  Geometry G;
  make_geometry(G, num_cols, num_projs, center, nullptr, sinq, cosq, quad);
  const size_t g2 = (size_t)num_cols * num_cols;
  parallel_for((long)num_projs, threads, [&](long p, int) {
    TraceWs ws(num_cols);
    std::vector<Seg>& buf = ws.segs;
    for (int c = 0; c < num_cols; ++c) {
      buf.clear();
      trace_ray(G, (int)p, c, ws, [&](const Seg& sg) { buf.push_back(sg); });
      for (int s = 0; s < num_slices; ++s) {
        const float* rc = recon + (size_t)s * g2;
        float acc = 0.f;
        for (const Seg& sg : buf) acc += rc[sg.idx] * sg.len;
        sim[((size_t)p * num_slices + s) * num_cols + c] = acc;
      }
    }
  });
  return 0;
}

int tor_fg(int alg, int num_slices, int num_cols, const float* recon,
           const float* W, float beta, float beta1, float delta, float delta1,
           float regw, int slice_id, int num_total_slices, float* F, float* G) {
  if ((alg != TOR_PML && alg != TOR_APMLR) || num_cols < 2 || num_slices < 1)
    return 1;
  tor_run_args a{};
  a.alg = alg;
  a.precision = TOR_F32;
  a.num_projs = 1;
  a.num_slices = num_slices;
  a.num_cols = num_cols;
  const float th = 0.f;
  a.theta = &th;
  std::vector<float> dummy((size_t)num_slices * num_cols, 0.f);
  a.sino = dummy.data();
  a.beta = beta;
  a.beta1 = beta1;
  a.delta = delta;
  a.delta1 = delta1;
  a.regw = regw;
  a.slice_id = slice_id;
  a.num_total_slices = num_total_slices;
  a.recon_in = recon;
  Run<float> run(a);
  const size_t g2 = (size_t)num_cols * num_cols;
  std::vector<float> rep((size_t)num_slices * 2 * g2, 0.f);
  for (int k = 0; k < num_slices; ++k)
    for (size_t j = 0; j < g2; ++j) rep[(size_t)k * 2 * g2 + 2 * j + 1] = W[j];
  std::vector<float> Fv, Gv;
  run.calculate_fg(rep, Fv, Gv);
  std::memcpy(F, Fv.data(), Fv.size() * sizeof(float));
  std::memcpy(G, Gv.data(), Gv.size() * sizeof(float));
  return 0;
}

double tor_last_loop_seconds(void) { return g_last_loop_seconds; }

}  // extern "C"
