/* Test infrastructure only: the CPU restatement ("the oracle") of Trace's
 * iterative-reconstruction hot path. Tests, smoke() and bench.py's CPU
 * baseline call it as the checker; the product never links it.
 *
 * Precision modes:
 *   TOR_F32: IEEE single precision with no contraction, one thread ->
 *            bit-identical to the reference (src/common/trace_utils.cc,
 *            src/sirt, src/mlem, src/pml and src/apmlr sources built with strict -O3).
 *   TOR_F64: the same algorithm with the reconstruction, replicas, F/G and
 *            every sum and update in double. The geometry (crossing points,
 *            pixel indices) is traced in float exactly as the reference does,
 *            so index lists are identical; lengths are the reference's float
 *            lengths widened (dlen=0) or recomputed in double from the float
 *            crossing points (dlen=1).
 */
#ifndef TRACE_ORACLE_H
#define TRACE_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { TOR_SIRT = 0, TOR_MLEM = 1, TOR_PML = 2, TOR_APMLR = 3 };
enum { TOR_F32 = 0, TOR_F64 = 1 };

/* Per-angle (quadrant, sinf, cosf) as SIRTReconSpace::Reduce computes them
 * (src/sirt/sirt.cc:117-121, quadrant rule src/common/trace_utils.cc:41-46). */
int tor_angle_table(int num_projs, const float* theta, float* sinq, float* cosq,
                    int32_t* quad);

/* TraceMetadata's derived geometry (src/common/trace_data.h:96-108):
 * mov and the g+1 grid lines (gridx == gridy). */
int tor_geometry(int num_cols, float center, float* mov, float* grid);

/* Segment counts per ray r = p*C + c (max(len-1,0)). */
int tor_trace_counts(int num_cols, int num_projs, float center,
                     const float* sinq, const float* cosq, const int32_t* quad,
                     int32_t* counts, int threads);

/* Segment lists: ray r's segments at offsets[r] .. offsets[r]+counts[r]-1.
 * len2 may be NULL. */
int tor_trace_fill(int num_cols, int num_projs, float center, const float* sinq,
                   const float* cosq, const int32_t* quad,
                   const int64_t* offsets, int32_t* idx, float* len,
                   float* len2, int threads);

typedef struct {
  int alg;            /* TOR_SIRT .. TOR_APMLR */
  int precision;      /* TOR_F32 / TOR_F64 */
  int dlen;           /* F64 only: 1 = lengths recomputed in double */
  int num_projs, num_slices, num_cols;
  float center;       /* <= 0 -> C/2 + 1 (trace_data.h:97) */
  const float* theta; /* radians, used when sinq is NULL */
  const float* sinq;  /* optional per-angle tables (all three or none) */
  const float* cosq;
  const int32_t* quad;
  const float* sino;  /* [P][S][C] */
  int apply_abs;      /* 1 = trace_utils::Absolute on the sinogram first */
  int n_iter;
  int threads;        /* replicas + tree merge as the DISP engine; 1 = exact order */
  float beta, beta1, delta, delta1, regw;
  int slice_id, num_total_slices; /* APMLR top/bottom selection (apmlr.cc:919-967) */
  int apmlr_fixed;    /* 0 = reference forward-projection slice offset, 1 = fixed */
  const void* recon_in;  /* optional start recon (same layout/type as recon_out) */
  void* recon_out;    /* (S + 2*halo) * C*C of float or double; halo = 1 for APMLR */
  void* iters_out;    /* optional n_iter snapshots of recon_out */
  void* replica_out;  /* optional S * 2*C*C: last iteration's combined replica */
} tor_run_args;

int tor_run(const tor_run_args* a);

/* Forward projection in the reference's order (CalculateSimdata,
 * sirt.cc:4-19): sim[p][s][c] = sum over ray (p,c) of recon[s][idx]*len,
 * accumulated sequentially in float. recon: S x C x C. */
int tor_forward(int num_cols, int num_projs, int num_slices, float center,
                const float* sinq, const float* cosq, const int32_t* quad,
                const float* recon, float* sim, int threads);

/* F and G of PML / APMLR for a given reconstruction (including APMLR's
 * halo slices: S + 2 slices) and per-pixel total length W (C x C), exactly
 * as CalculateFG leaves them (G includes W). F, G: S x C x C. */
int tor_fg(int alg, int num_slices, int num_cols, const float* recon,
           const float* W, float beta, float beta1, float delta, float delta1,
           float regw, int slice_id, int num_total_slices, float* F, float* G);

/* Seconds spent in the last tor_run's iteration loop (reduction + combine +
 * FG + update), the span the reference drivers' timers cover. */
double tor_last_loop_seconds(void);

#ifdef __cplusplus
}
#endif
#endif
