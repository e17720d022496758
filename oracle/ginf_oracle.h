/*
 * ginf_oracle.h -- CPU restatement of GridInfCuda's grid-MRF inference path.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / reference arm of bench.py may load this library, and only as
 * the checker (or as the timed CPU baseline).  The product library
 * (gridinfcuda_gb300) never links or calls it.
 *
 * Parity pin: every function here is checked bit-for-bit against the
 * reference's own CPU code (src/bp.cc, src/icm.cc, src/grid.cc compiled
 * unmodified into oracle/_ref by oracle/Makefile) on seeded inputs and against
 * the golden fixtures in tests/golden/, which that compiled reference produced.
 *
 * Conventions (the reference's, see src/include/matrix.h:9-51, utils.h:26-37):
 *   data costs  D  label-planar, index x + W*y + W*H*l   (Matrix(3, W, H, L))
 *   smoothness  V  L x L table, index fp + L*fq          (Matrix(2, L, L))
 *   labels         index x + W*y                         (Matrix(2, W, H))
 *   directions     S=0 (+y), E=1 (+x), N=2 (-y), W=3 (-x)
 *   model          0 EXPLICIT, 1 POTTS, 2 TRUNC_LINEAR, 3 TRUNC_QUAD (grid.h:9-14)
 * Messages are returned in the receiver layout used by the GPU library:
 *   msgs[((y*W + x)*4 + d)*L + l] = message sent TO (x,y) BY its neighbour in
 *   direction d.  Slots whose sender lies outside the grid are left at 0.
 */
#ifndef GINF_ORACLE_H
#define GINF_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Hierarchical BP with the reference's exact semantics (src/bp.cc:86-187),
 * including the stale-belief decode (bp.cc:65-84, 168-173).  levels == 1 is
 * decodeBp (bp.cc:182-187).  Interior labels are written, border labels are
 * left untouched.  msgs_out (nullable) receives the level-0 messages.
 * nthreads <= 0 uses every OpenMP thread.  Returns 0, or -1 on bad input. */
int orc_hbp_f32(int W, int H, int L, const float *D, const float *V, int model,
                int levels, int iters, int32_t *labels, float *msgs_out, int nthreads);
int orc_hbp_i32(int W, int H, int L, const int32_t *D, const int32_t *V, int model,
                int levels, int iters, int32_t *labels, int32_t *msgs_out, int nthreads);

/* Standard min-sum BP in FP64: subtract the receiver's message, apply the
 * O(L) distance transform (linear scans or Felzenszwalb-Huttenlocher lower
 * envelope for the quadratic model, O(L^2) for EXPLICIT), truncate, then
 * normalise (norm 0 = subtract mean, 1 = subtract min).  decode 0 = stale
 * belief (as bp.cc), 1 = fresh belief from the final messages. */
int orc_hbp_f64_std(int W, int H, int L, const float *D, const float *V, int model,
                    int levels, int iters, int decode, int norm, int32_t *labels,
                    double *msgs_out, int nthreads);

/* Synchronous (Jacobi) ICM, src/icm.cc:4-38, and raster Gauss-Seidel ICM,
 * src/icm.cc:40-67.  result receives a full copy of initial first. */
int orc_icm_sync_f32(int W, int H, int L, const float *D, const float *V,
                     const int32_t *initial, int iters, int32_t *result, int nthreads);
int orc_icm_sync_i32(int W, int H, int L, const int32_t *D, const int32_t *V,
                     const int32_t *initial, int iters, int32_t *result, int nthreads);
int orc_icm_async_f32(int W, int H, int L, const float *D, const float *V,
                      const int32_t *initial, int iters, int32_t *result);
int orc_icm_async_i32(int W, int H, int L, const int32_t *D, const int32_t *V,
                      const int32_t *initial, int iters, int32_t *result);

/* Energy of a labelling, src/grid.cc:102-125 (interior nodes, N and E edges).
 * _seq accumulates in the grid type in raster order exactly as the reference;
 * _f64 sums the same terms in double. */
float   orc_energy_f32_seq(int W, int H, int L, const float *D, const float *V, const int32_t *f);
int32_t orc_energy_i32_seq(int W, int H, int L, const int32_t *D, const int32_t *V, const int32_t *f);
double  orc_energy_f64(int W, int H, int L, const float *D, const float *V, const int32_t *f);
double  orc_energy_i32_f64(int W, int H, int L, const int32_t *D, const int32_t *V, const int32_t *f);

/* Alpha-beta swap, src/graphcut.cc:197-279 (decodeAlphaBeta, int grids):
 * push-relabel max-flow per label pair in the reference's raster order, with
 * the state it carries across pairs.  result receives a copy of initial
 * first.  Returns 0, or -1 on bad input or allocation failure. */
int orc_alpha_beta_i32(int W, int H, int L, const int32_t *D, const int32_t *V, const int32_t *initial, int iters,
                       int32_t *result);

/* Building blocks exposed for unit tests. */
void orc_pyramid_f32(int W, int H, int L, const float *D, float *Dc);   /* bp.cc:100-117 one level */
void orc_send_linear_f32(int L, const float *from, const float *in, float scale, float trunc, float *out);
void orc_dt_quad_f64(int L, const double *f, double s, double *out);
void orc_minconv_brute_f64(int L, const double *f, const double *V, double *out);

#ifdef __cplusplus
}
#endif
#endif
