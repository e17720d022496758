/*
 * ginf_oracle.c -- CPU restatement of GridInfCuda's BP / HBP / ICM / energy.
 *
 * TEST INFRASTRUCTURE ONLY: loaded by tests/, __graft_entry__.smoke() and the
 * CPU-baseline legs of bench.py, never by the product library.  Build recipe:
 * oracle/Makefile (gcc -O2 -fopenmp -ffp-contract=off, so that no multiply-add
 * is fused on either x86-64 or aarch64 hosts).
 *
 * Pinned bit-for-bit against the reference CPU code (oracle/_ref, built from
 * src/{grid,matrix,bp,icm}.cc) and the golden fixtures in tests/golden/.
 */
#include "ginf_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

enum { ORC_EXPLICIT = 0, ORC_POTTS = 1, ORC_LINEAR = 2, ORC_QUAD = 3 }; /* grid.h:9-14 */

static const int ORC_DX[4] = {0, 1, 0, -1}; /* utils.h:36 (S, E, N, W) */
static const int ORC_DY[4] = {1, 0, -1, 0}; /* utils.h:37 */
#define ORC_OPP(d) ((d) >= 2 ? (d) - 2 : (d) + 2) /* utils.h:10 */
#define ORC_MIN(a, b) (((a) < (b)) ? (a) : (b))   /* utils.h:16 */

static void orc_set_threads(int n)
{
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
    else omp_set_num_threads(omp_get_num_procs());
#else
    (void)n;
#endif
}

#define T float
#define SFX f32
#include "ginf_oracle_ref.inc"
#undef T
#undef SFX

#define T int32_t
#define SFX i32
#include "ginf_oracle_ref.inc"
#undef T
#undef SFX

/* ------------------------------------------------------------------------ */
/* Energy, src/grid.cc:102-125: interior nodes, data term plus the N and E    */
/* edges (dirY[N] = -1, dirX[E] = +1, utils.h:36-37).                         */

#define ORC_ENERGY_TERMS(ACC, CONV)                                                        \
    for (int y = 1; y < H - 1; y++) {                                                      \
        for (int x = 1; x < W - 1; x++) {                                                  \
            const int fl = f[(size_t)y * W + x];                                           \
            ACC += CONV(D[(size_t)x + (size_t)W * y + (size_t)W * H * fl]);                \
            ACC += CONV(V[fl + (size_t)L * f[(size_t)(y - 1) * W + x]]);                   \
            ACC += CONV(V[fl + (size_t)L * f[(size_t)y * W + x + 1]]);                     \
        }                                                                                  \
    }
#define ORC_ID(v) (v)
#define ORC_TO_D(v) ((double)(v))

float orc_energy_f32_seq(int W, int H, int L, const float *D, const float *V, const int32_t *f)
{
    float total = 0;
    ORC_ENERGY_TERMS(total, ORC_ID)
    return total;
}

int32_t orc_energy_i32_seq(int W, int H, int L, const int32_t *D, const int32_t *V, const int32_t *f)
{
    int32_t total = 0;
    ORC_ENERGY_TERMS(total, ORC_ID)
    return total;
}

double orc_energy_f64(int W, int H, int L, const float *D, const float *V, const int32_t *f)
{
    double total = 0;
    ORC_ENERGY_TERMS(total, ORC_TO_D)
    return total;
}

double orc_energy_i32_f64(int W, int H, int L, const int32_t *D, const int32_t *V, const int32_t *f)
{
    double total = 0;
    ORC_ENERGY_TERMS(total, ORC_TO_D)
    return total;
}

/* ------------------------------------------------------------------------ */
/* Building blocks.                                                           */

void orc_pyramid_f32(int W, int H, int L, const float *D, float *Dc)
{
    /* bp.cc:100-117 for one level, label-planar in and out. */
    const int w = (W + 1) / 2, h = (H + 1) / 2;
    memset(Dc, 0, sizeof(float) * (size_t)w * h * L);
    for (int y = 0; y < H; y++)
        for (int x = 0; x < W; x++)
            for (int i = 0; i < L; i++)
                Dc[(size_t)(x / 2) + (size_t)w * (y / 2) + (size_t)w * h * i] +=
                    D[(size_t)x + (size_t)W * y + (size_t)W * H * i];
}

void orc_send_linear_f32(int L, const float *from, const float *in, float scale, float trunc, float *out)
{
    send_f32(L, ORC_LINEAR, NULL, from, in, scale, trunc, out);
}

/* 1-D distance transform under a quadratic, min_q f(q) + s (p-q)^2, by the
 * lower envelope of parabolas: P. Felzenszwalb and D. Huttenlocher,
 * "Distance Transforms of Sampled Functions", Theory of Computing 8 (2012),
 * algorithm DT(f).  v holds the envelope's parabola vertices, z the
 * boundaries between them. */
static void dt_quad_f64(int L, const double *f, double s, double *out, int *v, double *z)
{
    if (!(s > 0)) {
        double m = f[0];
        for (int q = 1; q < L; q++) m = f[q] < m ? f[q] : m;
        for (int q = 0; q < L; q++) out[q] = m;
        return;
    }
    int k = 0;
    v[0] = 0;
    z[0] = -INFINITY;
    z[1] = INFINITY;
    for (int q = 1; q < L; q++) {
        double sq;
        for (;;) {
            const int p = v[k];
            sq = ((f[q] + s * q * q) - (f[p] + s * p * p)) / (2.0 * s * (q - p));
            if (sq <= z[k] && k > 0) {
                k--;
                continue;
            }
            break;
        }
        if (sq <= z[k]) {
            /* k == 0 and the new parabola dominates everywhere. */
            v[0] = q;
            z[0] = -INFINITY;
            z[1] = INFINITY;
            continue;
        }
        k++;
        v[k] = q;
        z[k] = sq;
        z[k + 1] = INFINITY;
    }
    k = 0;
    for (int q = 0; q < L; q++) {
        while (z[k + 1] < q) k++;
        const int p = v[k];
        out[q] = s * (double)(q - p) * (double)(q - p) + f[p];
    }
}

void orc_dt_quad_f64(int L, const double *f, double s, double *out)
{
    int *v = (int *)malloc(sizeof(int) * (size_t)L);
    double *z = (double *)malloc(sizeof(double) * (size_t)(L + 1));
    dt_quad_f64(L, f, s, out, v, z);
    free(v);
    free(z);
}

void orc_minconv_brute_f64(int L, const double *f, const double *V, double *out)
{
    for (int i = 0; i < L; i++) {
        double m = V[i] + f[0];
        for (int j = 1; j < L; j++) {
            const double c = V[i + (size_t)L * j] + f[j];
            m = c < m ? c : m;
        }
        out[i] = m;
    }
}

/* ------------------------------------------------------------------------ */
/* Standard min-sum BP in FP64 (the check for the standard message rule, the */
/* FP16 message store and the quadratic model).  Same schedule as bp.cc:     */
/* pyramid (bp.cc:100-117), coarse-to-fine copy (bp.cc:129-139), interior    */
/* checkerboard half-sweeps (bp.cc:148-150).                                  */

static void std_send_f64(int L, int model, const double *V, const double *from, const double *in,
                         double scale, double trunc, int norm, double *h, double *out, int *v, double *z)
{
    double minh = INFINITY;
    for (int i = 0; i < L; i++) {
        h[i] = from[i] - in[i];
        minh = h[i] < minh ? h[i] : minh;
    }
    if (model == ORC_LINEAR || model == ORC_POTTS) {
        for (int i = 0; i < L; i++) out[i] = h[i];
        for (int i = 1; i < L; i++) out[i] = ORC_MIN(out[i], out[i - 1] + scale);
        for (int i = L - 2; i >= 0; i--) out[i] = ORC_MIN(out[i], out[i + 1] + scale);
        for (int i = 0; i < L; i++) out[i] = ORC_MIN(out[i], minh + trunc);
    } else if (model == ORC_QUAD) {
        dt_quad_f64(L, h, scale, out, v, z);
        for (int i = 0; i < L; i++) out[i] = ORC_MIN(out[i], minh + trunc);
    } else {
        orc_minconv_brute_f64(L, h, V, out);
    }
    double c;
    if (norm == 1) {
        c = out[0];
        for (int i = 1; i < L; i++) c = out[i] < c ? out[i] : c;
    } else {
        c = 0;
        for (int i = 0; i < L; i++) c += out[i];
        c /= L;
    }
    for (int i = 0; i < L; i++) out[i] -= c;
}

int orc_hbp_f64_std(int W, int H, int L, const float *D, const float *Vf, int model,
                    int levels, int iters, int decode, int norm, int32_t *labels,
                    double *msgs_out, int nthreads)
{
    if (W <= 0 || H <= 0 || L < 2 || levels < 1 || iters < 0 || !D || !Vf || !labels) return -1;
    orc_set_threads(nthreads);
    const size_t L_ = (size_t)L;
    double *V = (double *)malloc(sizeof(double) * L_ * L_);
    for (size_t i = 0; i < L_ * L_; i++) V[i] = Vf[i];
    int *ws = (int *)malloc(sizeof(int) * levels), *hs = (int *)malloc(sizeof(int) * levels);
    double **data = (double **)calloc((size_t)levels, sizeof(double *));
    ws[0] = W;
    hs[0] = H;
    data[0] = (double *)malloc(sizeof(double) * (size_t)W * H * L_);
    for (int l = 0; l < L; l++)
        for (int y = 0; y < H; y++)
            for (int x = 0; x < W; x++)
                data[0][((size_t)y * W + x) * L_ + l] = D[(size_t)x + (size_t)W * y + (size_t)W * H * l];
    for (int t = 1; t < levels; t++) {
        ws[t] = (ws[t - 1] + 1) / 2;
        hs[t] = (hs[t - 1] + 1) / 2;
        data[t] = (double *)calloc((size_t)ws[t] * hs[t] * L_, sizeof(double));
        for (int y = 0; y < hs[t - 1]; y++)
            for (int x = 0; x < ws[t - 1]; x++)
                for (int i = 0; i < L; i++)
                    data[t][((size_t)(y / 2) * ws[t] + x / 2) * L_ + i] +=
                        data[t - 1][((size_t)y * ws[t - 1] + x) * L_ + i];
    }
    const double scale = V[L], trunc = V[L_ * (L - 1)];
    double *prev = NULL;
    int32_t *stale = NULL;
    for (int t = levels - 1; t >= 0; t--) {
        const int w = ws[t], h = hs[t];
        double *m = (double *)calloc((size_t)w * h * 4 * L_, sizeof(double));
        if (t != levels - 1) {
            const int wp = ws[t + 1];
            for (int y = 0; y < h; y++)
                for (int x = 0; x < w; x++)
                    memcpy(&m[((size_t)y * w + x) * 4 * L_],
                           &prev[((size_t)(y / 2) * wp + x / 2) * 4 * L_], sizeof(double) * 4 * L_);
            free(prev);
            free(data[t + 1]);
            data[t + 1] = NULL;
        }
        if (t == 0) stale = (int32_t *)calloc((size_t)w * h, sizeof(int32_t));
        const double *dt = data[t];
        for (int it = 0; it < iters; it++) {
#pragma omp parallel
            {
                double *from = (double *)malloc(sizeof(double) * L_);
                double *hb = (double *)malloc(sizeof(double) * L_);
                double *buf = (double *)malloc(sizeof(double) * L_);
                double *z = (double *)malloc(sizeof(double) * (L_ + 1));
                int *v = (int *)malloc(sizeof(int) * L_);
#pragma omp for schedule(static)
                for (int y = 1; y < h - 1; y++) {
                    for (int x = ((y + it) & 1) + 1; x < w - 1; x += 2) {
                        const size_t p = (size_t)y * w + x;
                        for (int i = 0; i < L; i++) {
                            from[i] = dt[p * L_ + i];
                            for (int d = 0; d < 4; d++) {
                                const size_t q = (size_t)(y + ORC_DY[d]) * w + (x + ORC_DX[d]);
                                from[i] += m[(q * 4 + ORC_OPP(d)) * L_ + i];
                            }
                        }
                        if (t == 0) {
                            double best = from[0];
                            int bl = 0;
                            for (int i = 1; i < L; i++)
                                if (from[i] < best) { best = from[i]; bl = i; }
                            stale[p] = bl;
                        }
                        for (int d = 0; d < 4; d++) {
                            const size_t q = (size_t)(y + ORC_DY[d]) * w + (x + ORC_DX[d]);
                            std_send_f64(L, model, V, from, &m[(q * 4 + ORC_OPP(d)) * L_], scale, trunc,
                                         norm, hb, buf, v, z);
                            memcpy(&m[(p * 4 + d) * L_], buf, sizeof(double) * L_);
                        }
                    }
                }
                free(from);
                free(hb);
                free(buf);
                free(z);
                free(v);
            }
        }
        prev = m;
    }
    for (int y = 1; y < H - 1; y++) {
        for (int x = 1; x < W - 1; x++) {
            const size_t p = (size_t)y * W + x;
            if (decode == 1) {
                double best = 0;
                int bl = 0;
                for (int i = 0; i < L; i++) {
                    double c = data[0][p * L_ + i];
                    for (int d = 0; d < 4; d++) {
                        const size_t q = (size_t)(y + ORC_DY[d]) * W + (x + ORC_DX[d]);
                        c += prev[(q * 4 + ORC_OPP(d)) * L_ + i];
                    }
                    if (i == 0 || c < best) { best = c; bl = i; }
                }
                labels[p] = bl;
            } else {
                labels[p] = stale[p];
            }
        }
    }
    if (msgs_out) {
        for (int y = 0; y < H; y++)
            for (int x = 0; x < W; x++)
                for (int d = 0; d < 4; d++) {
                    double *dst = &msgs_out[(((size_t)y * W + x) * 4 + d) * L_];
                    const int nx = x + ORC_DX[d], ny = y + ORC_DY[d];
                    if (nx < 0 || ny < 0 || nx >= W || ny >= H) memset(dst, 0, sizeof(double) * L_);
                    else memcpy(dst, &prev[(((size_t)ny * W + nx) * 4 + ORC_OPP(d)) * L_], sizeof(double) * L_);
                }
    }
    free(prev);
    free(stale);
    free(data[0]);
    free(data);
    free(ws);
    free(hs);
    free(V);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Alpha-beta swap by push-relabel max-flow, src/graphcut.cc:9-279 (int      */
/* grids only, graphcut.cc:281).  Restated statement by statement in the     */
/* reference's order, including what it carries from one label pair to the  */
/* next: nodes outside the alpha-beta partition keep the excess, height and  */
/* residues their last pair left (graphCutConstructGraph, :10-45, rewrites   */
/* only partition nodes), and those still take part in the active count, the */
/* relabels, the pushes and the reachability.  Residues per node: the four   */
/* directions, then the source slot (never used) and the sink slot,          */
/* slot-major (s * N + node) as the reference's Matrix(3, W, H, 6).          */

#define GC_SINK 5
#define GC_ITERS_PER_RELABEL 10 /* GINF_GRAPHCUT_NUM_ITERS_PER_GLOBAL_RELABEL, graphcut.h:8 */

static int gc_valid(int x, int y, int W, int H) { return x >= 0 && y >= 0 && x < W && y < H; }

/* graphCutConstructGraph, graphcut.cc:10-45 (residue plays the capacity). */
static void gc_construct(int W, int H, int L, const int32_t *D, const int32_t *V, const int32_t *f,
                         int32_t *height, int32_t *excess, int32_t *res, int alpha, int beta)
{
    const size_t N = (size_t)W * H;
    for (int y = 0; y < H; y++)
        for (int x = 0; x < W; x++) {
            const size_t p = (size_t)y * W + x;
            if (f[p] != alpha && f[p] != beta) continue;
            int32_t ac = 0, bc = 0;
            for (int d = 0; d < 4; d++) {
                const int nx = x + ORC_DX[d], ny = y + ORC_DY[d];
                if (gc_valid(nx, ny, W, H)) {
                    const int fn = f[(size_t)ny * W + nx];
                    if (fn == alpha || fn == beta) {
                        res[d * N + p] = V[alpha + (size_t)L * beta];
                    } else {
                        res[d * N + p] = 0;
                        ac += V[alpha + (size_t)L * fn];
                        bc += V[beta + (size_t)L * fn];
                    }
                } else {
                    res[d * N + p] = 0;
                }
            }
            excess[p] = D[p + N * (size_t)alpha] + ac;
            res[GC_SINK * N + p] = D[p + N * (size_t)beta] + bc;
            height[p] = 0;
        }
}

/* graphCutGlobalRelabel, graphcut.cc:91-140: breadth-first distances to the
 * sink over residual edges (a FIFO from the sink-adjacent nodes in raster
 * order); unreachable nodes get max(height, N + 2). */
static void gc_global_relabel(int W, int H, int32_t *height, const int32_t *res, int32_t *h, int32_t *queue)
{
    const size_t N = (size_t)W * H;
    size_t head = 0, tail = 0;
    for (size_t p = 0; p < N; p++) {
        h[p] = 0;
        if (res[GC_SINK * N + p]) {
            h[p] = 1;
            queue[tail++] = (int32_t)p;
        }
    }
    while (head < tail) {
        const int32_t p = queue[head++];
        const int x = p % W, y = p / W;
        for (int d = 0; d < 4; d++) {
            const int nx = x + ORC_DX[d], ny = y + ORC_DY[d];
            if (!gc_valid(nx, ny, W, H)) continue;
            const size_t q = (size_t)ny * W + nx;
            if (res[ORC_OPP(d) * N + q] && h[q] == 0) {
                h[q] = h[p] + 1;
                queue[tail++] = (int32_t)q;
            }
        }
    }
    for (size_t p = 0; p < N; p++) {
        if (h[p] == 0) h[p] = height[p] > (int32_t)N + 2 ? height[p] : (int32_t)N + 2;
        height[p] = h[p];
    }
}

/* graphCutPush / graphCutPushToPixel, graphcut.cc:143-177. */
static void gc_push(int W, int H, const int32_t *height, int32_t *excess, int32_t *res, int x, int y)
{
    const size_t N = (size_t)W * H, p = (size_t)y * W + x;
    if (!(excess[p] && height[p] < (int32_t)N + 2)) return;
    if (res[GC_SINK * N + p] && height[p] == 1) {
        const int32_t flow = ORC_MIN(res[GC_SINK * N + p], excess[p]);
        excess[p] -= flow;
        res[GC_SINK * N + p] -= flow;
    }
    for (int d = 0; d < 4; d++) {
        if (res[d * N + p] && height[p] == height[(size_t)(y + ORC_DY[d]) * W + x + ORC_DX[d]] + 1) {
            const size_t q = (size_t)(y + ORC_DY[d]) * W + x + ORC_DX[d];
            const int32_t flow = ORC_MIN(res[d * N + p], excess[p]);
            excess[p] -= flow;
            excess[q] += flow;
            res[d * N + p] -= flow;
            res[ORC_OPP(d) * N + q] += flow;
        }
    }
}

/* graphCutRelabel, graphcut.cc:180-195. */
static void gc_relabel(int W, int H, int32_t *height, const int32_t *excess, const int32_t *res, int x, int y)
{
    const size_t N = (size_t)W * H, p = (size_t)y * W + x;
    if (!(excess[p] && height[p] < (int32_t)N + 2)) return;
    if (res[GC_SINK * N + p]) {
        height[p] = 1;
    } else {
        int32_t mh = (int32_t)N + 2;
        for (int d = 0; d < 4; d++)
            if (res[d * N + p]) mh = ORC_MIN(mh, height[(size_t)(y + ORC_DY[d]) * W + x + ORC_DX[d]]);
        height[p] = mh + 1;
    }
}

/* graphCutFindReachable from every node with sink residue, graphcut.cc:47-58
 * and :253-260 (a recursive depth-first search there; the set it marks --
 * the nodes that reach the sink over residual edges -- is the same for an
 * explicit stack). */
static void gc_reachable(int W, int H, const int32_t *res, int32_t *reach, int32_t *stack)
{
    const size_t N = (size_t)W * H;
    memset(reach, 0, sizeof(int32_t) * N);
    size_t top = 0;
    for (size_t s = 0; s < N; s++) {
        if (!res[GC_SINK * N + s] || reach[s]) continue;
        reach[s] = 1;
        stack[top++] = (int32_t)s;
        while (top) {
            const int32_t p = stack[--top];
            const int x = p % W, y = p / W;
            for (int d = 0; d < 4; d++) {
                const int nx = x + ORC_DX[d], ny = y + ORC_DY[d];
                if (!gc_valid(nx, ny, W, H)) continue;
                const size_t q = (size_t)ny * W + nx;
                if (res[ORC_OPP(d) * N + q] && !reach[q]) {
                    reach[q] = 1;
                    stack[top++] = (int32_t)q;
                }
            }
        }
    }
}

int orc_alpha_beta_i32(int W, int H, int L, const int32_t *D, const int32_t *V, const int32_t *initial, int iters,
                       int32_t *result)
{
    if (W < 1 || H < 1 || L < 1 || iters < 0) return -1;
    const size_t N = (size_t)W * H;
    int32_t *excess = calloc(N, sizeof(int32_t)), *height = calloc(N, sizeof(int32_t));
    int32_t *res = calloc(N * 6, sizeof(int32_t)), *reach = calloc(N, sizeof(int32_t));
    int32_t *newr = malloc(N * sizeof(int32_t)), *h = malloc(N * sizeof(int32_t));
    int32_t *queue = malloc(N * sizeof(int32_t)), *stack = malloc(N * sizeof(int32_t));
    if (!excess || !height || !res || !reach || !newr || !h || !queue || !stack) return -1;
    memcpy(result, initial, N * sizeof(int32_t));
    memcpy(newr, initial, N * sizeof(int32_t));
    int32_t min_cost = orc_energy_i32_seq(W, H, L, D, V, result);
    int success = 1;
    for (int t = 0; t < iters && success; t++) {
        success = 0;
        for (int alpha = 0; alpha < L; alpha++)
            for (int beta = alpha + 1; beta < L; beta++) {
                gc_construct(W, H, L, D, V, result, height, excess, res, alpha, beta);
                for (;;) {
                    size_t active = 0;
                    for (size_t p = 0; p < N; p++)
                        if (excess[p] && height[p] < (int32_t)N + 2) active++;
                    if (active == 0) break;
                    gc_global_relabel(W, H, height, res, h, queue);
                    for (int i = 0; i < GC_ITERS_PER_RELABEL; i++) {
                        for (int y = 0; y < H; y++)
                            for (int x = 0; x < W; x++) gc_push(W, H, height, excess, res, x, y);
                        for (int y = 0; y < H; y++)
                            for (int x = 0; x < W; x++) gc_relabel(W, H, height, excess, res, x, y);
                    }
                }
                gc_reachable(W, H, res, reach, stack);
                for (size_t p = 0; p < N; p++)          /* graphCutLabelFromFlow, :60-72 */
                    if (newr[p] == alpha || newr[p] == beta) newr[p] = reach[p] ? alpha : beta;
                const int32_t cost = orc_energy_i32_seq(W, H, L, D, V, newr);
                if (cost < min_cost) {
                    min_cost = cost;
                    memcpy(result, newr, N * sizeof(int32_t));
                    success = 1;
                } else {
                    memcpy(newr, result, N * sizeof(int32_t));
                }
            }
    }
    free(excess); free(height); free(res); free(reach); free(newr); free(h); free(queue); free(stack);
    return 0;
}
