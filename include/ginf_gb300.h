/*
 * ginf_gb300.h -- C ABI of the GB300 (sm_103a) grid-MRF inference library.
 *
 * This is the drop-in boundary for GridInfCuda's inference path.  The C++
 * entry points of the reference (namespace ginf: decodeBp / decodeHbp /
 * gpuDecodeBp / gpuDecodeHbp, decodeIcmSync / decodeIcmAsync / gpuDecodeIcm,
 * Grid<T>::getLabelingCost) are re-implemented on top of these functions in
 * include/ginf/*.h; other hosts (Python ctypes, cgo, JNI ...) bind them
 * directly.  Plain pointers and sizes only, no exceptions across the ABI,
 * every function returns a status and never exits the process (the
 * reference's GINF_SAFE_CALL exits, src/include/gpu.h:36-48).
 *
 * Data layouts are the reference's Matrix layouts (src/matrix.cc:52-56,
 * first index fastest):
 *   data costs   label-planar, element (x, y, l) at x + W*y + W*H*l
 *   smoothness   L x L table, V(fp, fq) at fp + L*fq            (grid.h:22-23)
 *   labels       int32, (x, y) at x + W*y                       (Matrix(2, W, H))
 * Directions are S=0 (+y), E=1 (+x), N=2 (-y), W=3 (-x)         (utils.h:26-37)
 */
#ifndef GINF_GB300_H
#define GINF_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum ginf_status {
    GINF_OK = 0,
    GINF_ERR_INVALID_ARGUMENT = 1, /* bad size, null pointer, unknown enum   */
    GINF_ERR_UNSUPPORTED = 2,      /* valid request this build does not cover */
    GINF_ERR_CUDA = 3,             /* a CUDA runtime call or launch failed     */
    GINF_ERR_OUT_OF_MEMORY = 4,    /* device or pinned allocation failed       */
    GINF_ERR_TIMEOUT = 5,          /* a bounded device-side wait gave up       */
    GINF_ERR_NO_DEVICE = 6         /* no usable sm_103 device                  */
} ginf_status;

/* Smoothness models, same numbering as ginf::SmoothnessFunctions (grid.h:9-14). */
enum { GINF_SM_EXPLICIT = 0, GINF_SM_POTTS = 1, GINF_SM_TRUNC_LINEAR = 2, GINF_SM_TRUNC_QUAD = 3 };
/* Cost / message arithmetic type: the reference's float and int instantiations
 * (bp.cc:190-194), plus double for the FP64 oracle runs. */
enum { GINF_F32 = 0, GINF_I32 = 1, GINF_F64 = 2 };
/* Where the caller's buffers live. */
enum { GINF_HOST = 0, GINF_DEVICE = 1 };
/* Message rule.  REFERENCE reproduces src/bp.cc:21-63 exactly, including its
 * O(L^2) branch for EXPLICIT and TRUNC_QUAD that neither subtracts the
 * receiver's message nor normalises (bp.cc:55-62).  STANDARD is min-sum BP for
 * every model: subtract, distance transform (O(L) lower envelope for
 * TRUNC_QUAD), truncate, normalise.  The two agree for POTTS and TRUNC_LINEAR. */
enum { GINF_RULE_REFERENCE = 0, GINF_RULE_STANDARD = 1 };
/* Message store: the arithmetic type, or FP16 (F32 grids only; the update
 * still runs in FP32 and messages are min-normalised so they land in
 * [0, truncation]). */
enum { GINF_STORE_NATIVE = 0, GINF_STORE_F16 = 1 };
/* Final decode: STALE is the reference's argmin of each node's belief at its
 * last update (bp.cc:65-84, 168-173); FRESH recomputes beliefs from the final
 * messages. */
enum { GINF_DECODE_STALE = 0, GINF_DECODE_FRESH = 1 };
/* How host-resident costs reach the device (ginf_options.host_access). */
enum { GINF_HOST_AUTO = 0, GINF_HOST_COPY = 1 };
/* Message normalisation: subtract the mean (bp.cc:50-54) or the minimum. */
enum { GINF_NORM_MEAN = 0, GINF_NORM_MIN = 1 };

/* One grid MRF (the reference's ginf::Grid<T>, grid.h:16-81). */
typedef struct ginf_grid {
    int32_t width, height, num_labels;
    int32_t cost_type;       /* GINF_F32 or GINF_I32 (costs are read as this type) */
    int32_t sm_model;        /* GINF_SM_*                                         */
    int32_t memory;          /* GINF_HOST or GINF_DEVICE, for every buffer below   */
    const void *data_costs;  /* W*H*L elements, label-planar                      */
    const void *sm_costs;    /* L*L elements, V(fp, fq) at fp + L*fq              */
} ginf_grid;

typedef struct ginf_options {
    int32_t msg_rule;        /* GINF_RULE_*,   default REFERENCE            */
    int32_t msg_store;       /* GINF_STORE_*,  default NATIVE               */
    int32_t decode;          /* GINF_DECODE_*, default STALE                */
    int32_t normalize;       /* GINF_NORM_*,   default MEAN (F16 uses MIN)  */
    int32_t compute_type;    /* GINF_F32 / GINF_I32 / GINF_F64; -1 = cost_type */
    int32_t tile_nodes;      /* nodes per sweep tile (8, 16 or 32); 0 = default
                                (16), or the autotuned choice for batches        */
    int32_t sweeps_per_launch; /* batches: half-sweeps per persistent launch;
                                  0 = autotuned.  Single grids: 0 or 1 = one
                                  half-sweep per launch (default); k >= 2 =
                                  temporal blocking on FP32 grids with
                                  L <= 32 and the Potts / truncated-linear
                                  update: up to k half-sweeps per launch on
                                  thread-block clusters, the same results bit
                                  for bit (slower than one per launch on
                                  GB300 at these label counts, where the
                                  update is latency-bound, not HBM-bound)   */
    int32_t autotune;        /* batches: 0 = cached choice, else measure and cache;
                                1 = always measure; -1 = never (defaults)        */
    void *stream;            /* cudaStream_t to run on; NULL = legacy default */
    void *msgs_out;          /* optional: final level-0 messages, [H][W][4][L] of the
                                compute type, slot d = message from the neighbour in
                                direction d (0 where that neighbour is on the border
                                or off the grid); same memory kind as the grid     */
    int32_t host_access;     /* GINF_HOST grids: GINF_HOST_AUTO (default) lets the
                                device read the caller's costs in place when CUDA
                                reports them device-accessible (pinned memory, or
                                pageable memory on systems with pageable access),
                                fusing the transfer into the layout transform;
                                GINF_HOST_COPY always stages them by a copy      */
    int32_t stream_ordered;  /* ginf_decode_hbp / ginf_solve: 1 = stream-ordered.
                                The call enqueues its work on `stream` and returns;
                                host outputs (labels, energy) are valid once the
                                stream or ginf_workspace_sync(ws) has finished, and
                                the caller's host buffers must stay alive and
                                unchanged until then.  Needs a caller-owned
                                workspace and stats == NULL.  A device-side error
                                is reported by ginf_workspace_sync or by the next
                                call on the workspace.  Other calls ignore it.     */
    int64_t reserved[5];
} ginf_options;

/* Per-call measurements (filled when a non-null pointer is passed; the call
 * then synchronises its stream before returning). */
typedef struct ginf_stats {
    double total_ms;          /* whole call, device timeline                   */
    double upload_ms;         /* host->device copy of costs (host grids)        */
    double prepare_ms;        /* layout transform + pyramid                    */
    double sweep_ms;          /* all BP half-sweeps, all levels                */
    double level0_sweep_ms;   /* BP half-sweeps of the finest level            */
    double icm_ms;            /* ICM sweeps                                    */
    double energy_ms;         /* energy reduction                              */
    double download_ms;       /* device->host copy of results                  */
    int64_t kernel_launches;  /* kernels this call launched                    */
    int64_t level0_sweep_launches;
    int64_t node_label_iters; /* sum over levels of W_t*H_t*L*iterations       */
    int64_t h2d_bytes, d2h_bytes;
    int64_t warm_start_used;  /* learned solve: 1 = warm start kept, 0 = fell back */
    int64_t level0_alg_bytes; /* HBM bytes the finest level's sweep launches must move by
                                 their design (the roofline numerator)             */
} ginf_stats;

typedef struct ginf_workspace ginf_workspace;

/* Library information and errors. */
const char *ginf_version(void);
/* Message of the last failing call on this host thread ("" if none). */
const char *ginf_last_error(void);
void ginf_default_options(ginf_options *opt);

/* Reusable device buffers and events; one per host thread or stream.  A
 * workspace belongs to the device that is current at its first call; calls
 * from another device return GINF_ERR_INVALID_ARGUMENT.  Passing NULL to the
 * solver entry points allocates and frees per call, as the reference does
 * (src/gpu/bp.cu:141-222). */
ginf_status ginf_workspace_create(ginf_workspace **ws);
ginf_status ginf_workspace_destroy(ginf_workspace *ws);
/* Waits for the workspace's stream-ordered calls and reports a device-side
 * error any of them recorded. */
ginf_status ginf_workspace_sync(ginf_workspace *ws);

/* Hierarchical min-sum BP, num_levels == 1 being loopy BP.
 * Replaces ginf::decodeHbp (src/bp.cc:86-180), ginf::decodeBp (bp.cc:182-187),
 * ginf::gpuDecodeHbp (src/gpu/bp.cu:133-223) and ginf::gpuDecodeBp
 * (bp.cu:228-231), with the CPU code's semantics.  labels is W*H int32 in the
 * grid's memory kind; interior entries are written, border entries are left
 * as the caller set them (bp.cc:169-173). */
ginf_status ginf_decode_hbp(ginf_workspace *ws, const ginf_grid *grid, int32_t num_levels,
                            int32_t iters_per_level, int32_t *labels, const ginf_options *opt,
                            ginf_stats *stats);

/* ICM.  asynchronous == 0: Jacobi sweeps, replacing ginf::decodeIcmSync
 * (src/icm.cc:4-38) and ginf::gpuDecodeIcm (src/gpu/icm.cu:53-83).
 * asynchronous == 1: raster-order Gauss-Seidel, replacing ginf::decodeIcmAsync
 * (src/icm.cc:40-67), run as an exact anti-diagonal wavefront.
 * result (W*H) receives a copy of initial, then interior nodes are updated. */
ginf_status ginf_decode_icm(ginf_workspace *ws, const ginf_grid *grid, const int32_t *initial,
                            int32_t iters, int32_t asynchronous, int32_t *result,
                            const ginf_options *opt, ginf_stats *stats);

/* Alpha-beta swap, replacing ginf::decodeAlphaBeta (src/graphcut.cc:197-279)
 * and ginf::gpuDecodeAlphaBeta (src/include/graphcut.h:24-25; its GPU source
 * src/gpu/graphcut.cu does not compile): for up to `iters` passes over every
 * label pair alpha < beta, the min cut of the pair's graph by push-relabel,
 * the swap kept when it lowers the energy; stops after a pass without a
 * change.  int32 grids only (the reference instantiates it for int,
 * graphcut.cc:281).  The results are the reference's bit for bit, including
 * its raster-order pushes and relabels and the state it keeps across label
 * pairs.  result (W*H) receives a copy of initial, then the swaps.  One CTA
 * runs the whole solve; a solve that runs longer than 60 s on the device
 * returns GINF_ERR_TIMEOUT. */
ginf_status ginf_decode_alpha_beta(ginf_workspace *ws, const ginf_grid *grid, const int32_t *initial,
                                   int32_t iters, int32_t *result, const ginf_options *opt, ginf_stats *stats);

/* Energy of a labelling, ginf::Grid<T>::getLabelingCost(Matrix<int>*)
 * (src/grid.cc:102-125): interior nodes' data terms plus their N and E edges,
 * summed in FP64 on the device (deterministic order). */
ginf_status ginf_energy(ginf_workspace *ws, const ginf_grid *grid, const int32_t *labels,
                        double *energy, const ginf_options *opt);

/* HBP, then ICM refinement, then the FP64 energy, with one upload of the
 * costs: decodeHbp (bp.cc:86-180) + decodeIcmSync (icm.cc:4-38) +
 * getLabelingCost (grid.cc:102-125) in one call.  labels receives the refined
 * labelling (border entries keep the caller's values), energy may be NULL. */
ginf_status ginf_solve(ginf_workspace *ws, const ginf_grid *grid, int32_t num_levels,
                       int32_t iters_per_level, int32_t icm_iters, int32_t *labels, double *energy,
                       const ginf_options *opt, ginf_stats *stats);

/* Stereo data costs on the device: D(x, y, d) = coef * min(|left(x,y) -
 * right(max(x-d, 0), y)|, cap) for d < L, label-planar float32 into costs
 * (device memory, W*H*L).  left / right are W*H float32 images in the memory
 * kind given.  The GPU form of the cost loop in
 * examples/stereo/stereo.cc:28-34 (with x-d clamped at 0 instead of zero-cost
 * columns). */
ginf_status ginf_stereo_costs(int32_t width, int32_t height, int32_t num_labels, int32_t memory,
                              const float *left, const float *right, float coef, float cap,
                              float *costs, void *stream);

/* Stereo data costs by the reference example's own integer recipe
 * (examples/stereo/stereo.cc:28-34), on the device: for every column
 * x >= L-1, D(x, y, k) = min(|left(x,y) - right(x-k,y)|, cap) for k < L;
 * columns x < L-1 get zero cost, as the reference's zero-initialised grid
 * leaves them.  left / right are W*H 8-bit grey images (the example's
 * CV_LOAD_IMAGE_GRAYSCALE matrices) in the memory kind given; costs is
 * int32, label-planar, device memory (W*H*L), ready for a GINF_I32 grid.
 * The example uses L = 16 and cap = 20, then TruncLinear(10, 20) and 30
 * iterations of gpuDecodeBp. */
ginf_status ginf_stereo_costs_u8(int32_t width, int32_t height, int32_t num_labels, int32_t memory,
                                 const uint8_t *left, const uint8_t *right, int32_t cap, int32_t *costs,
                                 void *stream);

/* Batches: many independent grids, each solved by loopy BP (one level,
 * `iters` half-sweeps, the reference's semantics and stale-belief decode, as
 * ginf_decode_hbp with num_levels == 1).  The reference solves one grid per
 * call (src/include/bp.h:14-26); a batch solves them together in one
 * persistent cooperative launch per label group and `sweeps_per_launch`
 * half-sweeps, walking a work list of (grid, tile) entries, and replays the
 * whole solve from a CUDA graph captured at creation.  Grids: FP32 costs, Potts or
 * truncated-linear smoothness, 2 <= L <= 64, all buffers device memory; the
 * plan keeps the pointers, so later runs see whatever those buffers hold.
 * The tile size and half-sweeps per launch are given in `opt` or chosen by
 * the autotuner, which times the candidates on this batch and caches the
 * winner per mix of (label count, log2 node count) buckets in the JSON file
 * named by $GINF_AUTOTUNE_CACHE (default
 * $XDG_CACHE_HOME or ~/.cache/gridinfcuda_gb300_autotune.json).  A plan
 * runs only on the device current at its creation; runs from another device
 * return GINF_ERR_INVALID_ARGUMENT. */
typedef struct ginf_batch ginf_batch;
ginf_status ginf_batch_create(ginf_batch **batch, const ginf_grid *grids, int32_t *const *labels, int32_t count,
                              int32_t iters, const ginf_options *opt);
/* Replays the captured solve on `stream` (cudaStream_t) and waits for it. */
ginf_status ginf_batch_run(ginf_batch *batch, void *stream, ginf_stats *stats);
/* Stream-ordered replay: enqueues the captured solve on `stream` and returns.
 * Labels are valid once the stream (or ginf_batch_sync) has finished; a
 * batch's replays must not overlap one another (one stream, or a sync in
 * between).  A device-side error is reported by ginf_batch_sync or by the
 * next replay of the batch. */
ginf_status ginf_batch_enqueue(ginf_batch *batch, void *stream);
/* Waits for the batch's stream-ordered replays and reports a device-side
 * error any of them recorded. */
ginf_status ginf_batch_sync(ginf_batch *batch);
/* The tile size and half-sweeps per launch in use, and whether this plan
 * measured them (1) or took them from the options or the cache (0). */
ginf_status ginf_batch_config(const ginf_batch *batch, int32_t *tile_nodes, int32_t *sweeps_per_launch,
                              int32_t *tuned_now);
ginf_status ginf_batch_destroy(ginf_batch *batch);
/* Create, run once, destroy. */
ginf_status ginf_decode_bp_batch(const ginf_grid *grids, int32_t *const *labels, int32_t count, int32_t iters,
                                 const ginf_options *opt, ginf_stats *stats);

/* Learned warm start for hierarchical BP (new here: the reference has no
 * learned component).  A small BF16 convolutional network (3x3 convs,
 * L -> 32 -> 32 -> 32 -> L, ReLU, FP32 accumulate, tensor-core kernels) maps
 * the costs of pyramid level t, x = D_t / 4^t, to y = x + net(x) ~
 * (D_t + m) / 4^t, m being the sum of the messages the level's nodes should
 * start from: the converged finest-level messages averaged per block (or
 * the level's own beliefs; ginf_hbp_level_state produces either target).
 * Device buffers are FP32, [n][h][w][L]. */
typedef struct ginf_warmnet ginf_warmnet;
ginf_status ginf_warmnet_create(ginf_warmnet **net, int32_t num_labels, int32_t hidden, uint64_t seed);
/* Checkpoints hold the weights and the Adam state, with a checksum. */
ginf_status ginf_warmnet_load(ginf_warmnet **net, const char *path);
ginf_status ginf_warmnet_save(const ginf_warmnet *net, const char *path);
ginf_status ginf_warmnet_destroy(ginf_warmnet *net);
ginf_status ginf_warmnet_num_params(const ginf_warmnet *net, int64_t *count);
/* FP32 parameters, per layer the weights [cout][3][3][cin] then the biases. */
ginf_status ginf_warmnet_get_params(const ginf_warmnet *net, float *host);
ginf_status ginf_warmnet_set_params(ginf_warmnet *net, const float *host);
/* y = x + net(x).  x, y 16-byte aligned (GINF_ERR_CUDA otherwise); y may be x.
 * The convolutions run on tcgen05 with tensor-memory accumulators. */
ginf_status ginf_warmnet_forward(ginf_warmnet *net, const float *x, int32_t n, int32_t h, int32_t w, float *y,
                                 void *stream);
/* Mean-squared-error loss against target and the gradient of every
 * parameter (same order as get_params), without an update. */
ginf_status ginf_warmnet_gradients(ginf_warmnet *net, const float *x, const float *target, int32_t n, int32_t h,
                                   int32_t w, float *loss, float *grads_host, void *stream);
/* One Adam step (beta 0.9 / 0.999) on the mean-squared-error loss. */
ginf_status ginf_warmnet_train_step(ginf_warmnet *net, const float *x, const float *target, int32_t n, int32_t h,
                                    int32_t w, float lr, float *loss, void *stream);
/* Training data from this library's own BP: the network input of pyramid
 * level `level` (x = D_t / 4^t) and, when beliefs_out is given, a target:
 * target 0 = the level's beliefs / 4^t after hierarchical BP from the top of
 * a num_levels pyramid down to that level; target 1 = (D_t + m) / 4^t after
 * the whole schedule down to level 0, m being the mean over the node's
 * 2^t x 2^t fine block of the level-0 incoming-message sums.  Device buffers
 * [H_t][W_t][L]. */
ginf_status ginf_hbp_level_state(ginf_workspace *ws, const ginf_grid *grid, int32_t num_levels,
                                 int32_t iters_per_level, int32_t level, int32_t target, float *x_out,
                                 float *beliefs_out, const ginf_options *opt);
/* Hierarchical BP warm-started at level warm_level (1 <= warm_level <=
 * num_levels - 2): the network reads that level's costs (x = D_t / 4^t) and
 * its prediction y sets the level's messages (each incoming slot = 4^t/4 *
 * (y - x)); warm_iters half-sweeps run there (0: the messages go down
 * unchanged), levels warm_level-1 .. 1 run mid_iters (< 0: iters_per_level)
 * and level 0 iters_per_level, as in ginf_decode_hbp.
 * Fallback: the cold schedule first runs its levels down to warm_level+1
 * (the cheap ones); when the seeded result has a higher level-0 energy than
 * that level's labelling handed down to level 0, the seeded result is
 * discarded and the cold schedule resumes, giving exactly ginf_decode_hbp's
 * labels (stats->warm_start_used tells which). */
ginf_status ginf_decode_hbp_learned(ginf_workspace *ws, const ginf_grid *grid, int32_t num_levels,
                                    int32_t iters_per_level, int32_t warm_level, int32_t warm_iters,
                                    int32_t mid_iters, ginf_warmnet *net, int32_t *labels,
                                    const ginf_options *opt, ginf_stats *stats);

/* As ginf_decode_hbp_learned with the prediction supplied by the caller: a
 * device buffer [H_t][W_t][L] on the network's output scale (x = D_t / 4^t
 * plus the predicted message sum / 4^t).  Levels warm_level-1 .. 1 run
 * mid_iters half-sweeps (< 0: iters_per_level), level 0 iters_per_level.
 * fallback = 0 always keeps the seeded result (no cold pass; warm_level may
 * then be num_levels - 1). */
ginf_status ginf_decode_hbp_warm(ginf_workspace *ws, const ginf_grid *grid, int32_t num_levels,
                                 int32_t iters_per_level, int32_t warm_level, int32_t warm_iters,
                                 int32_t mid_iters, const float *prediction, int32_t fallback, int32_t *labels,
                                 const ginf_options *opt, ginf_stats *stats);

/* Loopy BP (one level, the reference message rule and stale-belief decode)
 * that allocates no device memory.  It has no counterpart in the reference.
 * It is meant for callers that cannot call cudaMalloc while they run: a
 * real-time loop that cannot afford the device-wide synchronisation and
 * unbounded latency of cudaMalloc / cudaFree, or a plugin whose host
 * application owns all device memory.  The caller passes device buffers
 * (grid->memory must be GINF_DEVICE) and device labels, as for
 * ginf_decode_hbp; the working set (the message records and a status word)
 * lives in one fixed array of GINF_NOALLOC_SCRATCH_BYTES in the library's
 * device image, which every GPU that loads the library holds until the
 * process exits.  A W x H grid with L labels needs exactly
 *     256 + W * H * 20 * Lp  bytes,   Lp = L rounded up to a multiple of 8
 * (one record of 5 * Lp four-byte elements per node -- its costs and four
 * incoming messages -- after a 256-byte status block), for FP32 and int32
 * alike; grids needing more than GINF_NOALLOC_SCRATCH_BYTES are rejected with
 * GINF_ERR_INVALID_ARGUMENT and nothing runs.  The first call on a device
 * looks up the array's device address (cudaGetSymbolAddress) with that device
 * current and keeps it for the process; make that first call before any
 * stream capture, and do not call cudaDeviceReset on that device afterwards
 * (a new context may place the array elsewhere).  All calls share the array:
 * calls whose work overlaps on the GPU race and must be serialised by the
 * caller.  The call synchronises `stream` (a cudaStream_t, NULL = legacy
 * default stream) before it returns. */
#define GINF_NOALLOC_SCRATCH_BYTES (48u * 1024u * 1024u)
ginf_status ginf_decode_bp_noalloc(const ginf_grid *grid, int32_t num_iters, int32_t *labels, void *stream);

/* Diagnostic (new here): runs the library's bounded device-side waits into
 * their time limit on purpose -- an mbarrier phase nothing completes and a
 * grid barrier one block short -- and returns the status words they recorded
 * (GINF_DEVICE_TIMEOUT expected in both).  Each wait gives up after about two
 * seconds and its kernel ends normally; the device stays usable. */
#define GINF_DEVICE_TIMEOUT 1
ginf_status ginf_selftest_bounded_waits(int32_t *mbarrier_status, int32_t *barrier_status);

#ifdef __cplusplus
}
#endif
#endif /* GINF_GB300_H */
