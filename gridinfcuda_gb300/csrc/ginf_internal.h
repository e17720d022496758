// ginf_internal.h -- host/device shared declarations of the GB300 library.
//
// HBM layout of one pyramid level ("records"): node (x, y) owns the record at
// rec + (y*W + x) * rec_bytes, label-contiguous:
//
//     [ D: Lp elements of the compute type T ][ in[0..3]: 4 x Lp elements of the store type M ]
//
// in[d] is the message sent TO the node BY its neighbour in direction d
// (S=0, E=1, N=2, W=3), i.e. messages are stored at the receiver.  A node's
// whole update input (its costs and its four incoming messages) is one
// contiguous, 16-byte aligned block that a single bulk TMA copy brings into
// shared memory, and each of its four outputs is one contiguous Lp-element
// slot of a neighbour's record.  Lp is L rounded up to a multiple of 8, so
// every slot is a whole number of 16-byte chunks for f16, f32, i32 and f64.
#pragma once

#include <atomic>
#include <cstddef>
#include <cstdint>
#include <mutex>

#include <cuda_runtime.h>

namespace ginf_gpu {

enum CType { CT_F32 = 0, CT_I32 = 1, CT_F64 = 2 };
enum Store { ST_NATIVE = 0, ST_F16 = 1 };
enum ReadMode { RD_OWN = 0, RD_ZERO = 1, RD_COARSE = 2 };
enum Mode { MODE_LINEAR = 0, MODE_REF_MINCONV = 1, MODE_STD_MINCONV = 2, MODE_STD_QUAD = 3 };

// Device status bits (OR-ed into the workspace's status word).
enum { DEV_ERR_TIMEOUT = 1, DEV_ERR_BOUNDS = 2 };

struct LevelGeom {
    int W = 0, H = 0;
    size_t rec_bytes = 0;   // record stride
    size_t offset = 0;      // byte offset of this level inside the records buffer
};

struct RecordFormat {
    int ctype = CT_F32;     // arithmetic / cost element type in the record
    int store = ST_NATIVE;  // message element type
    int L = 0, Lp = 0;
    uint32_t t_size = 4, m_size = 4;
    uint32_t d_bytes = 0, m_bytes = 0, rec_bytes = 0, slot_bytes = 0;
};

RecordFormat make_format(int ctype, int store, int L);

// Parameters of one checkerboard half-sweep launch.
struct SweepParams {
    int W, H, L, Lp;
    uint32_t rec_bytes, d_bytes, m_bytes, slot_bytes;
    unsigned char *rec;            // this level's records
    const unsigned char *crec;     // coarser level's records (RD_COARSE)
    int cW, cH;
    int iter;                      // nodes with x >= ((y+iter)&1)+1, step 2, are updated
    int read_mode;                 // ReadMode
    int mode;                      // Mode
    int norm_min;                  // 0 = subtract mean, 1 = subtract min
    const void *V;                 // L*L table of the compute type (device); the
                                   // kernel reads its slope V(0,1) and truncation
                                   // V(0,L-1) from it, as bp.cc:35,43 do
    int32_t *labels;               // level-0 labels (W*H) or nullptr
    int write_labels;
    int tiles_per_row, num_tiles;  // set by the launcher for the variant it runs
    int quad_radius;               // truncation radius of a quadratic table (kernel choice only)
    int quad_exact;                // 1: V(0,k) = V(0,1) k^2 exactly up to that radius, V(0,0) = 0
    int *status;
};

// Parameters of one launch of the temporal-blocking kernel (several
// half-sweeps of one level, FP32 records, L <= 32; sweep_cluster.cu).
struct ClusterSweepParams {
    int W, H, L;
    uint32_t rec_bytes, d_bytes, m_bytes, slot_bytes;
    uint32_t from_stride;          // bytes per belief vector in shared memory (odd number of 16-byte chunks)
    const unsigned char *rec_in;   // records read (this level, one buffer) ...
    unsigned char *rec_out;        // ... and written (the other buffer)
    int iter0;                     // level half-sweep index of the launch's first half-sweep
    int k;                         // half-sweeps in this launch (also the halo depth)
    int label_from;                // half-sweeps with index >= label_from write labels (INT_MAX: none)
    int read_mode;                 // RD_OWN, or RD_ZERO (messages start at zero)
    int write_d;                   // 1: write whole records (rec_out lacks the costs), 0: messages only
    int norm_min;
    const void *V;
    int32_t *labels;
    int *status;
    int bw, bh;                    // sub-block of one CTA (set by the launcher)
};

// Launches of the temporal-blocking kernel; eligible formats: FP32
// arithmetic, native store, L <= 32.
cudaError_t launch_cluster_sweeps(const RecordFormat &f, const ClusterSweepParams &p, cudaStream_t s);
// Deepest halo (most half-sweeps per launch) the kernel's region allows.
int cluster_sweep_max_halo(int L);
inline bool cluster_sweep_eligible(const RecordFormat &f, int mode) {
    return f.ctype == CT_F32 && f.store == ST_NATIVE && mode == MODE_LINEAR && f.L <= 32;
}
inline uint32_t cluster_from_stride(const RecordFormat &f) {
    const uint32_t chunks = f.d_bytes / 16;
    return 16u * (chunks % 2 == 0 ? chunks + 1 : chunks);
}

// Per-kernel launch state kept across calls, safe for concurrent host
// threads and separate per device (kernel attributes and occupancy belong to
// a device).  Instances live in static storage, where the atomics start at 0.
constexpr int kMaxDevices = 64;

inline int current_device() {
    int d = 0;
    if (cudaGetDevice(&d) != cudaSuccess) return 0;
    return d >= 0 && d < kMaxDevices ? d : 0;
}

// The dynamic shared memory a kernel may use: raised on a device, under a
// lock and only ever upward, the first time a launch needs more than the
// default 48 KB or than allowed so far.
struct SmemLimit {
    std::atomic<size_t> allowed[kMaxDevices];
    std::mutex lock;
    template <typename K>
    cudaError_t ensure(K kern, size_t bytes) {
        if (bytes <= 48 * 1024) return cudaSuccess;
        std::atomic<size_t> &a = allowed[current_device()];
        if (bytes <= a.load(std::memory_order_acquire)) return cudaSuccess;
        std::lock_guard<std::mutex> g(lock);
        if (bytes <= a.load(std::memory_order_relaxed)) return cudaSuccess;
        const cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
        if (e == cudaSuccess) a.store(bytes, std::memory_order_release);
        return e;
    }
};

// Resident blocks per SM of a kernel at a given dynamic shared memory size:
// the last answer per device, kept as one word (size + 1 in the high half,
// blocks in the low half) so readers never see a torn pair.
struct OccupancyMemo {
    std::atomic<uint64_t> last[kMaxDevices];
    template <typename K>
    cudaError_t blocks(K kern, int threads, size_t smem, int &occ) {
        std::atomic<uint64_t> &a = last[current_device()];
        const uint64_t key = (uint64_t)(smem + 1) << 32;
        const uint64_t v = a.load(std::memory_order_relaxed);
        if ((v & ~0xffffffffull) == key) {
            occ = (int)(uint32_t)v;
            return cudaSuccess;
        }
        const cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, threads, smem);
        if (e == cudaSuccess) a.store(key | (uint32_t)occ, std::memory_order_relaxed);
        return e;
    }
};

// Nodes per sweep tile (8, 16 or 32; 16 unless a tuned choice says otherwise).
struct SweepConfig {
    int nt = 16;
};

// Launch one half-sweep; returns the kernel launch error.
cudaError_t launch_sweep(const RecordFormat &f, const SweepConfig &cfg, SweepParams p, cudaStream_t s,
                         int num_sms);
// Launches of 64-byte-message kernels (L = 16, FP32) with at least this many
// 16-node tiles store their messages with ordinary stores (see tile_finish).
constexpr long kDirectStoreTiles = 16384;

// Largest L the sweep kernels are compiled for.
constexpr int kMaxLabels = 128;

// Auxiliary kernels (aux_kernels.cu).
cudaError_t launch_costs_to_records(const RecordFormat &f, int cost_type, const void *src, int W, int H,
                                    unsigned char *rec, cudaStream_t s);
// The layout transform fused with the level-1 pyramid sums.
cudaError_t launch_costs_to_records_pyr(const RecordFormat &f, int cost_type, const void *src, int W, int H,
                                        unsigned char *rec, unsigned char *crec, int cW, cudaStream_t s);
cudaError_t launch_pyramid(const RecordFormat &f, const unsigned char *frec, int fW, int fH, unsigned char *crec,
                           int cW, int cH, cudaStream_t s);
cudaError_t launch_init_messages(const RecordFormat &f, unsigned char *rec, int W, int H,
                                 const unsigned char *crec, int cW, int cH, cudaStream_t s);
cudaError_t launch_fill_interior(int32_t *labels, int W, int H, int32_t value, cudaStream_t s);
cudaError_t launch_decode_fresh(const RecordFormat &f, const unsigned char *rec, int W, int H, int32_t *labels,
                                cudaStream_t s);
cudaError_t launch_export_messages(const RecordFormat &f, const unsigned char *rec, int W, int H, void *dst,
                                   cudaStream_t s);
cudaError_t launch_icm_sync(const RecordFormat &f, const unsigned char *rec, int W, int H, const void *V,
                            const int32_t *old_labels, int32_t *new_labels, const uint8_t *chg_in, uint8_t *chg_out,
                            int *status, cudaStream_t s);
cudaError_t launch_icm_async_diag(const RecordFormat &f, const unsigned char *rec, int W, int H, const void *V,
                                  int32_t *labels, int diag, int *status, cudaStream_t s);
// Energy with costs addressed as base + node*node_stride + label*label_stride
// (elements of the compute type): records (rec_bytes/t_size, 1) or the
// caller's label-planar array (1, W*H).  partials holds num_partials doubles.
cudaError_t launch_energy(int ctype, const void *costs, size_t node_stride, size_t label_stride, int W, int H, int L,
                          const void *V, const int32_t *labels, double *partials, int num_partials, double *out,
                          int *status, cudaStream_t s);
int energy_num_partials(int W, int H);
cudaError_t launch_convert_table(int src_type, int dst_type, const void *src, void *dst, int n, cudaStream_t s);
// Warm-start helpers (FP32 records, native store).
cudaError_t launch_level_x(const RecordFormat &f, const unsigned char *rec, int W, int H, float scale, float *out,
                           cudaStream_t s);
cudaError_t launch_level_beliefs(const RecordFormat &f, const unsigned char *rec, int W, int H, float scale,
                                 float *out, cudaStream_t s);
cudaError_t launch_fine_labels(const RecordFormat &f, const unsigned char *rect, int Wt, int Ht, int t,
                               int32_t *lab_t, int32_t *lab0, int W0, int H0, cudaStream_t s);
cudaError_t launch_project_fine(const RecordFormat &f, const unsigned char *rec0, int W0, int H0,
                                const unsigned char *rect, int Wt, int Ht, int t, float *out, cudaStream_t s);
cudaError_t launch_warm_init(const RecordFormat &f, unsigned char *rec, int W, int H, const float *y, const float *x,
                             float factor, cudaStream_t s);

// Alpha-beta swap (graphcut.cu): int32 costs D (label-planar) and table V on
// the device; result holds the initial labelling and receives the final one;
// excess, height and res (6 * W * H, slot-major) must start at zero; newr,
// dist, q0 and q1 are W * H scratch words each.
struct AlphaBetaParams {
    int W, H, L;
    const int32_t *D, *V;
    int32_t *result, *newr, *excess, *height, *res, *dist, *q0, *q1;
    int iters;
    int *status;
};
cudaError_t launch_alpha_beta(const AlphaBetaParams &p, cudaStream_t s);

// Sets the message ginf_last_error() returns on this host thread.
void set_last_error(const char *msg);

cudaError_t launch_stereo_costs(int W, int H, int L, const float *left, const float *right, float coef, float cap,
                                float *costs, cudaStream_t s);
cudaError_t launch_stereo_costs_u8(int W, int H, int L, const uint8_t *left, const uint8_t *right, int cap,
                                   int32_t *costs, cudaStream_t s);

}  // namespace ginf_gpu
