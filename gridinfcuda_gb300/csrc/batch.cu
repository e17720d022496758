// batch.cu -- many independent grids solved together: one persistent,
// cooperative launch walks a work list of (grid, tile) entries for each
// half-sweep, with a bounded grid barrier between half-sweeps; the whole
// solve (layout transforms, initialisation, the persistent launches) is
// captured once into a CUDA graph and replayed.  The tile shape and the
// number of half-sweeps per persistent launch come from an autotuner that
// times the candidates on the batch itself and caches the winner per mix of
// (grid-size class, label count) buckets in a JSON file.
//
// The reference solves one grid per call (src/include/bp.h:14-26); batching
// is new here.  Every grid runs loopy BP with the reference's semantics.
#include <cuda_fp16.h>

#include <algorithm>
#include <atomic>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "ginf_gb300.h"
#include "sweep_impl.cuh"

namespace ginf_gpu {

struct BatchItem {
    unsigned char *rec;
    int32_t *labels;
    const float *V;
    int W, H, L, Lp;
    uint32_t rec_bytes, d_bytes, m_bytes, slot_bytes;
    int tiles_per_row, num_tiles;  // per half-sweep, for the launch's tile size
    int tile_base;                 // first work-list tile of this grid (within its group)
};

struct BatchLaunch {
    const BatchItem *items;
    int count, total_tiles;
    int it_begin, it_end, iters;
    int first_mode;           // RD_ZERO (fused start) or RD_OWN (messages initialised)
    unsigned int *barrier;    // {arrived, generation}
    int *status;
    uint32_t tile_smem;       // bytes of tile slots at the start of dynamic shared memory
    int bases_in_smem;        // the grids' tile bases follow the slots
};

// Index of the grid that owns work-list tile t (tile bases ascending).
__device__ __forceinline__ int batch_item_of(const BatchLaunch &b, const int *bases, int t) {
    int lo = 0, hi = b.count - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        const int base = bases ? bases[mid] : __ldg(&b.items[mid].tile_base);
        if (base <= t) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

__device__ __forceinline__ SweepParams batch_params(const BatchLaunch &b, const BatchItem &g, int it) {
    SweepParams p{};
    p.W = g.W;
    p.H = g.H;
    p.L = g.L;
    p.Lp = g.Lp;
    p.rec_bytes = g.rec_bytes;
    p.d_bytes = g.d_bytes;
    p.m_bytes = g.m_bytes;
    p.slot_bytes = g.slot_bytes;
    p.rec = g.rec;
    p.iter = it;
    p.read_mode = it == 0 ? b.first_mode : RD_OWN;
    p.mode = MODE_LINEAR;
    p.V = g.V;
    p.labels = g.labels;
    p.write_labels = it >= b.iters - 2;
    p.tiles_per_row = g.tiles_per_row;
    p.num_tiles = g.num_tiles;
    p.status = b.status;
    return p;
}


// Persistent kernel: half-sweeps it_begin..it_end-1 of every grid of one
// label bucket (L == LM when EXACT, else L < LM; one kernel per bucket keeps
// the register allocation of the single-grid sweep).  Within
// a half-sweep the tiles of all grids are independent: block k takes work-
// list tiles k, k + gridDim.x, ... and issues the bulk load of its next tile
// as soon as the current one is done (the grid owning a tile is found by a
// binary search over the tile bases, kept in shared memory).  Between
// half-sweeps each block waits for its own bulk stores, fences them against
// the next half-sweep's bulk loads and meets the others at the grid barrier.
template <int NW, int LM, bool EXACT, bool DIRECT = false>
__global__ void __launch_bounds__(NW * 32) batch_kernel(const BatchLaunch b) {
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ uint64_t full_bar;
    int *bases_s = reinterpret_cast<int *>(smem + b.tile_smem);
    if (threadIdx.x == 0) {
        mbar_init(&full_bar, NW * 32);
        fence_barrier_init();
    }
    if (b.bases_in_smem)
        for (int i = threadIdx.x; i < b.count; i += blockDim.x) bases_s[i] = b.items[i].tile_base;
    __syncthreads();
    const int *bases = b.bases_in_smem ? bases_s : nullptr;
    uint32_t parity = 0;
    for (int it = b.it_begin; it < b.it_end; ++it) {
        int t = blockIdx.x;
        SweepParams p{};
        int base = 0;
        if (t < b.total_tiles) {
            const BatchItem &g = b.items[batch_item_of(b, bases, t)];
            p = batch_params(b, g, it);
            base = g.tile_base;
            tile_load<NW>(p, t - base, smem, &full_bar);
        }
        for (; t < b.total_tiles; t += gridDim.x) {
            if (!tile_finish<float, float, LM, EXACT, NW, KIND_LINEAR, DIRECT>(
                    p, table_consts<float, KIND_LINEAR>(p.V, EXACT ? LM : p.L), t - base, smem, &full_bar, parity))
                return;
            const int tn = t + gridDim.x;
            if (tn < b.total_tiles) {
                const BatchItem &g = b.items[batch_item_of(b, bases, tn)];
                p = batch_params(b, g, it);
                base = g.tile_base;
                tile_load<NW>(p, tn - base, smem, &full_bar);
            }
        }
        bulk_wait_all();
        fence_proxy_async_global();
        if (it + 1 < b.it_end) {
            if (!grid_barrier(b.barrier, gridDim.x, b.status)) return;
            fence_proxy_async_global();
        }
    }
}

}  // namespace ginf_gpu

using namespace ginf_gpu;

namespace {

struct TuneChoice {
    int tile_nodes = 16;
    int sweeps_per_launch = 0;  // 0 = all half-sweeps in one launch
    double ms = 0.0;
};

std::string size_class_key(const ginf_grid &g) {
    int s = 0;
    for (long long n = (long long)g.width * g.height; n > 1; n >>= 1) ++s;
    return "L" + std::to_string(g.num_labels) + ":s" + std::to_string(s);
}

// Batch signature: the multiset of (label count, log2 of the node count)
// buckets, plus the iteration count.
std::string signature(const std::vector<ginf_grid> &grids, int iters) {
    std::map<std::string, int> counts;
    for (const auto &g : grids) counts[size_class_key(g)]++;
    std::string sig;
    for (const auto &kv : counts) sig += kv.first + "x" + std::to_string(kv.second) + ",";
    return sig + "it" + std::to_string(iters);
}

std::string cache_path() {
    if (const char *p = std::getenv("GINF_AUTOTUNE_CACHE")) return p;
    const char *base = std::getenv("XDG_CACHE_HOME");
    std::string dir = base ? std::string(base) : (std::getenv("HOME") ? std::string(std::getenv("HOME")) + "/.cache" : "/tmp");
    return dir + "/gridinfcuda_gb300_autotune.json";
}

std::mutex g_cache_mutex;

// The cache is a JSON object {"<signature>": {"tile_nodes": n,
// "sweeps_per_launch": s, "ms": t}, ...}, read and written whole.
std::map<std::string, TuneChoice> read_cache() {
    std::map<std::string, TuneChoice> out;
    FILE *f = std::fopen(cache_path().c_str(), "rb");
    if (!f) return out;
    std::string text;
    char buf[4096];
    size_t n;
    while ((n = std::fread(buf, 1, sizeof(buf), f)) > 0) text.append(buf, n);
    std::fclose(f);
    size_t pos = 0;
    while ((pos = text.find('"', pos)) != std::string::npos) {
        const size_t end = text.find('"', pos + 1);
        if (end == std::string::npos) break;
        const std::string key = text.substr(pos + 1, end - pos - 1);
        const size_t ob = text.find('{', end), cb = text.find('}', end);
        if (ob == std::string::npos || cb == std::string::npos || ob > cb) break;
        const std::string body = text.substr(ob, cb - ob);
        TuneChoice c;
        auto num = [&](const char *name, double &v) {
            const size_t k = body.find(name);
            if (k != std::string::npos) v = std::atof(body.c_str() + body.find(':', k) + 1);
        };
        double tn = 16, spl = 0, ms = 0;
        num("\"tile_nodes\"", tn);
        num("\"sweeps_per_launch\"", spl);
        num("\"ms\"", ms);
        c.tile_nodes = (int)tn;
        c.sweeps_per_launch = (int)spl;
        c.ms = ms;
        out[key] = c;
        pos = cb + 1;
    }
    return out;
}

void write_cache(const std::map<std::string, TuneChoice> &m) {
    const std::string path = cache_path();
    const std::string tmp = path + ".tmp";
    FILE *f = std::fopen(tmp.c_str(), "wb");
    if (!f) return;
    std::fprintf(f, "{\n");
    size_t i = 0;
    for (const auto &kv : m) {
        std::fprintf(f, "  \"%s\": {\"tile_nodes\": %d, \"sweeps_per_launch\": %d, \"ms\": %.4f}%s\n",
                     kv.first.c_str(), kv.second.tile_nodes, kv.second.sweeps_per_launch, kv.second.ms,
                     ++i < m.size() ? "," : "");
    }
    std::fprintf(f, "}\n");
    std::fclose(f);
    std::rename(tmp.c_str(), path.c_str());
}

ginf_status bfail(ginf_status s, const std::string &msg) {
    ginf_gpu::set_last_error(msg.c_str());
    return s;
}

#define GINF_BCK(call)                                                                                 \
    do {                                                                                               \
        cudaError_t e_ = (call);                                                                       \
        if (e_ != cudaSuccess) {                                                                       \
            cudaGetLastError();                                                                        \
            return bfail(e_ == cudaErrorMemoryAllocation ? GINF_ERR_OUT_OF_MEMORY : GINF_ERR_CUDA,      \
                         std::string(#call) + ": " + cudaGetErrorString(e_));                          \
        }                                                                                              \
    } while (0)

}  // namespace

// Grids whose label count falls in one bucket (LM = 16, 32 or 64; exact when
// L == LM), solved by one kernel instantiation; items first..first+count-1.
struct BatchGroup {
    int lm = 64;
    bool exact = true;
    int first = 0, count = 0;
    int total_tiles = 0;
    uint32_t max_slot = 0;
};

struct ginf_batch {
    int device = -1;  // the device the plan was built on (its buffers and graph live there)
    int count = 0, iters = 0;
    std::vector<ginf_grid> grids;
    std::vector<int32_t *> labels;
    std::vector<RecordFormat> fmt;
    unsigned char *arena = nullptr;
    size_t arena_bytes = 0;
    BatchItem *items_dev = nullptr;
    unsigned int *barrier = nullptr;
    int *status = nullptr;
    int *status_host = nullptr;
    std::vector<unsigned char *> rec;
    int num_sms = 0;
    uint32_t max_slot = 0;
    std::vector<BatchGroup> groups;  // grids by label bucket, in items order
    std::vector<int> order;          // grid index of each item
    TuneChoice choice;
    int launches_per_run = 0;
    cudaStream_t cap_stream = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    bool tuned_now = false;
    // Stream-ordered replays: `done` follows the last one; the device status
    // words of finished replays accumulate in `deferred`.
    cudaEvent_t done = nullptr;
    bool pending = false;
    std::atomic<int> deferred{0};
};

namespace {

int label_bucket(int L) { return L <= 16 ? 16 : (L <= 32 ? 32 : 64); }

// Groups the grids by label bucket (once, at creation).
void make_groups(ginf_batch *b) {
    b->groups.clear();
    b->order.clear();
    for (int lm : {16, 32, 64})
        for (int exact = 1; exact >= 0; --exact) {
            BatchGroup grp;
            grp.lm = lm;
            grp.exact = exact != 0;
            grp.first = (int)b->order.size();
            for (int i = 0; i < b->count; ++i) {
                const int L = b->grids[i].num_labels;
                if (label_bucket(L) != lm || (L == lm) != grp.exact) continue;
                b->order.push_back(i);
                grp.max_slot = std::max(grp.max_slot, b->fmt[i].slot_bytes);
            }
            grp.count = (int)b->order.size() - grp.first;
            if (grp.count > 0) b->groups.push_back(grp);
        }
}

// Items for a given tile size (8 * NW nodes), in group order, with tile
// bases counted from each group's start; copied to the device.
std::vector<BatchItem> make_items(ginf_batch *b, int tile_nodes) {
    std::vector<BatchItem> items(b->count);
    for (auto &grp : b->groups) {
        grp.total_tiles = 0;
        for (int k = grp.first; k < grp.first + grp.count; ++k) {
            const int i = b->order[k];
            const ginf_grid &g = b->grids[i];
            const RecordFormat &f = b->fmt[i];
            BatchItem &it = items[k];
            it.rec = b->rec[i];
            it.labels = b->labels[i];
            it.V = static_cast<const float *>(g.sm_costs);
            it.W = g.width;
            it.H = g.height;
            it.L = g.num_labels;
            it.Lp = f.Lp;
            it.rec_bytes = f.rec_bytes;
            it.d_bytes = f.d_bytes;
            it.m_bytes = f.m_bytes;
            it.slot_bytes = f.slot_bytes;
            const int n1 = g.width >= 3 ? (g.width - 3) / 2 + 1 : 0;
            it.tiles_per_row = (n1 + tile_nodes - 1) / tile_nodes;
            it.num_tiles = (g.width >= 3 && g.height >= 3) ? (g.height - 2) * it.tiles_per_row : 0;
            it.tile_base = grp.total_tiles;
            grp.total_tiles += it.num_tiles;
        }
    }
    return items;
}

template <int NW, int LM, bool EXACT, bool DIRECT = false>
cudaError_t launch_batch(BatchLaunch bl, uint32_t max_slot, int num_sms, cudaStream_t s) {
    auto kern = batch_kernel<NW, LM, EXACT, DIRECT>;
    bl.tile_smem = (uint32_t)(((size_t)NW * 8 * max_slot + 15) / 16 * 16);
    const size_t bases_bytes = sizeof(int) * (size_t)bl.count;
    bl.bases_in_smem = bases_bytes <= 16 * 1024 ? 1 : 0;
    const size_t smem = bl.tile_smem + (bl.bases_in_smem ? bases_bytes : 0);
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int occ = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, NW * 32, smem);
    if (e != cudaSuccess) return e;
    if (occ < 1) return cudaErrorInvalidConfiguration;
    int grid = occ * num_sms;
    if (grid > bl.total_tiles && bl.it_end - bl.it_begin == 1) grid = std::max(1, bl.total_tiles);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(NW * 32);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kern, bl);
}

template <int LM, bool EXACT>
cudaError_t launch_batch_nw(int tile_nodes, const BatchLaunch &bl, uint32_t max_slot, int num_sms, cudaStream_t s) {
    if constexpr (LM == 16 && EXACT) {
        // 64-byte messages: ordinary stores on large groups (see tile_finish).
        if (tile_nodes == 16 && bl.total_tiles >= kDirectStoreTiles)
            return launch_batch<2, LM, EXACT, true>(bl, max_slot, num_sms, s);
    }
    if (tile_nodes == 8) return launch_batch<1, LM, EXACT>(bl, max_slot, num_sms, s);
    if (tile_nodes == 32) return launch_batch<4, LM, EXACT>(bl, max_slot, num_sms, s);
    return launch_batch<2, LM, EXACT>(bl, max_slot, num_sms, s);
}

cudaError_t launch_group(const BatchGroup &grp, int tile_nodes, const BatchLaunch &bl, int num_sms, cudaStream_t s) {
    switch (grp.lm * 2 + (grp.exact ? 1 : 0)) {
        case 33: return launch_batch_nw<16, true>(tile_nodes, bl, grp.max_slot, num_sms, s);
        case 32: return launch_batch_nw<16, false>(tile_nodes, bl, grp.max_slot, num_sms, s);
        case 65: return launch_batch_nw<32, true>(tile_nodes, bl, grp.max_slot, num_sms, s);
        case 64: return launch_batch_nw<32, false>(tile_nodes, bl, grp.max_slot, num_sms, s);
        case 129: return launch_batch_nw<64, true>(tile_nodes, bl, grp.max_slot, num_sms, s);
        default: return launch_batch_nw<64, false>(tile_nodes, bl, grp.max_slot, num_sms, s);
    }
}

// Records the whole batch solve on stream s: layout transforms, start-up
// initialisation, counters, then per label group its persistent launches.
ginf_status record_solve(ginf_batch *b, const TuneChoice &c, cudaStream_t s, int &launches) {
    launches = 0;
    make_items(b, c.tile_nodes);  // the device copy was made before the capture
    const bool fused = b->iters >= 2;
    for (int i = 0; i < b->count; ++i) {
        const ginf_grid &g = b->grids[i];
        GINF_BCK(launch_costs_to_records(b->fmt[i], CT_F32, g.data_costs, g.width, g.height, b->rec[i], s));
        ++launches;
        if (!fused) {
            GINF_BCK(launch_init_messages(b->fmt[i], b->rec[i], g.width, g.height, nullptr, 0, 0, s));
            GINF_BCK(launch_fill_interior(b->labels[i], g.width, g.height, 0, s));
            launches += 2;
        }
    }
    GINF_BCK(cudaMemsetAsync(b->barrier, 0, 2 * sizeof(unsigned int), s));
    GINF_BCK(cudaMemsetAsync(b->status, 0, sizeof(int), s));
    if (b->iters == 0) return GINF_OK;
    const int spl = c.sweeps_per_launch <= 0 ? b->iters : std::min(c.sweeps_per_launch, b->iters);
    for (const BatchGroup &grp : b->groups) {
        if (grp.total_tiles == 0) continue;
        for (int it0 = 0; it0 < b->iters; it0 += spl) {
            BatchLaunch bl{};
            bl.items = b->items_dev + grp.first;
            bl.count = grp.count;
            bl.total_tiles = grp.total_tiles;
            bl.it_begin = it0;
            bl.it_end = std::min(b->iters, it0 + spl);
            bl.iters = b->iters;
            bl.first_mode = fused ? RD_ZERO : RD_OWN;
            bl.barrier = b->barrier;
            bl.status = b->status;
            const cudaError_t e = launch_group(grp, c.tile_nodes, bl, b->num_sms, s);
            if (e != cudaSuccess) {
                cudaGetLastError();
                return bfail(GINF_ERR_CUDA, std::string("persistent batch launch: ") + cudaGetErrorString(e));
            }
            ++launches;
        }
    }
    return GINF_OK;
}

void drop_graph(ginf_batch *b) {
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->exec = nullptr;
    b->graph = nullptr;
}

// Captures the solve for choice c into a CUDA graph.  The grids' tile
// descriptors depend only on the tile size: they are copied to the device
// here, before the capture, and the graph reads them from there.
ginf_status capture(ginf_batch *b, const TuneChoice &c) {
    drop_graph(b);
    const std::vector<BatchItem> items = make_items(b, c.tile_nodes);
    GINF_BCK(cudaMemcpy(b->items_dev, items.data(), sizeof(BatchItem) * items.size(), cudaMemcpyHostToDevice));
    GINF_BCK(cudaStreamBeginCapture(b->cap_stream, cudaStreamCaptureModeThreadLocal));
    int launches = 0;
    ginf_status st = record_solve(b, c, b->cap_stream, launches);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(b->cap_stream, &g);
    if (st != GINF_OK) {
        if (g) cudaGraphDestroy(g);
        return st;
    }
    if (e != cudaSuccess) {
        cudaGetLastError();
        return bfail(GINF_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
    }
    b->graph = g;
    e = cudaGraphInstantiate(&b->exec, g, 0);
    if (e != cudaSuccess) {
        cudaGetLastError();
        drop_graph(b);
        return bfail(GINF_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
    }
    b->choice = c;
    b->launches_per_run = launches;
    return GINF_OK;
}

ginf_status run_graph(ginf_batch *b, cudaStream_t s) {
    GINF_BCK(cudaGraphLaunch(b->exec, s));
    GINF_BCK(cudaMemcpyAsync(b->status_host, b->status, sizeof(int), cudaMemcpyDeviceToHost, s));
    GINF_BCK(cudaStreamSynchronize(s));
    if (*b->status_host & DEV_ERR_TIMEOUT)
        return bfail(GINF_ERR_TIMEOUT, "a device-side wait of the batch solve exceeded its time limit");
    return GINF_OK;
}

// Times each candidate (tile size x half-sweeps per launch) on the batch.
ginf_status autotune(ginf_batch *b) {
    std::vector<TuneChoice> cands;
    const int spls[3] = {1, 5, 0};
    for (int tn : {8, 16, 32})
        for (int spl : spls) {
            if (spl > 0 && spl >= b->iters) continue;
            TuneChoice c;
            c.tile_nodes = tn;
            c.sweeps_per_launch = spl;
            cands.push_back(c);
        }
    TuneChoice best;
    best.ms = 1e30;
    for (auto &c : cands) {
        ginf_status st = capture(b, c);
        if (st != GINF_OK) continue;
        st = run_graph(b, b->cap_stream);  // warm-up
        if (st != GINF_OK) return st;
        float total = 0.f;
        for (int r = 0; r < 3; ++r) {
            GINF_BCK(cudaEventRecord(b->ev0, b->cap_stream));
            GINF_BCK(cudaGraphLaunch(b->exec, b->cap_stream));
            GINF_BCK(cudaEventRecord(b->ev1, b->cap_stream));
            GINF_BCK(cudaEventSynchronize(b->ev1));
            float ms = 0.f;
            GINF_BCK(cudaEventElapsedTime(&ms, b->ev0, b->ev1));
            total += ms;
        }
        c.ms = total / 3.0;
        if (c.ms < best.ms) best = c;
    }
    if (best.ms >= 1e29) return bfail(GINF_ERR_CUDA, "no batch configuration could be captured");
    b->tuned_now = true;
    return capture(b, best);
}

}  // namespace

extern "C" {

ginf_status ginf_batch_create(ginf_batch **out, const ginf_grid *grids, int32_t *const *labels, int32_t count,
                              int32_t iters, const ginf_options *opt) {
    ginf_gpu::set_last_error("");
    if (!out || !grids || !labels || count < 1) return bfail(GINF_ERR_INVALID_ARGUMENT, "NULL argument or empty batch");
    if (iters < 0) return bfail(GINF_ERR_INVALID_ARGUMENT, "iters must be >= 0");
    for (int i = 0; i < count; ++i) {
        const ginf_grid &g = grids[i];
        if (g.memory != GINF_DEVICE || !g.data_costs || !g.sm_costs || !labels[i])
            return bfail(GINF_ERR_INVALID_ARGUMENT, "batch grid " + std::to_string(i) +
                                                        ": every buffer must be device memory and non-NULL");
        if (g.width < 1 || g.height < 1 || g.num_labels < 2 || g.num_labels > 64)
            return bfail(GINF_ERR_UNSUPPORTED, "batch grid " + std::to_string(i) + ": needs 2 <= L <= 64");
        if (g.cost_type != GINF_F32 || (g.sm_model != GINF_SM_TRUNC_LINEAR && g.sm_model != GINF_SM_POTTS))
            return bfail(GINF_ERR_UNSUPPORTED, "batch grid " + std::to_string(i) +
                                                   ": batches take FP32 costs with Potts or truncated-linear smoothness");
    }
    ginf_options defaults;
    ginf_default_options(&defaults);
    if (!opt) opt = &defaults;
    int dev = 0;
    GINF_BCK(cudaGetDevice(&dev));
    int major = 0, minor = 0, coop = 0;
    GINF_BCK(cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev));
    GINF_BCK(cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev));
    GINF_BCK(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
    if (major * 10 + minor != 103) return bfail(GINF_ERR_NO_DEVICE, "this library is built for sm_103 (GB300)");
    if (!coop) return bfail(GINF_ERR_NO_DEVICE, "the device does not support cooperative launches");

    ginf_batch *b = new ginf_batch();
    b->device = dev;
    b->count = count;
    b->iters = iters;
    b->grids.assign(grids, grids + count);
    b->labels.assign(labels, labels + count);
    GINF_BCK(cudaDeviceGetAttribute(&b->num_sms, cudaDevAttrMultiProcessorCount, dev));
    size_t total = 0;
    std::vector<size_t> off(count);
    for (int i = 0; i < count; ++i) {
        b->fmt.push_back(make_format(CT_F32, ST_NATIVE, grids[i].num_labels));
        b->max_slot = std::max(b->max_slot, b->fmt[i].slot_bytes);
        off[i] = total;
        total += ((size_t)grids[i].width * grids[i].height * b->fmt[i].rec_bytes + 255) / 256 * 256;
    }
    const size_t items_off = total;
    total += ((sizeof(BatchItem) * count + 255) / 256) * 256;
    const size_t ctl_off = total;
    total += 256;
    cudaError_t e = cudaMalloc(&b->arena, total);
    if (e != cudaSuccess) {
        cudaGetLastError();
        delete b;
        return bfail(GINF_ERR_OUT_OF_MEMORY, "batch records: " + std::string(cudaGetErrorString(e)));
    }
    b->arena_bytes = total;
    for (int i = 0; i < count; ++i) b->rec.push_back(b->arena + off[i]);
    make_groups(b);
    b->items_dev = reinterpret_cast<BatchItem *>(b->arena + items_off);
    b->barrier = reinterpret_cast<unsigned int *>(b->arena + ctl_off);
    b->status = reinterpret_cast<int *>(b->arena + ctl_off + 64);
    ginf_status st = GINF_OK;
    if (cudaMallocHost(&b->status_host, sizeof(int)) != cudaSuccess ||
        cudaStreamCreateWithFlags(&b->cap_stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&b->ev0) != cudaSuccess || cudaEventCreate(&b->ev1) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->done, cudaEventDisableTiming) != cudaSuccess) {
        cudaGetLastError();
        st = bfail(GINF_ERR_CUDA, "batch set-up failed");
    }
    if (st == GINF_OK) {
        TuneChoice c;
        const std::string sig = signature(b->grids, iters);
        bool have = false;
        if (opt->tile_nodes != 0 || opt->sweeps_per_launch != 0) {
            // An explicit choice (either knob) is used as given.
            c.tile_nodes = opt->tile_nodes == 8 || opt->tile_nodes == 32 ? opt->tile_nodes : 16;
            c.sweeps_per_launch = opt->sweeps_per_launch;
            have = true;
        } else if (opt->autotune != 1) {
            std::lock_guard<std::mutex> lock(g_cache_mutex);
            auto cache = read_cache();
            auto it = cache.find(sig);
            if (it != cache.end()) {
                c = it->second;
                have = true;
            } else if (opt->autotune == -1) {
                have = true;  // defaults, no measurement
            }
        }
        if (have) {
            st = capture(b, c);
        } else {
            st = autotune(b);
            if (st == GINF_OK) {
                std::lock_guard<std::mutex> lock(g_cache_mutex);
                auto cache = read_cache();
                cache[sig] = b->choice;
                write_cache(cache);
            }
        }
    }
    if (st != GINF_OK) {
        ginf_batch_destroy(b);
        return st;
    }
    *out = b;
    return GINF_OK;
}

namespace {

void CUDART_CB batch_replay_done(void *p) {
    ginf_batch *b = static_cast<ginf_batch *>(p);
    const int st = *b->status_host;
    if (st) b->deferred.fetch_or(st);
}

ginf_status batch_status_error(int st) {
    if (st & DEV_ERR_TIMEOUT)
        return bfail(GINF_ERR_TIMEOUT, "a device-side wait of the batch solve exceeded its time limit");
    return GINF_OK;
}

// Orders `s` after the batch's last stream-ordered replay and reports an
// error one of them recorded.
ginf_status batch_enter(ginf_batch *b, cudaStream_t s) {
    if (b->pending) GINF_BCK(cudaStreamWaitEvent(s, b->done, 0));
    return batch_status_error(b->deferred.exchange(0));
}

}  // namespace

namespace {
// A plan replays only on the device it was built on.
ginf_status check_batch_device(const ginf_batch *b) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return bfail(GINF_ERR_NO_DEVICE, "no current CUDA device");
    }
    if (dev != b->device)
        return bfail(GINF_ERR_INVALID_ARGUMENT, "batch was built on device " + std::to_string(b->device) +
                                                    ", the calling thread's current device is " + std::to_string(dev));
    return GINF_OK;
}
}  // namespace

ginf_status ginf_batch_enqueue(ginf_batch *b, void *stream) {
    ginf_gpu::set_last_error("");
    if (!b || !b->exec) return bfail(GINF_ERR_INVALID_ARGUMENT, "batch is NULL or has no captured solve");
    if (ginf_status st = check_batch_device(b); st != GINF_OK) return st;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    ginf_status st = batch_enter(b, s);
    if (st != GINF_OK) return st;
    GINF_BCK(cudaGraphLaunch(b->exec, s));
    GINF_BCK(cudaMemcpyAsync(b->status_host, b->status, sizeof(int), cudaMemcpyDeviceToHost, s));
    GINF_BCK(cudaLaunchHostFunc(s, batch_replay_done, b));
    GINF_BCK(cudaEventRecord(b->done, s));
    b->pending = true;
    return GINF_OK;
}

ginf_status ginf_batch_sync(ginf_batch *b) {
    ginf_gpu::set_last_error("");
    if (!b) return bfail(GINF_ERR_INVALID_ARGUMENT, "batch is NULL");
    if (b->pending) {
        GINF_BCK(cudaEventSynchronize(b->done));
        b->pending = false;
    }
    return batch_status_error(b->deferred.exchange(0));
}

ginf_status ginf_batch_run(ginf_batch *b, void *stream, ginf_stats *stats) {
    ginf_gpu::set_last_error("");
    if (!b || !b->exec) return bfail(GINF_ERR_INVALID_ARGUMENT, "batch is NULL or has no captured solve");
    if (ginf_status st = check_batch_device(b); st != GINF_OK) return st;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    {
        ginf_status st = batch_enter(b, s);
        if (st != GINF_OK) return st;
    }
    if (stats) {
        std::memset(stats, 0, sizeof(*stats));
        GINF_BCK(cudaEventRecord(b->ev0, s));
    }
    GINF_BCK(cudaGraphLaunch(b->exec, s));
    if (stats) GINF_BCK(cudaEventRecord(b->ev1, s));
    GINF_BCK(cudaMemcpyAsync(b->status_host, b->status, sizeof(int), cudaMemcpyDeviceToHost, s));
    GINF_BCK(cudaStreamSynchronize(s));
    if (*b->status_host & DEV_ERR_TIMEOUT)
        return bfail(GINF_ERR_TIMEOUT, "a device-side wait of the batch solve exceeded its time limit");
    if (stats) {
        float ms = 0.f;
        GINF_BCK(cudaEventElapsedTime(&ms, b->ev0, b->ev1));
        stats->total_ms = ms;
        stats->sweep_ms = ms;
        stats->kernel_launches = b->launches_per_run;
        int64_t nli = 0;
        for (const auto &g : b->grids) nli += (int64_t)g.width * g.height * g.num_labels * b->iters;
        stats->node_label_iters = nli;
    }
    return GINF_OK;
}

ginf_status ginf_batch_config(const ginf_batch *b, int32_t *tile_nodes, int32_t *sweeps_per_launch,
                              int32_t *tuned_now) {
    if (!b) return bfail(GINF_ERR_INVALID_ARGUMENT, "batch is NULL");
    if (tile_nodes) *tile_nodes = b->choice.tile_nodes;
    if (sweeps_per_launch) *sweeps_per_launch = b->choice.sweeps_per_launch <= 0 ? b->iters : b->choice.sweeps_per_launch;
    if (tuned_now) *tuned_now = b->tuned_now ? 1 : 0;
    return GINF_OK;
}

ginf_status ginf_batch_destroy(ginf_batch *b) {
    if (!b) return GINF_OK;
    if (b->pending) cudaEventSynchronize(b->done);
    if (b->done) cudaEventDestroy(b->done);
    drop_graph(b);
    if (b->arena) cudaFree(b->arena);
    if (b->status_host) cudaFreeHost(b->status_host);
    if (b->cap_stream) cudaStreamDestroy(b->cap_stream);
    if (b->ev0) cudaEventDestroy(b->ev0);
    if (b->ev1) cudaEventDestroy(b->ev1);
    delete b;
    return GINF_OK;
}

ginf_status ginf_decode_bp_batch(const ginf_grid *grids, int32_t *const *labels, int32_t count, int32_t iters,
                                 const ginf_options *opt, ginf_stats *stats) {
    ginf_batch *b = nullptr;
    ginf_status st = ginf_batch_create(&b, grids, labels, count, iters, opt);
    if (st != GINF_OK) return st;
    st = ginf_batch_run(b, opt ? opt->stream : nullptr, stats);
    ginf_batch_destroy(b);
    return st;
}

}  // extern "C"
