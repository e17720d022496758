// capi.cu -- implementation of the C ABI declared in include/ginf_gb300.h.
//
// Host-side driver of the inference path: argument checks, the workspace
// arena, host<->device copies, the HBP level loop (bp.cc:86-180 /
// bp.cu:133-223), ICM (icm.cc:4-67), the energy (grid.cc:102-125) and status
// reporting.  Every entry point is synchronous, like the reference (its
// cudaMemcpy calls block, gpu.h:59,123): it returns after its stream has
// drained, with the device status word checked.
#include <cuda_fp16.h>

#include <algorithm>
#include <climits>
#include <cstdio>
#include <atomic>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "ginf_gb300.h"
#include "ginf_internal.h"

using namespace ginf_gpu;

namespace ginf_gpu {
ginf_status warmnet_forward(ginf_warmnet *n, const float *x, int nimg, int h, int w, float **y_out, int *status,
                            cudaStream_t s);
int warmnet_labels(const ginf_warmnet *n);

template <typename T, typename M>
cudaError_t launch_sweep_tm(const RecordFormat &, const SweepConfig &, const SweepParams &, cudaStream_t, int);

cudaError_t launch_sweep(const RecordFormat &f, const SweepConfig &cfg, SweepParams p, cudaStream_t s, int num_sms) {
    if (f.store == ST_F16) return launch_sweep_tm<float, __half>(f, cfg, p, s, num_sms);
    switch (f.ctype) {
        case CT_F32: return launch_sweep_tm<float, float>(f, cfg, p, s, num_sms);
        case CT_I32: return launch_sweep_tm<int, int>(f, cfg, p, s, num_sms);
        case CT_F64: return launch_sweep_tm<double, double>(f, cfg, p, s, num_sms);
    }
    return cudaErrorInvalidValue;
}

}  // namespace ginf_gpu

namespace {

thread_local std::string g_last_error;

ginf_status fail(ginf_status s, const std::string &msg) {
    g_last_error = msg;
    return s;
}

ginf_status cuda_fail(cudaError_t e, const char *what) {
    if (e == cudaErrorMemoryAllocation) {
        cudaGetLastError();
        return fail(GINF_ERR_OUT_OF_MEMORY, std::string(what) + ": " + cudaGetErrorString(e));
    }
    return fail(GINF_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define GINF_CK(call)                                          \
    do {                                                       \
        cudaError_t e_ = (call);                               \
        if (e_ != cudaSuccess) return cuda_fail(e_, #call);    \
    } while (0)

#define GINF_TRY(call)                                         \
    do {                                                       \
        ginf_status s_ = (call);                               \
        if (s_ != GINF_OK) return s_;                          \
    } while (0)

size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

}  // namespace

// Reusable device state of one caller (thread / stream).
struct ginf_workspace {
    int device = -1;
    int num_sms = 0;
    unsigned char *arena = nullptr;
    size_t arena_bytes = 0;
    int *status_host = nullptr;   // pinned
    double *energy_host = nullptr;  // pinned
    cudaEvent_t ev[10] = {};
    bool events = false;
    // Stream-ordered calls: `done` is recorded behind the last one; later
    // calls on this workspace order their stream after it.  Device status
    // words of finished stream-ordered calls accumulate in `deferred`.
    cudaEvent_t done = nullptr;
    bool pending = false;
    std::atomic<int> deferred{0};
};

namespace {

enum { EV_START, EV_UPLOAD, EV_PREPARE, EV_L0_START, EV_SWEEPS, EV_ICM, EV_ENERGY, EV_END, EV_COUNT };

// A workspace belongs to the device of its first call: its buffers and
// events live there, so calls from another device are refused.
ginf_status check_device(ginf_workspace *ws) {
    int dev = 0;
    GINF_CK(cudaGetDevice(&dev));
    if (ws->device == dev) return GINF_OK;
    if (ws->device >= 0)
        return fail(GINF_ERR_INVALID_ARGUMENT, "workspace belongs to device " + std::to_string(ws->device) +
                                                   ", the calling thread's current device is " + std::to_string(dev));
    cudaDeviceProp prop;
    cudaError_t e = cudaGetDeviceProperties(&prop, dev);
    if (e != cudaSuccess) return fail(GINF_ERR_NO_DEVICE, std::string("no CUDA device: ") + cudaGetErrorString(e));
    if (prop.major * 10 + prop.minor != 103)
        return fail(GINF_ERR_NO_DEVICE, std::string("this library is built for sm_103 (GB300); device is ") +
                                            prop.name);
    ws->device = dev;
    ws->num_sms = prop.multiProcessorCount;
    return GINF_OK;
}

ginf_status device_status_error(int st) {
    if (st & DEV_ERR_TIMEOUT) return fail(GINF_ERR_TIMEOUT, "a device-side wait exceeded its time limit");
    if (st & DEV_ERR_BOUNDS) return fail(GINF_ERR_INVALID_ARGUMENT, "a label is outside [0, num_labels)");
    return GINF_OK;
}

// Readies the workspace for a call on `stream`: the stream waits for the
// workspace's last stream-ordered call, and a device error that call
// recorded is reported now.
ginf_status ws_init(ginf_workspace *ws, cudaStream_t stream) {
    GINF_TRY(check_device(ws));
    if (!ws->status_host) {
        GINF_CK(cudaMallocHost(&ws->status_host, 64));
        ws->energy_host = reinterpret_cast<double *>(ws->status_host + 8);
    }
    if (!ws->events) {
        for (int i = 0; i < EV_COUNT; ++i) GINF_CK(cudaEventCreate(&ws->ev[i]));
        GINF_CK(cudaEventCreateWithFlags(&ws->done, cudaEventDisableTiming));
        ws->events = true;
    }
    if (ws->pending) GINF_CK(cudaStreamWaitEvent(stream, ws->done, 0));
    return device_status_error(ws->deferred.exchange(0));
}

// Carves sub-buffers out of one growing device allocation.
struct Arena {
    std::vector<size_t> sizes;
    size_t add(size_t bytes) {
        sizes.push_back(align_up(bytes, 256));
        return sizes.size() - 1;
    }
    size_t total() const {
        size_t t = 0;
        for (size_t s : sizes) t += s;
        return t;
    }
    unsigned char *ptr(unsigned char *base, size_t id) const {
        size_t off = 0;
        for (size_t i = 0; i < id; ++i) off += sizes[i];
        return base + off;
    }
};

ginf_status ws_reserve(ginf_workspace *ws, size_t bytes) {
    if (bytes <= ws->arena_bytes) return GINF_OK;
    if (ws->arena) {
        cudaFree(ws->arena);
        ws->arena = nullptr;
        ws->arena_bytes = 0;
    }
    cudaError_t e = cudaMalloc(&ws->arena, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(GINF_ERR_OUT_OF_MEMORY, "cudaMalloc of " + std::to_string(bytes) + " bytes failed: " +
                                                cudaGetErrorString(e));
    }
    ws->arena_bytes = bytes;
    return GINF_OK;
}

// Per-call workspace: the caller's, or a temporary one freed on exit.
struct WsGuard {
    ginf_workspace *ws;
    bool owned;
    explicit WsGuard(ginf_workspace *w) : ws(w), owned(w == nullptr) {
        if (owned) ws = new ginf_workspace();
    }
    ~WsGuard() {
        if (owned) ginf_workspace_destroy(ws);
    }
};

size_t type_size(int t) { return t == GINF_F64 ? 8 : 4; }

ginf_status check_grid(const ginf_grid *g) {
    if (!g) return fail(GINF_ERR_INVALID_ARGUMENT, "grid is NULL");
    if (g->width < 1 || g->height < 1) return fail(GINF_ERR_INVALID_ARGUMENT, "grid width/height must be >= 1");
    if (g->num_labels < 2)
        return fail(GINF_ERR_INVALID_ARGUMENT,
                    "num_labels must be >= 2 (the reference reads V(0,1) out of bounds for one label, bp.cc:35)");
    if (g->cost_type != GINF_F32 && g->cost_type != GINF_I32)
        return fail(GINF_ERR_INVALID_ARGUMENT, "cost_type must be GINF_F32 or GINF_I32");
    if (g->sm_model < GINF_SM_EXPLICIT || g->sm_model > GINF_SM_TRUNC_QUAD)
        return fail(GINF_ERR_INVALID_ARGUMENT, "unknown smoothness model");
    if (g->memory != GINF_HOST && g->memory != GINF_DEVICE)
        return fail(GINF_ERR_INVALID_ARGUMENT, "memory must be GINF_HOST or GINF_DEVICE");
    if (!g->data_costs || !g->sm_costs) return fail(GINF_ERR_INVALID_ARGUMENT, "data_costs / sm_costs is NULL");
    const double elems = (double)g->width * g->height * g->num_labels;
    if (elems > 4.0e10) return fail(GINF_ERR_INVALID_ARGUMENT, "grid too large");
    return GINF_OK;
}

struct Resolved {
    int ctype;      // compute type
    int store;      // ST_*
    int mode;       // Mode
    int norm_min;
    int decode;
    int host_access;
    int async;
    int cluster_k;  // most half-sweeps per temporal-blocking launch; 0 = one per launch
    SweepConfig cfg;
    cudaStream_t stream;
};

ginf_status resolve(const ginf_grid *g, const ginf_options *o, Resolved &r) {
    ginf_options d;
    ginf_default_options(&d);
    if (!o) o = &d;
    r.ctype = o->compute_type < 0 ? g->cost_type : o->compute_type;
    if (r.ctype != GINF_F32 && r.ctype != GINF_I32 && r.ctype != GINF_F64)
        return fail(GINF_ERR_INVALID_ARGUMENT, "unknown compute_type");
    if (o->msg_store != GINF_STORE_NATIVE && o->msg_store != GINF_STORE_F16)
        return fail(GINF_ERR_INVALID_ARGUMENT, "unknown msg_store");
    if (o->msg_store == GINF_STORE_F16 && r.ctype != GINF_F32)
        return fail(GINF_ERR_UNSUPPORTED, "the FP16 message store needs FP32 arithmetic");
    r.store = o->msg_store == GINF_STORE_F16 ? ST_F16 : ST_NATIVE;
    if (o->msg_rule != GINF_RULE_REFERENCE && o->msg_rule != GINF_RULE_STANDARD)
        return fail(GINF_ERR_INVALID_ARGUMENT, "unknown msg_rule");
    if (o->decode != GINF_DECODE_STALE && o->decode != GINF_DECODE_FRESH)
        return fail(GINF_ERR_INVALID_ARGUMENT, "unknown decode");
    if (o->normalize != GINF_NORM_MEAN && o->normalize != GINF_NORM_MIN)
        return fail(GINF_ERR_INVALID_ARGUMENT, "unknown normalize");
    const int m = g->sm_model;
    if (m == GINF_SM_POTTS || m == GINF_SM_TRUNC_LINEAR) r.mode = MODE_LINEAR;
    else if (o->msg_rule == GINF_RULE_REFERENCE) r.mode = MODE_REF_MINCONV;
    else if (m == GINF_SM_TRUNC_QUAD && r.ctype != GINF_I32) r.mode = MODE_STD_QUAD;
    else r.mode = MODE_STD_MINCONV;
    r.norm_min = (o->normalize == GINF_NORM_MIN || r.store == ST_F16) ? 1 : 0;
    r.decode = o->decode;
    if (o->tile_nodes != 0 && o->tile_nodes != 8 && o->tile_nodes != 16 && o->tile_nodes != 32)
        return fail(GINF_ERR_INVALID_ARGUMENT, "tile_nodes must be 0, 8, 16 or 32");
    r.cfg.nt = o->tile_nodes == 0 ? 16 : o->tile_nodes;
    if (o->host_access != GINF_HOST_AUTO && o->host_access != GINF_HOST_COPY)
        return fail(GINF_ERR_INVALID_ARGUMENT, "unknown host_access");
    r.host_access = o->host_access;
    if (o->sweeps_per_launch < 0) return fail(GINF_ERR_INVALID_ARGUMENT, "sweeps_per_launch must be >= 0");
    r.cluster_k = o->sweeps_per_launch >= 2 ? o->sweeps_per_launch : 0;
    r.async = o->stream_ordered != 0;
    r.stream = static_cast<cudaStream_t>(o->stream);
    return GINF_OK;
}

// A device-readable address of the host buffer p, or nullptr when the
// device cannot read it in place: page-locked memory (its mapped device
// pointer) or, where the device reads pageable memory coherently (Grace
// systems), the pointer itself.
const void *host_device_view(const void *p) {
    cudaPointerAttributes pa;
    if (cudaPointerGetAttributes(&pa, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (pa.type == cudaMemoryTypeHost) return pa.devicePointer;
    if (pa.type == cudaMemoryTypeUnregistered) {
        int dev = 0, pageable = 0;
        if (cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, dev) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;
        }
        return pageable ? p : nullptr;
    }
    return nullptr;
}

struct Level {
    int W, H;
    size_t off;  // byte offset within the records buffer
};

std::vector<Level> level_sizes(int W, int H, int levels, size_t rec_bytes, size_t &total) {
    std::vector<Level> lv(levels);
    size_t off = 0;
    for (int t = 0; t < levels; ++t) {
        lv[t].W = t == 0 ? W : (lv[t - 1].W + 1) / 2;  // ceil(w/2), bp.cc:101-102
        lv[t].H = t == 0 ? H : (lv[t - 1].H + 1) / 2;
        lv[t].off = off;
        off += align_up((size_t)lv[t].W * lv[t].H * rec_bytes, 256);
    }
    total = off;
    return lv;
}

// Everything a BP / ICM / energy pipeline run needs on the device.
struct Prepared {
    RecordFormat f;
    std::vector<Level> lv;
    unsigned char *rec = nullptr;  // records of all levels
    unsigned char *rec2 = nullptr; // second record buffer of the temporal-blocking launches (largest level)
    void *Vt = nullptr;            // table in the compute type
    int32_t *lab = nullptr;        // device labels (caller's or a copy)
    int32_t *lab2 = nullptr;       // second label buffer (ICM ping-pong)
    uint8_t *chg = nullptr;        // ICM change flags, two W*H byte maps (ping-pong)
    double *partials = nullptr;    // energy partials, status word follows
    int num_partials = 0;
    int *status = nullptr;
    double *energy = nullptr;
    void *msgs_stage = nullptr;
    int64_t launches = 0;
};

struct Call {
    ginf_workspace *ws;
    const ginf_grid *g;
    Resolved r;
    ginf_stats *stats;
    int64_t launches = 0;
    int64_t h2d = 0, d2h = 0;
    void ev(int i) {
        if (stats) cudaEventRecord(ws->ev[i], r.stream);
    }
};

// Uploads costs and table, builds level-0 records and the pyramid.
// levels == 0 builds a D-only record (ICM / energy).
ginf_status prepare(Call &c, Prepared &P, int levels, bool want_lab2, const int32_t *labels_in, int32_t *labels_dev) {
    const ginf_grid *g = c.g;
    const int W = g->width, H = g->height, L = g->num_labels;
    const bool bp = levels > 0;
    P.f = make_format(c.r.ctype, c.r.store, L);
    if (!bp) {
        P.f.m_bytes = 0;
        P.f.rec_bytes = P.f.d_bytes;
    }
    size_t rec_total = 0;
    P.lv = level_sizes(W, H, bp ? levels : 1, P.f.rec_bytes, rec_total);
    const size_t cost_bytes = (size_t)W * H * L * type_size(g->cost_type);
    const size_t table_in = (size_t)L * L * type_size(g->cost_type);
    const size_t table_t = (size_t)L * L * P.f.t_size;
    const size_t lab_bytes = (size_t)W * H * sizeof(int32_t);
    P.num_partials = energy_num_partials(W, H);

    const bool host = g->memory == GINF_HOST;
    // Host costs the device can read in place are read by the layout
    // transform itself (the transfer fused into it); others are staged.
    const void *host_view = host && c.r.host_access == GINF_HOST_AUTO ? host_device_view(g->data_costs) : nullptr;
    // Temporal blocking alternates between a level's records and a second
    // buffer as large as the largest level.
    const bool two_buffers = bp && c.r.cluster_k >= 2 && cluster_sweep_eligible(P.f, c.r.mode);
    Arena a;
    const size_t id_rec = a.add(rec_total);
    const size_t id_rec2 = two_buffers ? a.add((size_t)W * H * P.f.rec_bytes) : 0;
    const size_t id_stage = host && !host_view ? a.add(cost_bytes) : 0;
    const size_t id_tin = a.add(table_in);
    const size_t id_t = a.add(table_t);
    const size_t id_lab = (labels_dev == nullptr) ? a.add(lab_bytes) : 0;
    const size_t id_lab2 = want_lab2 ? a.add(lab_bytes) : 0;
    const size_t id_chg = want_lab2 ? a.add(2 * (size_t)W * H) : 0;
    const size_t id_part = a.add(sizeof(double) * (P.num_partials + 1) + 64);
    GINF_TRY(ws_reserve(c.ws, a.total()));
    unsigned char *base = c.ws->arena;
    P.rec = a.ptr(base, id_rec);
    P.rec2 = two_buffers ? a.ptr(base, id_rec2) : nullptr;
    P.Vt = a.ptr(base, id_t);
    P.lab = labels_dev ? labels_dev : reinterpret_cast<int32_t *>(a.ptr(base, id_lab));
    P.lab2 = want_lab2 ? reinterpret_cast<int32_t *>(a.ptr(base, id_lab2)) : nullptr;
    P.chg = want_lab2 ? a.ptr(base, id_chg) : nullptr;
    P.partials = reinterpret_cast<double *>(a.ptr(base, id_part));
    P.status = reinterpret_cast<int *>(P.partials + P.num_partials);
    P.energy = P.partials + P.num_partials + 1;
    cudaStream_t s = c.r.stream;

    GINF_CK(cudaMemsetAsync(P.status, 0, sizeof(int), s));
    // Costs and table on the device, in the caller's element type.
    const void *costs_dev = g->data_costs;
    const void *table_dev = g->sm_costs;
    if (host) {
        if (host_view) {
            costs_dev = host_view;
        } else {
            unsigned char *stage = a.ptr(base, id_stage);
            GINF_CK(cudaMemcpyAsync(stage, g->data_costs, cost_bytes, cudaMemcpyHostToDevice, s));
            costs_dev = stage;
        }
        unsigned char *tin = a.ptr(base, id_tin);
        GINF_CK(cudaMemcpyAsync(tin, g->sm_costs, table_in, cudaMemcpyHostToDevice, s));
        c.h2d += cost_bytes + table_in;
        table_dev = tin;
    }
    if (labels_in) {
        // Labels the device copy starts from (border values are read by ICM
        // and preserved for the caller).
        GINF_CK(cudaMemcpyAsync(P.lab, labels_in, lab_bytes, host ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice,
                                s));
        if (host) c.h2d += lab_bytes;
    }
    c.ev(EV_UPLOAD);
    if (c.r.ctype == g->cost_type) {
        GINF_CK(cudaMemcpyAsync(P.Vt, table_dev, table_t, cudaMemcpyDeviceToDevice, s));
    } else {
        GINF_CK(launch_convert_table(g->cost_type, c.r.ctype, table_dev, P.Vt, L * L, s));
        ++c.launches;
    }
    // Level 0 records, with level 1's costs formed on the way when there is
    // a pyramid; then the coarser levels.
    const int nlv = (int)P.lv.size();
    if (nlv >= 2)
        GINF_CK(launch_costs_to_records_pyr(P.f, g->cost_type, costs_dev, W, H, P.rec, P.rec + P.lv[1].off,
                                            P.lv[1].W, s));
    else
        GINF_CK(launch_costs_to_records(P.f, g->cost_type, costs_dev, W, H, P.rec, s));
    ++c.launches;
    for (int t = 2; t < nlv; ++t) {
        GINF_CK(launch_pyramid(P.f, P.rec + P.lv[t - 1].off, P.lv[t - 1].W, P.lv[t - 1].H, P.rec + P.lv[t].off,
                               P.lv[t].W, P.lv[t].H, s));
        ++c.launches;
    }
    c.ev(EV_PREPARE);
    return GINF_OK;
}

// Truncation radius of a quadratic table, with the comparisons of the
// device's quad_radius (sweep_impl.cuh): V(0,k) < V(0,L-1) for k <= r on a
// nondecreasing profile; 9 means "wider than any window".
template <typename T>
int quad_radius_host(const std::vector<unsigned char> &col, int L) {
    const T *v = reinterpret_cast<const T *>(col.data());
    const T trunc = v[L - 1];
    int r = 0;
    T prev = v[0];
    for (int k = 1; k < L && k <= 9; ++k) {
        if (v[k] < prev) return 9;
        prev = v[k];
        if (!(v[k] < trunc)) break;
        r = k;
    }
    if (!(v[0] <= trunc)) return 9;
    return r;
}

// Whether V(0,0) = 0 and V(0,k) = V(0,1) k^2 exactly for k <= r (the pass
// form of the quadratic transform assumes that profile).
template <typename T>
bool quad_exact_host(const std::vector<unsigned char> &col, int r) {
    const T *v = reinterpret_cast<const T *>(col.data());
    if (!(v[0] == T(0))) return false;
    for (int k = 1; k <= r; ++k)
        if (!(v[k] == v[1] * T(k * k))) return false;
    return true;
}

ginf_status table_radius(Call &c, Prepared &P, int &radius, int &exact) {
    const int L = P.f.L;
    std::vector<unsigned char> col((size_t)L * P.f.t_size);
    // V(0,k) = V[L*k]: one element per table row.
    GINF_CK(cudaMemcpy2DAsync(col.data(), P.f.t_size, P.Vt, (size_t)L * P.f.t_size, P.f.t_size, L,
                              cudaMemcpyDeviceToHost, c.r.stream));
    GINF_CK(cudaStreamSynchronize(c.r.stream));
    radius = P.f.ctype == CT_F64 ? quad_radius_host<double>(col, L) : quad_radius_host<float>(col, L);
    exact = 0;
    if (P.f.ctype == CT_F32 && radius <= 4) exact = quad_exact_host<float>(col, radius) ? 1 : 0;
    return GINF_OK;
}

// Bytes a half-sweep must move through HBM: per updated node its costs and
// four incoming messages in, four outgoing messages out.
int64_t sweep_alg_bytes(const RecordFormat &f, const Level &lv) {
    const int64_t nodes = (int64_t)(lv.W - 2) * (lv.H - 2) / 2;
    return nodes * ((int64_t)f.d_bytes + 8 * (int64_t)f.m_bytes);
}

// The HBP level loop on prepared records, levels `from` down to `to`:
// bp.cc:121-166 (bp.cu:180-205).  Level `from` starts from zero messages at
// the top of the pyramid, from the coarser level otherwise, or from the
// messages already in its records when top_initialised.
ginf_status run_levels(Call &c, Prepared &P, int iters, int64_t &nli, int from, int to, bool top_initialised) {
    const RecordFormat &f = P.f;
    cudaStream_t s = c.r.stream;
    int radius = 9, quad_exact = 0;
    if (c.r.mode == MODE_STD_QUAD) GINF_TRY(table_radius(c, P, radius, quad_exact));
    const int T = (int)P.lv.size();
    const bool stale = c.r.decode == GINF_DECODE_STALE;
    const int W0 = P.lv[0].W, H0 = P.lv[0].H;
    // Nodes a level-0 colour never updates keep the argmin of a zero belief.
    if (to == 0 && stale && iters < 2 && W0 >= 3 && H0 >= 3) {
        GINF_CK(launch_fill_interior(P.lab, W0, H0, 0, s));
        ++c.launches;
    }
    for (int t = from; t >= to; --t) {
        const Level &lv = P.lv[t];
        unsigned char *rec = P.rec + lv.off;
        const bool interior = lv.W >= 3 && lv.H >= 3;
        // Two or more half-sweeps write every slot an interior sender owns, so
        // the first sweep can read its inputs straight from the coarser level
        // (or as zeros at the top) and no initialisation pass is needed.
        const bool fused = iters >= 2 && interior;
        int first = RD_OWN;
        if (t == from && top_initialised) {
            first = RD_OWN;
        } else if (t == T - 1) {
            if (fused) first = RD_ZERO;
            else {
                GINF_CK(launch_init_messages(f, rec, lv.W, lv.H, nullptr, 0, 0, s));
                ++c.launches;
            }
        } else {
            const Level &cl = P.lv[t + 1];
            if (fused) first = RD_COARSE;
            else {
                GINF_CK(launch_init_messages(f, rec, lv.W, lv.H, P.rec + cl.off, cl.W, cl.H, s));
                ++c.launches;
            }
        }
        if (t == 0) c.ev(EV_L0_START);
        if (!interior) continue;
        const int n1 = (lv.W - 3) / 2 + 1;
        SweepParams p{};
        p.W = lv.W;
        p.H = lv.H;
        p.L = f.L;
        p.Lp = f.Lp;
        p.rec_bytes = f.rec_bytes;
        p.d_bytes = f.d_bytes;
        p.m_bytes = f.m_bytes;
        p.slot_bytes = f.slot_bytes;
        p.rec = rec;
        if (t + 1 < T) {
            p.crec = P.rec + P.lv[t + 1].off;
            p.cW = P.lv[t + 1].W;
            p.cH = P.lv[t + 1].H;
        }
        p.mode = c.r.mode;
        p.norm_min = c.r.norm_min;
        p.V = P.Vt;
        p.labels = P.lab;
        p.quad_radius = radius;
        p.quad_exact = quad_exact;
        p.tiles_per_row = (n1 + c.r.cfg.nt - 1) / c.r.cfg.nt;
        p.num_tiles = (lv.H - 2) * p.tiles_per_row;
        p.status = P.status;
        // Half-sweeps [0, it_end) run one per launch; the rest, when the level
        // qualifies, several per launch in an even number of temporal-blocking
        // launches that alternate between the records and the second buffer
        // (so the level ends in its own records).  A level fed from the
        // coarser one takes its first half-sweep one per launch.
        int it_end = iters;
        int nlaunch = 0, kmax = 0;
        if (P.rec2 && iters >= 2) {
            const int start = first == RD_COARSE ? 1 : 0;
            const int rem = iters - start;
            kmax = std::min(c.r.cluster_k, cluster_sweep_max_halo(f.L));
            nlaunch = (rem + kmax - 1) / kmax;
            if (nlaunch % 2) ++nlaunch;
            if (rem >= 2 && nlaunch <= rem) it_end = start;
            else nlaunch = 0;
        }
        for (int it = 0; it < it_end; ++it) {
            p.iter = it;
            p.read_mode = it == 0 ? first : RD_OWN;
            p.write_labels = (t == 0 && stale && it >= iters - 2) ? 1 : 0;
            GINF_CK(launch_sweep(f, c.r.cfg, p, s, c.ws->num_sms));
            ++c.launches;
            if (t == 0 && c.stats) {
                ++c.stats->level0_sweep_launches;
                c.stats->level0_alg_bytes += sweep_alg_bytes(f, lv);
            }
        }
        if (nlaunch > 0) {
            ClusterSweepParams q{};
            q.W = lv.W;
            q.H = lv.H;
            q.L = f.L;
            q.rec_bytes = f.rec_bytes;
            q.d_bytes = f.d_bytes;
            q.m_bytes = f.m_bytes;
            q.slot_bytes = f.slot_bytes;
            q.from_stride = cluster_from_stride(f);
            q.norm_min = c.r.norm_min;
            q.V = P.Vt;
            q.labels = P.lab;
            q.status = P.status;
            q.label_from = (t == 0 && stale) ? iters - 2 : INT_MAX;
            const int rem = iters - it_end;
            int it0 = it_end;
            for (int l = 0; l < nlaunch; ++l) {
                q.k = rem / nlaunch + (l < rem % nlaunch ? 1 : 0);
                q.iter0 = it0;
                q.rec_in = l % 2 == 0 ? rec : P.rec2;
                q.rec_out = l % 2 == 0 ? P.rec2 : rec;
                q.write_d = l == 0 ? 1 : 0;
                q.read_mode = (l == 0 && it_end == 0 && first == RD_ZERO) ? RD_ZERO : RD_OWN;
                GINF_CK(launch_cluster_sweeps(f, q, s));
                ++c.launches;
                if (t == 0 && c.stats) {
                    ++c.stats->level0_sweep_launches;
                    c.stats->level0_alg_bytes += q.k * sweep_alg_bytes(f, lv);
                }
                it0 += q.k;
            }
        }
        nli += (int64_t)lv.W * lv.H * f.L * iters;
    }
    if (to == 0) {
        if (!stale && W0 >= 3 && H0 >= 3) {
            GINF_CK(launch_decode_fresh(f, P.rec, W0, H0, P.lab, s));
            ++c.launches;
        }
        c.ev(EV_SWEEPS);
    }
    return GINF_OK;
}

ginf_status run_bp(Call &c, Prepared &P, int iters, int64_t &nli) {
    nli = 0;
    return run_levels(c, P, iters, nli, (int)P.lv.size() - 1, 0, false);
}

// Jacobi ICM (icm.cc:4-38) from P.lab, result in P.lab.
ginf_status run_icm_sync(Call &c, Prepared &P, int iters) {
    const int W = c.g->width, H = c.g->height;
    const size_t lab_bytes = (size_t)W * H * sizeof(int32_t);
    cudaStream_t s = c.r.stream;
    if (iters <= 0 || W < 3 || H < 3) return GINF_OK;
    GINF_CK(cudaMemcpyAsync(P.lab2, P.lab, lab_bytes, cudaMemcpyDeviceToDevice, s));
    const size_t plane = (size_t)W * H;
    GINF_CK(cudaMemsetAsync(P.chg, 0, 2 * plane, s));
    int32_t *src = P.lab, *dst = P.lab2;
    for (int it = 0; it < iters; ++it) {
        // Sweep it reads the flags sweep it-1 wrote (none on the first).
        const uint8_t *chg_in = it == 0 ? nullptr : P.chg + ((it - 1) & 1) * plane;
        uint8_t *chg_out = P.chg + (it & 1) * plane;
        GINF_CK(launch_icm_sync(P.f, P.rec, W, H, P.Vt, src, dst, chg_in, chg_out, P.status, s));
        ++c.launches;
        std::swap(src, dst);
    }
    if (src != P.lab) GINF_CK(cudaMemcpyAsync(P.lab, src, lab_bytes, cudaMemcpyDeviceToDevice, s));
    return GINF_OK;
}

ginf_status run_icm_async(Call &c, Prepared &P, int iters) {
    const int W = c.g->width, H = c.g->height;
    if (iters <= 0 || W < 3 || H < 3) return GINF_OK;
    for (int it = 0; it < iters; ++it)
        for (int diag = 2; diag <= (W - 2) + (H - 2); ++diag) {
            GINF_CK(launch_icm_async_diag(P.f, P.rec, W, H, P.Vt, P.lab, diag, P.status, c.r.stream));
            ++c.launches;
        }
    return GINF_OK;
}

ginf_status run_energy(Call &c, Prepared &P) {
    const int W = c.g->width, H = c.g->height;
    GINF_CK(launch_energy(P.f.ctype, P.rec, P.f.rec_bytes / P.f.t_size, 1, W, H, P.f.L, P.Vt, P.lab, P.partials,
                          P.num_partials, P.energy, P.status, c.r.stream));
    c.launches += 2;
    return GINF_OK;
}

// Drains the stream, reads the device status word, fills the stats.
ginf_status finish(Call &c, int64_t nli) {
    cudaStream_t s = c.r.stream;
    GINF_CK(cudaStreamSynchronize(s));
    if (c.stats) {
        ginf_stats *st = c.stats;
        auto ms = [&](int a, int b) {
            float v = 0.f;
            if (cudaEventElapsedTime(&v, c.ws->ev[a], c.ws->ev[b]) != cudaSuccess) {
                cudaGetLastError();
                return 0.0;
            }
            return (double)v;
        };
        st->total_ms = ms(EV_START, EV_END);
        st->upload_ms = ms(EV_START, EV_UPLOAD);
        st->prepare_ms = ms(EV_UPLOAD, EV_PREPARE);
        st->sweep_ms = ms(EV_PREPARE, EV_SWEEPS);
        st->level0_sweep_ms = ms(EV_L0_START, EV_SWEEPS);
        st->icm_ms = ms(EV_SWEEPS, EV_ICM);
        st->energy_ms = ms(EV_ICM, EV_ENERGY);
        st->download_ms = ms(EV_ENERGY, EV_END);
        st->kernel_launches = c.launches;
        st->node_label_iters = nli;
        st->h2d_bytes = c.h2d;
        st->d2h_bytes = c.d2h;
    }
    return GINF_OK;
}

ginf_status read_status(Call &c, Prepared &P) {
    GINF_CK(cudaMemcpyAsync(c.ws->status_host, P.status, sizeof(int), cudaMemcpyDeviceToHost, c.r.stream));
    GINF_CK(cudaStreamSynchronize(c.r.stream));
    return device_status_error(*c.ws->status_host);
}

// Completion of a stream-ordered call, run by CUDA behind the call's work.
struct Completion {
    ginf_workspace *ws;
    double *energy_out;
};

void CUDART_CB on_complete(void *p) {
    Completion *d = static_cast<Completion *>(p);
    const int st = *d->ws->status_host;
    if (st) d->ws->deferred.fetch_or(st);
    if (d->energy_out) *d->energy_out = *d->ws->energy_host;
    delete d;
}

// Ends a call.  A synchronous call waits for its stream and reports the
// device status; a stream-ordered call queues the status read (and the hand-
// over of the energy to *energy_out) behind its work and returns at once.
ginf_status complete(Call &c, Prepared &P, int64_t nli, double *energy_out) {
    if (!c.r.async) {
        GINF_TRY(read_status(c, P));
        if (energy_out) *energy_out = *c.ws->energy_host;
        return finish(c, nli);
    }
    cudaStream_t s = c.r.stream;
    GINF_CK(cudaMemcpyAsync(c.ws->status_host, P.status, sizeof(int), cudaMemcpyDeviceToHost, s));
    Completion *d = new Completion{c.ws, energy_out};
    cudaError_t e = cudaLaunchHostFunc(s, on_complete, d);
    if (e != cudaSuccess) {
        delete d;
        return cuda_fail(e, "cudaLaunchHostFunc");
    }
    GINF_CK(cudaEventRecord(c.ws->done, s));
    c.ws->pending = true;
    return GINF_OK;
}

// A stream-ordered call needs a caller-owned workspace and no stats.
ginf_status check_async(const Call &c, const ginf_workspace *wsp) {
    if (!c.r.async) return GINF_OK;
    if (!wsp) return fail(GINF_ERR_INVALID_ARGUMENT, "a stream-ordered call needs a workspace");
    if (c.stats) return fail(GINF_ERR_INVALID_ARGUMENT, "a stream-ordered call takes no stats");
    return GINF_OK;
}

void begin(Call &c) {
    if (c.stats) {
        std::memset(c.stats, 0, sizeof(ginf_stats));
        c.ev(EV_START);
    }
}

ginf_status labels_to_caller(Call &c, Prepared &P, int32_t *labels, bool interior_only) {
    const ginf_grid *g = c.g;
    if (g->memory != GINF_HOST) return GINF_OK;  // written in place
    const int W = g->width, H = g->height;
    cudaStream_t s = c.r.stream;
    if (interior_only) {
        if (W < 3 || H < 3) return GINF_OK;
        GINF_CK(cudaMemcpy2DAsync(labels + W + 1, W * sizeof(int32_t), P.lab + W + 1, W * sizeof(int32_t),
                                  (W - 2) * sizeof(int32_t), H - 2, cudaMemcpyDeviceToHost, s));
        c.d2h += (int64_t)(W - 2) * (H - 2) * 4;
    } else {
        GINF_CK(cudaMemcpyAsync(labels, P.lab, (size_t)W * H * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
        c.d2h += (int64_t)W * H * 4;
    }
    return GINF_OK;
}

ginf_status export_msgs(Call &c, Prepared &P, const ginf_options *o) {
    if (!o || !o->msgs_out) return GINF_OK;
    const ginf_grid *g = c.g;
    const int W = g->width, H = g->height, L = g->num_labels;
    const size_t bytes = (size_t)W * H * 4 * L * P.f.t_size;
    cudaStream_t s = c.r.stream;
    if (g->memory == GINF_DEVICE) {
        GINF_CK(launch_export_messages(P.f, P.rec, W, H, o->msgs_out, s));
        ++c.launches;
        return GINF_OK;
    }
    void *tmp = nullptr;
    GINF_CK(cudaMallocAsync(&tmp, bytes, s));
    cudaError_t e = launch_export_messages(P.f, P.rec, W, H, tmp, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(o->msgs_out, tmp, bytes, cudaMemcpyDeviceToHost, s);
    cudaFreeAsync(tmp, s);
    if (e != cudaSuccess) return cuda_fail(e, "message export");
    ++c.launches;
    c.d2h += bytes;
    return GINF_OK;
}

}  // namespace

void ginf_gpu::set_last_error(const char *msg) { g_last_error = msg; }

// ===========================================================================
// C ABI

extern "C" {

const char *ginf_version(void) { return "gridinfcuda-gb300 0.1 (sm_103a)"; }

const char *ginf_last_error(void) { return g_last_error.c_str(); }

void ginf_default_options(ginf_options *opt) {
    if (!opt) return;
    std::memset(opt, 0, sizeof(*opt));
    opt->msg_rule = GINF_RULE_REFERENCE;
    opt->msg_store = GINF_STORE_NATIVE;
    opt->decode = GINF_DECODE_STALE;
    opt->normalize = GINF_NORM_MEAN;
    opt->compute_type = -1;
}

ginf_status ginf_workspace_create(ginf_workspace **ws) {
    if (!ws) return fail(GINF_ERR_INVALID_ARGUMENT, "ws is NULL");
    *ws = new ginf_workspace();
    return GINF_OK;
}

ginf_status ginf_workspace_sync(ginf_workspace *ws) {
    g_last_error.clear();
    if (!ws) return fail(GINF_ERR_INVALID_ARGUMENT, "ws is NULL");
    if (ws->pending) {
        GINF_CK(cudaEventSynchronize(ws->done));
        ws->pending = false;
    }
    return device_status_error(ws->deferred.exchange(0));
}

ginf_status ginf_workspace_destroy(ginf_workspace *ws) {
    if (!ws) return GINF_OK;
    if (ws->pending) cudaEventSynchronize(ws->done);
    if (ws->arena) cudaFree(ws->arena);
    if (ws->status_host) cudaFreeHost(ws->status_host);
    if (ws->events) {
        for (int i = 0; i < EV_COUNT; ++i) cudaEventDestroy(ws->ev[i]);
        cudaEventDestroy(ws->done);
    }
    delete ws;
    return GINF_OK;
}

ginf_status ginf_decode_hbp(ginf_workspace *wsp, const ginf_grid *grid, int32_t num_levels, int32_t iters_per_level,
                            int32_t *labels, const ginf_options *opt, ginf_stats *stats) {
    g_last_error.clear();
    GINF_TRY(check_grid(grid));
    if (num_levels < 1) return fail(GINF_ERR_INVALID_ARGUMENT, "num_levels must be >= 1");
    if (iters_per_level < 0) return fail(GINF_ERR_INVALID_ARGUMENT, "iters_per_level must be >= 0");
    if (!labels) return fail(GINF_ERR_INVALID_ARGUMENT, "labels is NULL");
    Call c;
    GINF_TRY(resolve(grid, opt, c.r));
    if (grid->num_labels > kMaxLabels)
        return fail(GINF_ERR_UNSUPPORTED, "num_labels above " + std::to_string(kMaxLabels) + " is not compiled in");
    WsGuard guard(wsp);
    c.ws = guard.ws;
    c.g = grid;
    c.stats = stats;
    GINF_TRY(check_async(c, wsp));
    GINF_TRY(ws_init(c.ws, c.r.stream));
    begin(c);
    Prepared P;
    const bool host = grid->memory == GINF_HOST;
    // Device labels: the caller's buffer, or a copy holding the caller's labels
    // so the untouched border goes back unchanged.
    GINF_TRY(prepare(c, P, num_levels, false, nullptr, host ? nullptr : labels));
    int64_t nli = 0;
    GINF_TRY(run_bp(c, P, iters_per_level, nli));
    c.ev(EV_ICM);
    c.ev(EV_ENERGY);
    GINF_TRY(export_msgs(c, P, opt));
    GINF_TRY(labels_to_caller(c, P, labels, true));
    c.ev(EV_END);
    return complete(c, P, nli, nullptr);
}

ginf_status ginf_decode_icm(ginf_workspace *wsp, const ginf_grid *grid, const int32_t *initial, int32_t iters,
                            int32_t asynchronous, int32_t *result, const ginf_options *opt, ginf_stats *stats) {
    g_last_error.clear();
    GINF_TRY(check_grid(grid));
    if (!initial || !result) return fail(GINF_ERR_INVALID_ARGUMENT, "initial / result is NULL");
    if (iters < 0) return fail(GINF_ERR_INVALID_ARGUMENT, "iters must be >= 0");
    Call c;
    GINF_TRY(resolve(grid, opt, c.r));
    WsGuard guard(wsp);
    c.ws = guard.ws;
    c.g = grid;
    c.stats = stats;
    GINF_TRY(ws_init(c.ws, c.r.stream));
    begin(c);
    Prepared P;
    const bool host = grid->memory == GINF_HOST;
    GINF_TRY(prepare(c, P, 0, !asynchronous, initial, host ? nullptr : result));
    c.ev(EV_L0_START);
    c.ev(EV_SWEEPS);
    if (asynchronous) GINF_TRY(run_icm_async(c, P, iters));
    else GINF_TRY(run_icm_sync(c, P, iters));
    c.ev(EV_ICM);
    c.ev(EV_ENERGY);
    GINF_TRY(labels_to_caller(c, P, result, false));
    c.ev(EV_END);
    GINF_TRY(read_status(c, P));
    return finish(c, 0);
}

ginf_status ginf_decode_alpha_beta(ginf_workspace *wsp, const ginf_grid *grid, const int32_t *initial, int32_t iters,
                                   int32_t *result, const ginf_options *opt, ginf_stats *stats) {
    g_last_error.clear();
    GINF_TRY(check_grid(grid));
    if (!initial || !result) return fail(GINF_ERR_INVALID_ARGUMENT, "initial / result is NULL");
    if (iters < 0) return fail(GINF_ERR_INVALID_ARGUMENT, "iters must be >= 0");
    if (grid->cost_type != GINF_I32)
        return fail(GINF_ERR_UNSUPPORTED,
                    "the alpha-beta swap takes int32 grids (the reference instantiates it for int only)");
    const int W = grid->width, H = grid->height, L = grid->num_labels;
    const size_t N = (size_t)W * H;
    if (N > (size_t)0x7ffffff0) return fail(GINF_ERR_INVALID_ARGUMENT, "grid too large for int32 heights");
    Call c;
    GINF_TRY(resolve(grid, opt, c.r));
    WsGuard guard(wsp);
    c.ws = guard.ws;
    c.g = grid;
    c.stats = stats;
    GINF_TRY(ws_init(c.ws, c.r.stream));
    begin(c);
    const bool host = grid->memory == GINF_HOST;
    const size_t cost_bytes = N * L * sizeof(int32_t), table_bytes = (size_t)L * L * sizeof(int32_t);
    const size_t lab = N * sizeof(int32_t);
    Arena a;
    const size_t id_d = host ? a.add(cost_bytes) : 0;
    const size_t id_v = host ? a.add(table_bytes) : 0;
    const size_t id_res = a.add(lab);
    const size_t id_zero = a.add(8 * lab);  // excess, height, six residue slots: zeroed together
    const size_t id_scr = a.add(4 * lab);   // newResult, distances, two frontiers
    const size_t id_st = a.add(64);
    GINF_TRY(ws_reserve(c.ws, a.total()));
    unsigned char *base = c.ws->arena;
    cudaStream_t s = c.r.stream;
    AlphaBetaParams p{};
    p.W = W;
    p.H = H;
    p.L = L;
    p.D = static_cast<const int32_t *>(grid->data_costs);
    p.V = static_cast<const int32_t *>(grid->sm_costs);
    if (host) {
        GINF_CK(cudaMemcpyAsync(a.ptr(base, id_d), grid->data_costs, cost_bytes, cudaMemcpyHostToDevice, s));
        GINF_CK(cudaMemcpyAsync(a.ptr(base, id_v), grid->sm_costs, table_bytes, cudaMemcpyHostToDevice, s));
        p.D = reinterpret_cast<const int32_t *>(a.ptr(base, id_d));
        p.V = reinterpret_cast<const int32_t *>(a.ptr(base, id_v));
        c.h2d += cost_bytes + table_bytes + lab;
    }
    p.result = reinterpret_cast<int32_t *>(a.ptr(base, id_res));
    int32_t *zero = reinterpret_cast<int32_t *>(a.ptr(base, id_zero));
    p.excess = zero;
    p.height = zero + N;
    p.res = zero + 2 * N;
    int32_t *scr = reinterpret_cast<int32_t *>(a.ptr(base, id_scr));
    p.newr = scr;
    p.dist = scr + N;
    p.q0 = scr + 2 * N;
    p.q1 = scr + 3 * N;
    p.iters = iters;
    p.status = reinterpret_cast<int *>(a.ptr(base, id_st));
    GINF_CK(cudaMemcpyAsync(p.result, initial, lab, host ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice, s));
    // The reference's excess, height and residue matrices start at zero
    // (src/matrix.cc:21-27) and keep their values from one label pair to the
    // next.
    GINF_CK(cudaMemsetAsync(zero, 0, 8 * lab, s));
    GINF_CK(cudaMemsetAsync(p.status, 0, sizeof(int), s));
    c.ev(EV_UPLOAD);
    c.ev(EV_PREPARE);
    c.ev(EV_L0_START);
    c.ev(EV_SWEEPS);
    GINF_CK(launch_alpha_beta(p, s));
    ++c.launches;
    c.ev(EV_ICM);
    c.ev(EV_ENERGY);
    GINF_CK(cudaMemcpyAsync(result, p.result, lab, host ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice, s));
    if (host) c.d2h += lab;
    c.ev(EV_END);
    GINF_CK(cudaMemcpyAsync(c.ws->status_host, p.status, sizeof(int), cudaMemcpyDeviceToHost, s));
    GINF_CK(cudaStreamSynchronize(s));
    GINF_TRY(device_status_error(*c.ws->status_host));
    return finish(c, 0);
}

ginf_status ginf_energy(ginf_workspace *wsp, const ginf_grid *grid, const int32_t *labels, double *energy,
                        const ginf_options *opt) {
    g_last_error.clear();
    GINF_TRY(check_grid(grid));
    if (!labels || !energy) return fail(GINF_ERR_INVALID_ARGUMENT, "labels / energy is NULL");
    Call c;
    GINF_TRY(resolve(grid, opt, c.r));
    WsGuard guard(wsp);
    c.ws = guard.ws;
    c.g = grid;
    c.stats = nullptr;
    GINF_TRY(ws_init(c.ws, c.r.stream));
    const int W = grid->width, H = grid->height, L = grid->num_labels;
    const bool host = grid->memory == GINF_HOST;
    const size_t ts = type_size(grid->cost_type);
    const size_t cost_bytes = (size_t)W * H * L * ts, table_bytes = (size_t)L * L * ts;
    const size_t lab_bytes = (size_t)W * H * sizeof(int32_t);
    const int np = energy_num_partials(W, H);
    Arena a;
    const size_t id_c = host ? a.add(cost_bytes) : 0;
    const size_t id_v = host ? a.add(table_bytes) : 0;
    const size_t id_l = host ? a.add(lab_bytes) : 0;
    const size_t id_p = a.add(sizeof(double) * (np + 1) + 64);
    GINF_TRY(ws_reserve(c.ws, a.total()));
    unsigned char *base = c.ws->arena;
    cudaStream_t s = c.r.stream;
    const void *costs = grid->data_costs, *V = grid->sm_costs;
    const int32_t *lab = labels;
    if (host) {
        void *dc = a.ptr(base, id_c), *dv = a.ptr(base, id_v), *dl = a.ptr(base, id_l);
        GINF_CK(cudaMemcpyAsync(dc, costs, cost_bytes, cudaMemcpyHostToDevice, s));
        GINF_CK(cudaMemcpyAsync(dv, V, table_bytes, cudaMemcpyHostToDevice, s));
        GINF_CK(cudaMemcpyAsync(dl, labels, lab_bytes, cudaMemcpyHostToDevice, s));
        costs = dc;
        V = dv;
        lab = static_cast<const int32_t *>(dl);
    }
    double *partials = reinterpret_cast<double *>(a.ptr(base, id_p));
    int *status = reinterpret_cast<int *>(partials + np);
    double *out = partials + np + 1;
    GINF_CK(cudaMemsetAsync(status, 0, sizeof(int), s));
    GINF_CK(launch_energy(grid->cost_type, costs, 1, (size_t)W * H, W, H, L, V, lab, partials, np, out, status, s));
    GINF_CK(cudaMemcpyAsync(c.ws->energy_host, out, sizeof(double), cudaMemcpyDeviceToHost, s));
    GINF_CK(cudaMemcpyAsync(c.ws->status_host, status, sizeof(int), cudaMemcpyDeviceToHost, s));
    GINF_CK(cudaStreamSynchronize(s));
    if (*c.ws->status_host & DEV_ERR_BOUNDS) return fail(GINF_ERR_INVALID_ARGUMENT, "a label is outside [0, num_labels)");
    *energy = *c.ws->energy_host;
    return GINF_OK;
}

ginf_status ginf_solve(ginf_workspace *wsp, const ginf_grid *grid, int32_t num_levels, int32_t iters_per_level,
                       int32_t icm_iters, int32_t *labels, double *energy, const ginf_options *opt,
                       ginf_stats *stats) {
    g_last_error.clear();
    GINF_TRY(check_grid(grid));
    if (num_levels < 1) return fail(GINF_ERR_INVALID_ARGUMENT, "num_levels must be >= 1");
    if (iters_per_level < 0 || icm_iters < 0) return fail(GINF_ERR_INVALID_ARGUMENT, "iteration counts must be >= 0");
    if (!labels) return fail(GINF_ERR_INVALID_ARGUMENT, "labels is NULL");
    Call c;
    GINF_TRY(resolve(grid, opt, c.r));
    if (grid->num_labels > kMaxLabels)
        return fail(GINF_ERR_UNSUPPORTED, "num_labels above " + std::to_string(kMaxLabels) + " is not compiled in");
    WsGuard guard(wsp);
    c.ws = guard.ws;
    c.g = grid;
    c.stats = stats;
    GINF_TRY(check_async(c, wsp));
    GINF_TRY(ws_init(c.ws, c.r.stream));
    begin(c);
    Prepared P;
    const bool host = grid->memory == GINF_HOST;
    // The caller's labels seed the device copy: ICM reads the border labels.
    GINF_TRY(prepare(c, P, num_levels, true, host ? labels : nullptr, host ? nullptr : labels));
    int64_t nli = 0;
    GINF_TRY(run_bp(c, P, iters_per_level, nli));
    GINF_TRY(run_icm_sync(c, P, icm_iters));
    c.ev(EV_ICM);
    GINF_TRY(run_energy(c, P));
    c.ev(EV_ENERGY);
    GINF_TRY(export_msgs(c, P, opt));
    GINF_TRY(labels_to_caller(c, P, labels, true));
    if (energy) {
        GINF_CK(cudaMemcpyAsync(c.ws->energy_host, P.energy, sizeof(double), cudaMemcpyDeviceToHost, c.r.stream));
        c.d2h += sizeof(double);
    }
    c.ev(EV_END);
    return complete(c, P, nli, energy);
}

// The learned warm start needs FP32 arithmetic, the native store and the
// truncated-linear / Potts update.
ginf_status check_learned(const ginf_grid *grid, const Resolved &r) {
    if (r.ctype != GINF_F32 || r.store != ST_NATIVE || r.mode != MODE_LINEAR)
        return fail(GINF_ERR_UNSUPPORTED, "the warm start runs FP32 BP with Potts / truncated-linear smoothness");
    if (grid->memory != GINF_DEVICE) return fail(GINF_ERR_INVALID_ARGUMENT, "the warm start takes device buffers");
    return GINF_OK;
}

ginf_status ginf_hbp_level_state(ginf_workspace *wsp, const ginf_grid *grid, int32_t num_levels,
                                 int32_t iters_per_level, int32_t level, int32_t target, float *x_out,
                                 float *beliefs_out, const ginf_options *opt) {
    g_last_error.clear();
    GINF_TRY(check_grid(grid));
    if (num_levels < 1 || level < 0 || level >= num_levels || iters_per_level < 0)
        return fail(GINF_ERR_INVALID_ARGUMENT, "need 0 <= level < num_levels and iters_per_level >= 0");
    Call c;
    GINF_TRY(resolve(grid, opt, c.r));
    GINF_TRY(check_learned(grid, c.r));
    if (grid->num_labels > kMaxLabels) return fail(GINF_ERR_UNSUPPORTED, "too many labels");
    WsGuard guard(wsp);
    c.ws = guard.ws;
    c.g = grid;
    c.stats = nullptr;
    GINF_TRY(ws_init(c.ws, c.r.stream));
    Prepared P;
    GINF_TRY(prepare(c, P, num_levels, false, nullptr, nullptr));
    const Level &lt = P.lv[level];
    const float scale = (float)(1u << (2 * level));
    if (x_out) GINF_CK(launch_level_x(P.f, P.rec + lt.off, lt.W, lt.H, scale, x_out, c.r.stream));
    if (beliefs_out) {
        int64_t nli = 0;
        if (target == 1) {
            // the whole schedule, then the level-0 message sums averaged per block
            GINF_TRY(run_levels(c, P, iters_per_level, nli, num_levels - 1, 0, false));
            GINF_CK(launch_project_fine(P.f, P.rec, P.lv[0].W, P.lv[0].H, P.rec + lt.off, lt.W, lt.H, level,
                                        beliefs_out, c.r.stream));
        } else {
            GINF_TRY(run_levels(c, P, iters_per_level, nli, num_levels - 1, level, false));
            GINF_CK(launch_level_beliefs(P.f, P.rec + lt.off, lt.W, lt.H, scale, beliefs_out, c.r.stream));
        }
    }
    GINF_TRY(read_status(c, P));
    return GINF_OK;
}

// Level-0 energy of the labelling level t hands down (each level-0 node
// takes its block's argmin of D_t / 4^t + incoming messages); into dst
// (device double).
ginf_status handed_down_energy(Call &c, Prepared &P, int t, int32_t *lab_t, int32_t *lab0, double *partials, int np,
                               double *dst) {
    const Level &lt = P.lv[t];
    const Level &l0 = P.lv[0];
    cudaStream_t s = c.r.stream;
    GINF_CK(launch_fine_labels(P.f, P.rec + lt.off, lt.W, lt.H, t, lab_t, lab0, l0.W, l0.H, s));
    GINF_CK(launch_energy(P.f.ctype, P.rec, P.f.rec_bytes / P.f.t_size, 1, l0.W, l0.H, P.f.L, P.Vt, lab0, partials,
                          np, dst, P.status, s));
    c.launches += 4;
    return GINF_OK;
}

}  // extern "C"

// Hierarchical BP with level t seeded from a prediction: by the network when
// net is given (pred is then NULL), else from the caller's device buffer pred
// ([H_t][W_t][L], the network's output scale).
static ginf_status decode_hbp_seeded(ginf_workspace *wsp, const ginf_grid *grid, int32_t num_levels,
                                     int32_t iters_per_level, int32_t warm_level, int32_t warm_iters,
                                     int32_t mid_iters, ginf_warmnet *net, const float *pred, int32_t fallback,
                                     int32_t *labels, const ginf_options *opt, ginf_stats *stats) {
    g_last_error.clear();
    GINF_TRY(check_grid(grid));
    if ((!net && !pred) || !labels) return fail(GINF_ERR_INVALID_ARGUMENT, "prediction / labels is NULL");
    if (num_levels < 2 || warm_level < 1 || warm_level >= num_levels || iters_per_level < 0 || warm_iters < 0)
        return fail(GINF_ERR_INVALID_ARGUMENT, "need 1 <= warm_level < num_levels and iteration counts >= 0");
    if (net && warmnet_labels(net) != grid->num_labels)
        return fail(GINF_ERR_INVALID_ARGUMENT, "the network was built for another label count");
    Call c;
    GINF_TRY(resolve(grid, opt, c.r));
    GINF_TRY(check_learned(grid, c.r));
    WsGuard guard(wsp);
    c.ws = guard.ws;
    c.g = grid;
    c.stats = stats;
    GINF_TRY(ws_init(c.ws, c.r.stream));
    begin(c);
    Prepared P;
    GINF_TRY(prepare(c, P, num_levels, false, nullptr, labels));
    cudaStream_t s = c.r.stream;
    const int t = warm_level;
    const int sl = t + 1;  // the cold screening level
    if (fallback && sl > num_levels - 1)
        return fail(GINF_ERR_INVALID_ARGUMENT, "the fallback needs a pyramid level above warm_level");
    const Level &lt = P.lv[t];
    const Level &l0 = P.lv[0];
    const size_t nx = (size_t)lt.W * lt.H * P.f.L;
    const int np = energy_num_partials(l0.W, l0.H);
    const size_t lab_s_bytes = fallback ? align_up((size_t)P.lv[sl].W * P.lv[sl].H * sizeof(int32_t), 256) : 0;
    const size_t lab0_bytes = fallback ? align_up((size_t)l0.W * l0.H * sizeof(int32_t), 256) : 0;
    unsigned char *scratch = nullptr;
    const size_t scratch_bytes = align_up(nx * sizeof(float), 256) + lab_s_bytes + lab0_bytes + sizeof(double) * (np + 2);
    GINF_CK(cudaMallocAsync(reinterpret_cast<void **>(&scratch), scratch_bytes, s));
    float *x = reinterpret_cast<float *>(scratch);
    int32_t *lab_s = reinterpret_cast<int32_t *>(scratch + align_up(nx * sizeof(float), 256));
    int32_t *lab0 = reinterpret_cast<int32_t *>(reinterpret_cast<unsigned char *>(lab_s) + lab_s_bytes);
    double *partials = reinterpret_cast<double *>(reinterpret_cast<unsigned char *>(lab0) + lab0_bytes);
    double *energies = partials + np;  // [cold screen, warm result]
    ginf_status st = GINF_OK;
    int64_t nli = 0;
    float *y = const_cast<float *>(pred);
    double e_host[2] = {0.0, 0.0};
    const float scale = (float)(1u << (2 * t));
    bool warm = true;
    if (mid_iters < 0) mid_iters = iters_per_level;
    do {
        cudaError_t e;
        if (fallback) {
            // Cold schedule down to the level above the seeded one (cheap):
            // its handed-down labelling is the bar the seeded result must meet,
            // and its state is where the cold fallback resumes.
            if ((st = run_levels(c, P, iters_per_level, nli, num_levels - 1, sl, false)) != GINF_OK) break;
            if ((st = handed_down_energy(c, P, sl, lab_s, lab0, partials, np, energies)) != GINF_OK) break;
        }
        // Network input and prediction at level t.
        if ((e = launch_level_x(P.f, P.rec + lt.off, lt.W, lt.H, scale, x, s)) != cudaSuccess) {
            st = cuda_fail(e, "level costs");
            break;
        }
        ++c.launches;
        if (net) {
            if ((st = warmnet_forward(net, x, 1, lt.H, lt.W, &y, P.status, s)) != GINF_OK) break;
            c.launches += 5;
        }
        // Seeded path: level-t messages from the prediction, its own sweeps,
        // then the finer levels.
        if ((e = launch_warm_init(P.f, P.rec + lt.off, lt.W, lt.H, y, x, scale / 4.f, s)) != cudaSuccess) {
            st = cuda_fail(e, "warm init");
            break;
        }
        ++c.launches;
        if (warm_iters > 0 && (st = run_levels(c, P, warm_iters, nli, t, t, true)) != GINF_OK) break;
        if (t > 1 && (st = run_levels(c, P, mid_iters, nli, t - 1, 1, false)) != GINF_OK) break;
        if ((st = run_levels(c, P, iters_per_level, nli, 0, 0, false)) != GINF_OK) break;
        if (fallback) {
            if ((e = launch_energy(P.f.ctype, P.rec, P.f.rec_bytes / P.f.t_size, 1, l0.W, l0.H, P.f.L, P.Vt, P.lab,
                                   partials, np, energies + 1, P.status, s)) != cudaSuccess ||
                (e = cudaMemcpyAsync(e_host, energies, 2 * sizeof(double), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
                (e = cudaStreamSynchronize(s)) != cudaSuccess) {
                st = cuda_fail(e, "seeded energy");
                break;
            }
            c.launches += 2;
            // A seeded result above the cold coarse labelling's energy is
            // discarded: the cold schedule resumes below the screening level,
            // which gives exactly the plain hierarchical result.
            warm = e_host[1] <= e_host[0];
            if (!warm && (st = run_levels(c, P, iters_per_level, nli, sl - 1, 0, false)) != GINF_OK) break;
        }
    } while (false);
    cudaFreeAsync(scratch, s);
    if (st != GINF_OK) return st;
    c.ev(EV_ICM);
    c.ev(EV_ENERGY);
    GINF_TRY(labels_to_caller(c, P, labels, true));
    c.ev(EV_END);
    GINF_TRY(read_status(c, P));
    st = finish(c, nli);
    if (stats) stats->warm_start_used = warm ? 1 : 0;
    return st;
}

extern "C" {

ginf_status ginf_decode_hbp_learned(ginf_workspace *wsp, const ginf_grid *grid, int32_t num_levels,
                                    int32_t iters_per_level, int32_t warm_level, int32_t warm_iters,
                                    int32_t mid_iters, ginf_warmnet *net, int32_t *labels, const ginf_options *opt,
                                    ginf_stats *stats) {
    if (!net) return fail(GINF_ERR_INVALID_ARGUMENT, "net is NULL");
    return decode_hbp_seeded(wsp, grid, num_levels, iters_per_level, warm_level, warm_iters, mid_iters, net, nullptr,
                             1, labels, opt, stats);
}

ginf_status ginf_decode_hbp_warm(ginf_workspace *wsp, const ginf_grid *grid, int32_t num_levels,
                                 int32_t iters_per_level, int32_t warm_level, int32_t warm_iters, int32_t mid_iters,
                                 const float *prediction, int32_t fallback, int32_t *labels, const ginf_options *opt,
                                 ginf_stats *stats) {
    if (!prediction) return fail(GINF_ERR_INVALID_ARGUMENT, "prediction is NULL");
    return decode_hbp_seeded(wsp, grid, num_levels, iters_per_level, warm_level, warm_iters, mid_iters, nullptr,
                             prediction, fallback, labels, opt, stats);
}

ginf_status ginf_stereo_costs(int32_t width, int32_t height, int32_t num_labels, int32_t memory, const float *left,
                              const float *right, float coef, float cap, float *costs, void *stream) {
    g_last_error.clear();
    if (width < 1 || height < 1 || num_labels < 1) return fail(GINF_ERR_INVALID_ARGUMENT, "bad size");
    if (!left || !right || !costs) return fail(GINF_ERR_INVALID_ARGUMENT, "NULL buffer");
    if (memory != GINF_HOST && memory != GINF_DEVICE) return fail(GINF_ERR_INVALID_ARGUMENT, "bad memory kind");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const size_t img = (size_t)width * height * sizeof(float);
    const float *l = left, *r = right;
    float *tmp = nullptr;
    cudaError_t e = cudaSuccess;
    if (memory == GINF_HOST) {
        GINF_CK(cudaMallocAsync(&tmp, 2 * img, s));
        e = cudaMemcpyAsync(tmp, left, img, cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(tmp + (size_t)width * height, right, img, cudaMemcpyHostToDevice, s);
        l = tmp;
        r = tmp + (size_t)width * height;
    }
    if (e == cudaSuccess) e = launch_stereo_costs(width, height, num_labels, l, r, coef, cap, costs, s);
    if (tmp) cudaFreeAsync(tmp, s);  // stream-ordered: after the copies and the kernel
    if (e != cudaSuccess) return cuda_fail(e, "stereo costs");
    GINF_CK(cudaStreamSynchronize(s));
    return GINF_OK;
}

ginf_status ginf_stereo_costs_u8(int32_t width, int32_t height, int32_t num_labels, int32_t memory,
                                 const uint8_t *left, const uint8_t *right, int32_t cap, int32_t *costs,
                                 void *stream) {
    g_last_error.clear();
    if (width < 1 || height < 1 || num_labels < 1) return fail(GINF_ERR_INVALID_ARGUMENT, "bad size");
    if (!left || !right || !costs) return fail(GINF_ERR_INVALID_ARGUMENT, "NULL buffer");
    if (memory != GINF_HOST && memory != GINF_DEVICE) return fail(GINF_ERR_INVALID_ARGUMENT, "bad memory kind");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const size_t img = (size_t)width * height;
    const uint8_t *l = left, *r = right;
    uint8_t *tmp = nullptr;
    cudaError_t e = cudaSuccess;
    if (memory == GINF_HOST) {
        GINF_CK(cudaMallocAsync(&tmp, 2 * img, s));
        e = cudaMemcpyAsync(tmp, left, img, cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess) e = cudaMemcpyAsync(tmp + img, right, img, cudaMemcpyHostToDevice, s);
        l = tmp;
        r = tmp + img;
    }
    if (e == cudaSuccess) e = launch_stereo_costs_u8(width, height, num_labels, l, r, cap, costs, s);
    if (tmp) cudaFreeAsync(tmp, s);
    if (e != cudaSuccess) return cuda_fail(e, "stereo costs");
    GINF_CK(cudaStreamSynchronize(s));
    return GINF_OK;
}

}  // extern "C"
