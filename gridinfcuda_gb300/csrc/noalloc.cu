// noalloc.cu -- loopy BP that allocates no device memory.
//
// Some callers cannot call cudaMalloc while they run: a real-time loop that
// cannot afford the device-wide synchronisation and unbounded latency of
// cudaMalloc/cudaFree, or a plugin inside a host application that owns every
// byte of device memory and hands out only the buffers it manages.  For them
// ginf_decode_bp_noalloc keeps its working set -- the per-node message
// records of one pyramid level and a status word -- in a fixed array in the
// library's own device image instead of a workspace.  The caller still passes
// the costs, the smoothness table and the labels as device buffers.
//
// The array is GINF_NOALLOC_SCRATCH_BYTES (48 MiB) on every GPU that loads
// the library, held until the process exits.  Every call on a device shares
// it and it keeps the last call's contents; each call zeroes the status word
// and (re)initialises every record word it reads, so stale contents never
// leak into a result.  Two calls whose work overlaps on the GPU (different
// streams, or different host threads) race on the array and corrupt each
// other: serialise them.
#include <cstdio>
#include <mutex>

#include "ginf_gb300.h"
#include "ginf_internal.h"

namespace {

static __device__ __align__(256) unsigned char g_noalloc_scratch[GINF_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 128;
constexpr size_t kStatusBytes = 256;  // status word, padded to keep the records 256-byte aligned

struct DeviceSetup {
    bool done = false;
    unsigned char *scratch = nullptr;  // device address of g_noalloc_scratch
    int num_sms = 0;
};

std::mutex g_setup_mutex;
DeviceSetup g_setup[kMaxDevices];

// Host code cannot use g_noalloc_scratch directly (in host code the name is
// only a stand-in); its device address comes from cudaGetSymbolAddress, once
// per device, with that device current.  The address is kept for the life of
// the process: a cudaDeviceReset on that device after the first call would
// leave it stale (the header says so).
ginf_status setup_device(int dev, DeviceSetup &out) {
    if (dev < 0 || dev >= kMaxDevices) {
        ginf_gpu::set_last_error("ginf_decode_bp_noalloc: device ordinal out of range");
        return GINF_ERR_NO_DEVICE;
    }
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    DeviceSetup &s = g_setup[dev];
    if (!s.done) {
        int major = 0, minor = 0, sms = 0;
        if (cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
            cudaGetLastError();
            ginf_gpu::set_last_error("ginf_decode_bp_noalloc: cannot query the device");
            return GINF_ERR_NO_DEVICE;
        }
        if (major * 10 + minor != 103) {
            ginf_gpu::set_last_error("ginf_decode_bp_noalloc: this library is built for sm_103 (GB300)");
            return GINF_ERR_NO_DEVICE;
        }
        void *ptr = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (e != cudaSuccess || ptr == nullptr) {
            cudaGetLastError();
            char msg[160];
            std::snprintf(msg, sizeof(msg), "ginf_decode_bp_noalloc: cudaGetSymbolAddress failed: %s",
                          cudaGetErrorString(e));
            ginf_gpu::set_last_error(msg);
            return GINF_ERR_CUDA;
        }
        s.scratch = static_cast<unsigned char *>(ptr);
        s.num_sms = sms;
        s.done = true;
    }
    out = s;
    return GINF_OK;
}

ginf_status cuda_error(cudaError_t e, const char *what) {
    char msg[200];
    std::snprintf(msg, sizeof(msg), "ginf_decode_bp_noalloc: %s: %s", what, cudaGetErrorString(e));
    ginf_gpu::set_last_error(msg);
    return GINF_ERR_CUDA;
}

}  // namespace

extern "C" ginf_status ginf_decode_bp_noalloc(const ginf_grid *grid, int32_t num_iters, int32_t *labels,
                                              void *stream) {
    using namespace ginf_gpu;
    set_last_error("");
    if (!grid || !labels || !grid->data_costs || !grid->sm_costs) {
        set_last_error("ginf_decode_bp_noalloc: NULL grid, buffer or labels");
        return GINF_ERR_INVALID_ARGUMENT;
    }
    if (grid->memory != GINF_DEVICE) {
        set_last_error("ginf_decode_bp_noalloc: every buffer must be device memory (memory = GINF_DEVICE)");
        return GINF_ERR_INVALID_ARGUMENT;
    }
    const int W = grid->width, H = grid->height, L = grid->num_labels;
    if (W < 1 || H < 1 || L < 2 || L > kMaxLabels || num_iters < 0 ||
        (grid->cost_type != GINF_F32 && grid->cost_type != GINF_I32) || grid->sm_model < GINF_SM_EXPLICIT ||
        grid->sm_model > GINF_SM_TRUNC_QUAD) {
        set_last_error("ginf_decode_bp_noalloc: bad size, label count (2..128), iteration count, type or model");
        return GINF_ERR_INVALID_ARGUMENT;
    }
    const RecordFormat f = make_format(grid->cost_type == GINF_F32 ? CT_F32 : CT_I32, ST_NATIVE, L);
    const size_t need = kStatusBytes + (size_t)W * H * f.rec_bytes;
    if (need > (size_t)GINF_NOALLOC_SCRATCH_BYTES) {
        char msg[240];
        std::snprintf(msg, sizeof(msg),
                      "ginf_decode_bp_noalloc: a %dx%dx%d grid needs %zu bytes of scratch, more than the fixed "
                      "maximum of %u bytes (48 MiB); use ginf_decode_hbp",
                      W, H, L, need, (unsigned)GINF_NOALLOC_SCRATCH_BYTES);
        set_last_error(msg);
        return GINF_ERR_INVALID_ARGUMENT;
    }
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        cudaGetLastError();
        set_last_error("ginf_decode_bp_noalloc: no CUDA device");
        return GINF_ERR_NO_DEVICE;
    }
    DeviceSetup ds;
    const ginf_status st = setup_device(dev, ds);
    if (st != GINF_OK) return st;

    cudaStream_t s = static_cast<cudaStream_t>(stream);
    int *status = reinterpret_cast<int *>(ds.scratch);
    unsigned char *rec = ds.scratch + kStatusBytes;
    const int mode = (grid->sm_model == GINF_SM_POTTS || grid->sm_model == GINF_SM_TRUNC_LINEAR) ? MODE_LINEAR
                                                                                                 : MODE_REF_MINCONV;
    if ((e = cudaMemsetAsync(status, 0, sizeof(int), s)) != cudaSuccess) return cuda_error(e, "status reset");
    if ((e = launch_costs_to_records(f, f.ctype, grid->data_costs, W, H, rec, s)) != cudaSuccess)
        return cuda_error(e, "cost layout");
    const bool interior = W >= 3 && H >= 3;
    const bool fused = num_iters >= 2 && interior;
    if (!fused) {
        // Fewer than two half-sweeps leave messages unwritten: zero them, and
        // give never-updated interior nodes the argmin of a zero belief.
        if ((e = launch_init_messages(f, rec, W, H, nullptr, 0, 0, s)) != cudaSuccess)
            return cuda_error(e, "message init");
        if ((e = launch_fill_interior(labels, W, H, 0, s)) != cudaSuccess) return cuda_error(e, "label init");
    }
    if (interior) {
        SweepParams p{};
        p.W = W;
        p.H = H;
        p.L = L;
        p.Lp = f.Lp;
        p.rec_bytes = f.rec_bytes;
        p.d_bytes = f.d_bytes;
        p.m_bytes = f.m_bytes;
        p.slot_bytes = f.slot_bytes;
        p.rec = rec;
        p.mode = mode;
        p.norm_min = 0;
        p.V = grid->sm_costs;
        p.labels = labels;
        p.status = status;
        const int n1 = (W - 3) / 2 + 1;
        SweepConfig cfg;
        p.tiles_per_row = (n1 + cfg.nt - 1) / cfg.nt;
        p.num_tiles = (H - 2) * p.tiles_per_row;
        for (int it = 0; it < num_iters; ++it) {
            p.iter = it;
            p.read_mode = (it == 0 && fused) ? RD_ZERO : RD_OWN;
            p.write_labels = it >= num_iters - 2 ? 1 : 0;
            if ((e = launch_sweep(f, cfg, p, s, ds.num_sms)) != cudaSuccess) return cuda_error(e, "half-sweep");
        }
    }
    int st_host = 0;
    if ((e = cudaMemcpyAsync(&st_host, status, sizeof(int), cudaMemcpyDeviceToHost, s)) != cudaSuccess)
        return cuda_error(e, "status read");
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_error(e, "synchronise");
    if (st_host & DEV_ERR_TIMEOUT) {
        set_last_error("ginf_decode_bp_noalloc: a device-side wait exceeded its time limit");
        return GINF_ERR_TIMEOUT;
    }
    return GINF_OK;
}
