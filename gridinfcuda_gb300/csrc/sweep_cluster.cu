// sweep_cluster.cu -- several checkerboard half-sweeps per launch (temporal
// blocking) for FP32 grids with L <= 32, on thread-block clusters.
//
// One cluster of cx x cy CTAs (the shape of 4 x 4, 2 x 4, 4 x 2 or 2 x 2
// that keeps the most CTAs resident) holds a region of RW x RH nodes -- both
// colours, every node's whole
// record -- in the distributed shared memory of its CTAs, each CTA a
// bw x bh sub-block.  The region is the cluster's core of
// (RW - 2k) x (RH - 2k) nodes plus a halo k nodes deep, k being the number
// of half-sweeps the launch runs:
//   1. every CTA brings its sub-block's records in from HBM with one bulk
//      (TMA) copy per node, completion counted on an mbarrier;
//   2. half-sweep j = 0 .. k-1 updates the nodes of its colour inside the
//      region shrunk by j on every side (the nodes whose inputs are still
//      exact: the halo's stale messages travel one node per half-sweep), each
//      node exactly as the one-half-sweep kernel does -- belief by the
//      node's four lanes, then lane (node, dir) forms the message towards dir
//      in the reference's operation order (src/bp.cc:7-63) -- and writes it
//      straight into the neighbour's record in shared memory, through the
//      cluster's distributed shared memory when the neighbour belongs to
//      another CTA; one cluster barrier ends each half-sweep;
//   3. the core's records go back to HBM.
// Neighbouring clusters read one another's cores as halos, so a launch reads
// one record buffer and writes the other (the caller alternates them; the
// first launch of a level also writes the costs into the second buffer).
// The per-node arithmetic is the one-half-sweep kernel's, so results are
// bit-identical to it and to the reference.  Per node and launch the HBM
// traffic is one record in (times the halo overhead) and four messages out,
// against k x (record in + four messages out) / 2 for k single half-sweeps.
//
// Measured on GB300 this is slower than one half-sweep per launch (384x288,
// L = 16, 50 half-sweeps: 0.63 ms at 4 per launch against 0.49 ms; 1920x1080:
// 10.6 ms against 6.8 ms): at L <= 32 the update is bound by the latency of
// its sequential scans, not by HBM, and one resident CTA per SM (20 warps),
// the cluster barriers, the halo's repeated updates and the clusters' GPC
// packing cost more than the traffic saved.  It is therefore opt-in
// (ginf_options.sweeps_per_launch >= 2).
//
// Shared-memory layout of a sub-block: slot ly * bw + (x & 1) * bw / 2 +
// (lx >> 1) for the node at (lx, ly) of the sub-block (global column x), so
// the nodes one half-sweep updates in a row are consecutive slots; a slot is
// the record padded to an odd number of 16-byte chunks (eight consecutive
// slots start in eight different bank groups).  Behind the slots, per warp,
// eight "from" vectors (belief sums) with the same odd-chunk padding.
#include <climits>

#include "sweep_impl.cuh"

namespace ginf_gpu {

namespace {

// Sub-block shape per label bucket: 640 slots of 336 B (L <= 16, 20 warps)
// or 320 slots of 656 B (L <= 32, 10 warps), about 220 KB of shared memory
// with the from vectors, one CTA per SM.
template <int LMAX>
struct ClusterShape;
template <>
struct ClusterShape<16> {
    static constexpr int BW = 32, BH = 20, NW = 20;
};
template <>
struct ClusterShape<32> {
    static constexpr int BW = 16, BH = 20, NW = 10;
};

// Slot of the node at sub-block coordinates (lx, ly), global column x.
__device__ __forceinline__ int cl_slot(int lx, int ly, int x, int bw) {
    return ly * bw + (x & 1) * (bw >> 1) + (lx >> 1);
}

// Belief of one node by its four lanes into the from vector (not over the
// costs: they are read again by later half-sweeps).  Lane `dir` takes the
// 16-byte chunks dir, dir + 4, ...; from = D + in_S + in_E + in_N + in_W in
// that order (bp.cc:10-17).  Returns the lane's first minimum.
template <int LMAX, bool EXACT>
__device__ __forceinline__ void cl_belief(const unsigned char *slot, unsigned char *from, uint32_t d_bytes,
                                          uint32_t m_bytes, int L, int dir, float &best, int &bl) {
    constexpr int B = 4;
    constexpr int NCH = LMAX / B;
    const unsigned char *mb = slot + d_bytes;
#pragma unroll
    for (int j = 0; j < (NCH + 3) / 4; ++j) {
        const int c = (4 * j + dir) * B;
        if (c < LMAX && (EXACT || c < L)) {
            float v[B], a[B];
            load_t<float, B>(slot + c * sizeof(float), v);
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                MIO<float, float>::load(mb + e * m_bytes + c * sizeof(float), a);
#pragma unroll
                for (int kk = 0; kk < B; ++kk) v[kk] = v[kk] + a[kk];
            }
            store_t<float, B>(from + c * sizeof(float), v);
#pragma unroll
            for (int kk = 0; kk < B; ++kk) {
                const int i = c + kk;
                if ((EXACT || i < L) && (bl == 0x7fffffff || v[kk] < best)) {
                    best = v[kk];
                    bl = i;
                }
            }
        }
    }
}

// Truncated-linear / Potts message (bp.cc:26-54), the arithmetic of
// message_linear: h = from - in[dir], min of h, forward and backward
// min-plus scans with slope `scale`, truncation at min(h) + trunc, the mean
// (or the minimum) subtracted; stored when `send`: at `local` (this CTA's
// shared memory) when that is given, else at the distributed-shared-memory
// address `dst` (another CTA's).
template <int LMAX, bool EXACT>
__device__ __forceinline__ void cl_message(const unsigned char *from, const unsigned char *in, unsigned char *local,
                                           uint32_t dst, int L, float scale, float trunc, int norm_min, bool send) {
    constexpr int B = 4;
    float o[LMAX];
#pragma unroll
    for (int c = 0; c < LMAX; c += B) {
        if (EXACT || c < L) {
            float a[B], f[B];
            MIO<float, float>::load(in + c * sizeof(float), a);
            load_t<float, B>(from + c * sizeof(float), f);
#pragma unroll
            for (int k = 0; k < B; ++k) o[c + k] = f[k] - a[k];
        }
    }
    float minh = o[0];
#pragma unroll
    for (int i = 1; i < LMAX; ++i)
        if (EXACT || i < L) minh = rmin(minh, o[i]);
#pragma unroll
    for (int i = 1; i < LMAX; ++i)
        if (EXACT || i < L) o[i] = rmin(o[i], o[i - 1] + scale);
#pragma unroll
    for (int i = LMAX - 2; i >= 0; --i)
        if (EXACT || i + 1 < L) o[i] = rmin(o[i], o[i + 1] + scale);
    minh += trunc;
    float val = 0.f;
#pragma unroll
    for (int i = 0; i < LMAX; ++i)
        if (EXACT || i < L) {
            o[i] = rmin(o[i], minh);
            val += o[i];
        }
    if (norm_min) {
        val = o[0];
#pragma unroll
        for (int i = 1; i < LMAX; ++i)
            if (EXACT || i < L) val = rmin(val, o[i]);
    } else {
        val = mean_of<float, LMAX, EXACT>(val, L);
    }
    if (send && local) {
#pragma unroll
        for (int c = 0; c < LMAX; c += B)
            if (EXACT || c < L)
                *reinterpret_cast<float4 *>(local + c * sizeof(float)) =
                    make_float4(o[c] - val, o[c + 1] - val, o[c + 2] - val, o[c + 3] - val);
    } else if (send) {
#pragma unroll
        for (int c = 0; c < LMAX; c += B)
            if (EXACT || c < L)
                st_dsmem_v4(dst + c * sizeof(float), o[c] - val, o[c + 1] - val, o[c + 2] - val, o[c + 3] - val);
    }
}

template <int LMAX, bool EXACT, int NW>
__global__ void __launch_bounds__(NW * 32, 1) cluster_sweep_kernel(const ClusterSweepParams p) {
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ uint64_t bar;
    launch_dependents();
    const int cx = (int)cluster_nctaid_x(), cy = (int)cluster_nctaid_y();
    const int rx = (int)cluster_ctaid_x(), ry = (int)cluster_ctaid_y();
    const int tx = (int)clusterid_x(), ty = (int)clusterid_y();
    const int k = p.k, bw = p.bw, bh = p.bh, hw = bw >> 1;
    const int RW = cx * bw, RH = cy * bh;
    const int cw = RW - 2 * k, ch = RH - 2 * k;
    const int X0 = tx * cw - k, Y0 = ty * ch - k;     // region origin
    const int xb = X0 + rx * bw, yb = Y0 + ry * bh;   // this CTA's sub-block origin
    const int cx0 = tx * cw, cy0 = ty * ch;           // core origin
    const int W = p.W, H = p.H;
    const int L = EXACT ? LMAX : p.L;
    const int nslots = bw * bh;
    const uint32_t sb = p.slot_bytes;
    unsigned char *from_base = smem + (size_t)nslots * sb;
    const TableConsts<float> tc = table_consts<float, KIND_LINEAR>(p.V, L);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) {
        mbar_init(&bar, NW * 32);
        fence_barrier_init();
    }
    __syncthreads();
    // Records are written by the previous kernel in the stream.
    grid_dependency_wait();

    // 1. Records of the sub-block's nodes inside the grid: whole records, or
    //    the costs only when the level starts from zero messages.
    auto slot_node = [&](int s, int &x, int &y) {
        const int ly = s / bw, r = s - ly * bw;
        const int par = r >= hw ? 1 : 0, n = r - par * hw;
        const int lx = 2 * n + ((par + xb) & 1);
        x = xb + lx;
        y = yb + ly;
        return x >= 0 && y >= 0 && x < W && y < H;
    };
    const uint32_t load_bytes = p.read_mode == RD_OWN ? p.rec_bytes : p.d_bytes;
    {
        uint32_t bytes = 0;
        for (int s = threadIdx.x; s < nslots; s += NW * 32) {
            int x, y;
            if (slot_node(s, x, y)) bytes += load_bytes;
        }
        mbar_arrive_expect_tx(&bar, bytes);
        for (int s = threadIdx.x; s < nslots; s += NW * 32) {
            int x, y;
            if (slot_node(s, x, y))
                bulk_load(smem + (size_t)s * sb, p.rec_in + ((size_t)y * W + x) * p.rec_bytes, load_bytes, &bar);
        }
    }
    const bool got = mbar_wait_bounded(&bar, 0, p.status);
    const bool ok = __syncthreads_and(got) != 0;
    // Incoming slots that hold zero: every one when the level starts from zero
    // messages, else those whose sender is a border node (border nodes never
    // update, bp.cc:149-150; their slots are never written).
    if (ok) {
        for (int q = threadIdx.x; q < nslots * 4; q += NW * 32) {
            const int s = q >> 2, d = q & 3;
            int x, y;
            if (!slot_node(s, x, y)) continue;
            const int qx = x + dir_dx(d), qy = y + dir_dy(d);
            const bool border = qx <= 0 || qy <= 0 || qx >= W - 1 || qy >= H - 1;
            if (p.read_mode != RD_OWN || border) zero_bytes(smem + (size_t)s * sb + p.d_bytes + d * p.m_bytes, p.m_bytes);
        }
    }
    // Every CTA's slots are filled before any neighbour writes into them.
    cluster_sync();

    // 2. k half-sweeps.
    const uint32_t smem_base = smem_addr(smem);
    const int node_k = lane & 7, dir = lane >> 3;
    unsigned char *from = from_base + (size_t)(warp * 8 + node_k) * p.from_stride;
    const int groups = hw >> 3;  // groups of eight same-colour nodes per row
    const int tasks = bh * groups;
    for (int j = 0; j < k; ++j) {
        const int it = p.iter0 + j;
        if (ok) {
            // Rows and columns (region coordinates) whose nodes update now.
            const int lo = j, hix = RW - j, hiy = RH - j;
            for (int t = warp; t < tasks; t += NW) {
                const int ly = t / groups, g = t - ly * groups;
                const int y = yb + ly;
                const int par = (y + it + 1) & 1;  // nodes with x + y + it odd (bp.cc:149-150)
                const int n = g * 8 + node_k;
                const int lx = 2 * n + ((par + xb) & 1);
                const int x = xb + lx;
                const int xr = x - X0, yr = y - Y0;
                const bool act = x >= 1 && x <= W - 2 && y >= 1 && y <= H - 2 && xr >= lo && xr < hix &&
                                 yr >= lo && yr < hiy;
                const unsigned char *slot = smem + (size_t)(ly * bw + par * hw + n) * sb;
                float best = pos_inf<float>();
                int label = 0x7fffffff;
                if (act) cl_belief<LMAX, EXACT>(slot, from, p.d_bytes, p.m_bytes, L, dir, best, label);
                argmin_combine(best, label);
                __syncwarp();
                if (act) {
                    // The neighbour towards dir receives the message in its slot OPP(dir).
                    const int qx = x + dir_dx(dir), qy = y + dir_dy(dir);
                    const int qxr = qx - X0, qyr = qy - Y0;
                    const bool send = qxr >= 0 && qxr < RW && qyr >= 0 && qyr < RH;
                    uint32_t dst = 0;
                    unsigned char *local = nullptr;
                    if (send) {
                        const int qrx = qxr / bw, qry = qyr / bh;
                        const int qs = cl_slot(qxr - qrx * bw, qyr - qry * bh, qx, bw);
                        const uint32_t qoff = (uint32_t)qs * sb + p.d_bytes + opp_dir(dir) * p.m_bytes;
                        if (qrx == rx && qry == ry) local = smem + qoff;
                        else dst = dsmem_addr(smem_base + qoff, (uint32_t)(qry * cx + qrx));
                    }
                    cl_message<LMAX, EXACT>(from, slot + p.d_bytes + dir * p.m_bytes, local, dst, L, tc.scale,
                                            tc.trunc, p.norm_min, send);
                    // Stale-belief decode (bp.cc:65-84): the core's nodes record
                    // the argmin of their last update.
                    if (dir == 0 && it >= p.label_from && x >= cx0 && x < cx0 + cw && y >= cy0 && y < cy0 + ch)
                        p.labels[(size_t)y * W + x] = label;
                }
                __syncwarp();
            }
        }
        cluster_sync();
    }

    // 3. The core's records back to HBM (16-byte chunks, consecutive threads
    //    on consecutive chunks of a node): the four incoming messages, and the
    //    costs too when the output buffer does not hold them yet.
    if (ok) {
        const uint32_t off = p.write_d ? 0u : p.d_bytes;
        const int cpn = (int)((p.rec_bytes - off) >> 4);
        for (int q = threadIdx.x; q < nslots * cpn; q += NW * 32) {
            const int s = q / cpn, c = q - s * cpn;
            int x, y;
            if (!slot_node(s, x, y)) continue;
            if (x < cx0 || x >= cx0 + cw || y < cy0 || y >= cy0 + ch) continue;
            const uint4 v = *reinterpret_cast<const uint4 *>(smem + (size_t)s * sb + off + 16 * c);
            *reinterpret_cast<uint4 *>(p.rec_out + ((size_t)y * W + x) * p.rec_bytes + off + 16 * c) = v;
        }
    }
}

struct ClusterLaunchState {
    SmemLimit smem;
    std::atomic<int> shape[kMaxDevices];  // 0 = not chosen yet, else cx * 16 + cy; -1 = no cluster fits
    std::mutex lock;
};

// The cluster shape for a kernel on the current device: of 4 x 4, 2 x 4,
// 4 x 2 and 2 x 2 CTAs, the one that keeps the most CTAs resident (clusters
// are placed within one GPC, so a GPC's SMs beyond a multiple of the
// cluster size stay idle), the larger one (less halo) on ties.
template <typename K>
cudaError_t cluster_shape(K kern, ClusterLaunchState &st, size_t smem, int threads, int &cx, int &cy) {
    std::atomic<int> &a = st.shape[current_device()];
    int v = a.load(std::memory_order_acquire);
    if (v == 0) {
        std::lock_guard<std::mutex> g(st.lock);
        v = a.load(std::memory_order_relaxed);
        if (v == 0) {
            cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
            if (e != cudaSuccess) return e;
            const int cand[4][2] = {{4, 4}, {2, 4}, {4, 2}, {2, 2}};
            v = -1;
            int best_ctas = 0;
            for (auto &c : cand) {
                cudaLaunchConfig_t lc = {};
                lc.gridDim = dim3(c[0], c[1]);
                lc.blockDim = dim3(threads);
                lc.dynamicSmemBytes = smem;
                cudaLaunchAttribute attr[1];
                attr[0].id = cudaLaunchAttributeClusterDimension;
                attr[0].val.clusterDim.x = c[0];
                attr[0].val.clusterDim.y = c[1];
                attr[0].val.clusterDim.z = 1;
                lc.attrs = attr;
                lc.numAttrs = 1;
                int n = 0;
                e = cudaOccupancyMaxActiveClusters(&n, kern, &lc);
                if (e != cudaSuccess) {
                    cudaGetLastError();
                    continue;
                }
                if (n * c[0] * c[1] > best_ctas) {
                    best_ctas = n * c[0] * c[1];
                    v = c[0] * 16 + c[1];
                }
            }
            a.store(v, std::memory_order_release);
        }
    }
    if (v < 0) return cudaErrorInvalidClusterSize;
    cx = v / 16;
    cy = v % 16;
    return cudaSuccess;
}

template <int LMAX, bool EXACT>
cudaError_t launch_cluster_lm(const ClusterSweepParams &params, cudaStream_t s) {
    using S = ClusterShape<LMAX>;
    static ClusterLaunchState state;
    auto kern = cluster_sweep_kernel<LMAX, EXACT, S::NW>;
    ClusterSweepParams p = params;
    p.bw = S::BW;
    p.bh = S::BH;
    const size_t smem = (size_t)S::BW * S::BH * p.slot_bytes + (size_t)S::NW * 8 * p.from_stride;
    cudaError_t e = state.smem.ensure(kern, smem);
    if (e != cudaSuccess) return e;
    int cx = 0, cy = 0;
    if ((e = cluster_shape(kern, state, smem, S::NW * 32, cx, cy)) != cudaSuccess) return e;
    const int cw = cx * S::BW - 2 * p.k, ch = cy * S::BH - 2 * p.k;
    if (cw < 1 || ch < 1) return cudaErrorInvalidValue;
    const int tiles_x = (p.W + cw - 1) / cw, tiles_y = (p.H + ch - 1) / ch;
    cudaLaunchConfig_t lc = {};
    lc.gridDim = dim3(tiles_x * cx, tiles_y * cy);
    lc.blockDim = dim3(S::NW * 32);
    lc.dynamicSmemBytes = smem;
    lc.stream = s;
    cudaLaunchAttribute attr[2];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = cx;
    attr[0].val.clusterDim.y = cy;
    attr[0].val.clusterDim.z = 1;
    attr[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[1].val.programmaticStreamSerializationAllowed = 1;
    lc.attrs = attr;
    lc.numAttrs = 2;
    return cudaLaunchKernelEx(&lc, kern, p);
}

}  // namespace

int cluster_sweep_max_halo(int L) {
    // Region sides are cx * BW and cy * BH with cx, cy >= 2: the core keeps at
    // least one node for a halo below half the shorter side.
    if (L <= 16) return (2 * ClusterShape<16>::BH - 1) / 2;
    return (2 * ClusterShape<32>::BW - 1) / 2;
}

cudaError_t launch_cluster_sweeps(const RecordFormat &f, const ClusterSweepParams &p, cudaStream_t s) {
    if (f.ctype != CT_F32 || f.store != ST_NATIVE || f.L > 32) return cudaErrorInvalidValue;
    if (f.L == 16) return launch_cluster_lm<16, true>(p, s);
    if (f.L == 32) return launch_cluster_lm<32, true>(p, s);
    if (f.L < 16) return launch_cluster_lm<16, false>(p, s);
    return launch_cluster_lm<32, false>(p, s);
}

}  // namespace ginf_gpu
