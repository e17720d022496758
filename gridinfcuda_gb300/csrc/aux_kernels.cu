// aux_kernels.cu -- every kernel of the inference path other than the
// half-sweep: cost layout transform, HBP pyramid, coarse-to-fine message
// initialisation, label fills, fresh-belief decode, message export, ICM
// (Jacobi and exact Gauss-Seidel wavefront), FP64 energy, stereo costs.
#include <cuda_fp16.h>

#include "ginf_internal.h"

namespace ginf_gpu {

namespace {

__device__ __forceinline__ int ddx(int d) { return d == 1 ? 1 : (d == 3 ? -1 : 0); }  // utils.h:36
__device__ __forceinline__ int ddy(int d) { return d == 0 ? 1 : (d == 2 ? -1 : 0); }  // utils.h:37

__device__ __forceinline__ bool on_border(int x, int y, int W, int H) {
    return x == 0 || y == 0 || x == W - 1 || y == H - 1;
}

template <typename M>
__device__ __forceinline__ double msg_to_double(M v) {
    return (double)v;
}
template <>
__device__ __forceinline__ double msg_to_double<__half>(__half v) {
    return (double)__half2float(v);
}

// 16-byte loads of E = 16/sizeof(T) consecutive elements.
template <typename T>
struct IcmIO {
    __device__ static void load(const T *p, T *o) {
        const uint4 v = *reinterpret_cast<const uint4 *>(p);
        const T *e = reinterpret_cast<const T *>(&v);
#pragma unroll
        for (int k = 0; k < (int)(16 / sizeof(T)); ++k) o[k] = e[k];
    }
};

constexpr int kThreads = 256;

inline unsigned blocks_for(size_t n, int per_block = kThreads) { return (unsigned)((n + per_block - 1) / per_block); }

// ---------------------------------------------------------------------------
// Label-planar costs (x + W*y + W*H*l, the reference's Matrix(3,W,H,L)) into
// the D part of level-0 records.  One block transposes 32 nodes x Lp labels
// through shared memory (stride 33 avoids bank conflicts); reads are
// coalesced along x, writes along l.  Labels L..Lp-1 are zero-filled.
template <typename Tin, typename T>
__global__ void k_costs_to_records(const Tin *__restrict__ src, int W, int H, int L, int Lp,
                                   unsigned char *__restrict__ rec, uint32_t rec_bytes) {
    extern __shared__ __align__(16) unsigned char sm_raw[];
    T *tile = reinterpret_cast<T *>(sm_raw);
    const int x0 = blockIdx.x * 32;
    const int tx = threadIdx.x, ty = threadIdx.y;
    // 16-byte chunks of consecutive labels (Lp is a multiple of 8).
    constexpr int E = 16 / sizeof(T);
    const int cpn = Lp / E;
    const int nn = min(32, W - x0);
    for (int y = blockIdx.y; y < H; y += gridDim.y) {
        for (int l = ty; l < Lp; l += 8) {
            const int x = x0 + tx;
            T v = T(0);
            if (l < L && x < W) v = (T)src[(size_t)x + (size_t)W * y + (size_t)W * H * l];
            tile[l * 33 + tx] = v;
        }
        __syncthreads();
        for (int q = ty * 32 + tx; q < nn * cpn; q += 256) {
            const int i = q / cpn, l0 = (q - i * cpn) * E;
            alignas(16) T v[E];
#pragma unroll
            for (int e = 0; e < E; ++e) v[e] = tile[(l0 + e) * 33 + i];
            *reinterpret_cast<uint4 *>(rec + ((size_t)y * W + x0 + i) * rec_bytes + (size_t)l0 * sizeof(T)) =
                *reinterpret_cast<const uint4 *>(v);
        }
        __syncthreads();
    }
}

// The same transform for two level-0 rows (2Y, 2Y+1) per block, which also
// writes the level-1 costs of the 16 coarse nodes those 32 columns cover:
// each sum is formed from the transposed tiles in shared memory in the
// order k_pyramid uses, so level 0 is not read back for level 1.
template <typename Tin, typename T>
__global__ void k_costs_to_records_pyr(const Tin *__restrict__ src, int W, int H, int L, int Lp,
                                       unsigned char *__restrict__ rec, unsigned char *__restrict__ crec, int cW,
                                       uint32_t rec_bytes) {
    extern __shared__ __align__(16) unsigned char sm_raw[];
    T *tile = reinterpret_cast<T *>(sm_raw);  // [2][Lp][33]
    const int x0 = blockIdx.x * 32;
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int cH = (H + 1) / 2;
    for (int Y = blockIdx.y; Y < cH; Y += gridDim.y) {
    const int rows = min(2, H - 2 * Y);
    for (int r = 0; r < rows; ++r) {
        const int y = 2 * Y + r;
        for (int l = ty; l < Lp; l += 8) {
            const int x = x0 + tx;
            T v = T(0);
            if (l < L && x < W) v = (T)src[(size_t)x + (size_t)W * y + (size_t)W * H * l];
            tile[(r * Lp + l) * 33 + tx] = v;
        }
    }
    __syncthreads();
    // Records are written in 16-byte chunks of consecutive labels (Lp is a
    // multiple of 8, so a node's D part is a whole number of chunks).
    constexpr int E = 16 / sizeof(T);
    const int cpn = Lp / E;
    const int nn = min(32, W - x0);
    for (int r = 0; r < rows; ++r) {
        const int y = 2 * Y + r;
        for (int q = ty * 32 + tx; q < nn * cpn; q += 256) {
            const int i = q / cpn, l0 = (q - i * cpn) * E;
            alignas(16) T v[E];
#pragma unroll
            for (int e = 0; e < E; ++e) v[e] = tile[(r * Lp + l0 + e) * 33 + i];
            *reinterpret_cast<uint4 *>(rec + ((size_t)y * W + x0 + i) * rec_bytes + (size_t)l0 * sizeof(T)) =
                *reinterpret_cast<const uint4 *>(v);
        }
    }
    const int cn = min(16, cW - x0 / 2);
    for (int q = ty * 32 + tx; q < cn * cpn; q += 256) {
        const int i = q / cpn, l0 = (q - i * cpn) * E;
        const int dxn = min(2, W - (x0 + 2 * i));  // fine columns of this coarse node
        alignas(16) T acc[E];
#pragma unroll
        for (int e = 0; e < E; ++e) {
            acc[e] = T(0);
            if (l0 + e < L) {
                for (int r = 0; r < rows; ++r)
                    for (int dx = 0; dx < dxn; ++dx) acc[e] += tile[(r * Lp + l0 + e) * 33 + 2 * i + dx];
            }
        }
        *reinterpret_cast<uint4 *>(crec + ((size_t)Y * cW + x0 / 2 + i) * rec_bytes + (size_t)l0 * sizeof(T)) =
            *reinterpret_cast<const uint4 *>(acc);
    }
    __syncthreads();  // the tiles are refilled for the next row pair
    }
}

// k_costs_to_records_pyr for 4-byte elements and a padded label count LP of
// 16, 32, 64 or 128, over XC columns per block (launched with 32: at 64 the
// larger tile leaves fewer blocks, and loads in flight, per SM, and the
// 1920x1080x64 transform took 0.34 ms against 0.28 ms): the loops are
// unrolled and the plane pointers advanced instead of recomputed.  A warp's store instruction covers
// G consecutive 16-byte chunks (G = 8, or 4 at LP = 16) of 32 / G nodes:
// chunk c of node i reads tile column i at labels 4c..4c+3, bank 4c + i + e
// (row stride XC + 1), so with G = 8 the 32 lanes hit 32 different banks, and
// each node's chunks form one contiguous G * 16-byte run in its record.
// Level-1 sums keep k_pyramid's order (rows, then columns, from zero).
template <typename Tin, typename T, int LP, int XC>
__global__ void __launch_bounds__(256) k_costs_to_records_pyr_lp(const Tin *__restrict__ src, int W, int H, int L,
                                                                 unsigned char *__restrict__ rec,
                                                                 unsigned char *__restrict__ crec, int cW,
                                                                 uint32_t rec_bytes) {
    static_assert(sizeof(T) == 4 && LP % 16 == 0 && XC % 32 == 0, "4-byte elements, whole 16-label groups");
    constexpr int E = 4, CPN = LP / E;
    constexpr int G = CPN < 8 ? CPN : 8, NG = 32 / G, CB = CPN / G;
    constexpr int S = XC + 1;  // tile row stride
    extern __shared__ __align__(16) unsigned char sm_raw[];
    T *tile = reinterpret_cast<T *>(sm_raw);  // [2][LP][S]
    const int x0 = blockIdx.x * XC;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int cH = (H + 1) / 2;
    const size_t plane = (size_t)W * H;
    const int nn = min(XC, W - x0);
    const int cn = min(XC / 2, cW - x0 / 2);
    for (int Y = blockIdx.y; Y < cH; Y += gridDim.y) {
        const int rows = min(2, H - 2 * Y);
        // Warp w loads the planes w, w + 8, ...; lane = column (mod 32).
#pragma unroll
        for (int r = 0; r < 2; ++r) {
#pragma unroll
            for (int h = 0; h < XC / 32; ++h) {
                const int x = x0 + lane + 32 * h;
                const bool ok = r < rows && x < W;
                const Tin *p = src + (ok ? (size_t)W * (2 * Y + r) + x + plane * w : 0);
#pragma unroll
                for (int k = 0; k < LP / 8; ++k) {
                    const int l = w + 8 * k;
                    T v = T(0);
                    if (ok && l < L) v = (T)*p;
                    p += ok ? 8 * plane : 0;
                    tile[(r * LP + l) * S + lane + 32 * h] = v;
                }
            }
        }
        __syncthreads();
        // Level 0: (XC / 32) * CPN store groups of 32 chunks per row.
#pragma unroll
        for (int r = 0; r < 2; ++r) {
            if (r < rows) {
                const size_t row0 = (size_t)(2 * Y + r) * W + x0;
#pragma unroll
                for (int gi = w; gi < CPN * (XC / 32); gi += 8) {
                    const int i = (gi / CB) * NG + lane / G, c = (gi % CB) * G + lane % G;
                    if (i < nn) {
                        alignas(16) T v[E];
#pragma unroll
                        for (int e = 0; e < E; ++e) v[e] = tile[(r * LP + 4 * c + e) * S + i];
                        *reinterpret_cast<uint4 *>(rec + (row0 + i) * rec_bytes + (size_t)c * 16) =
                            *reinterpret_cast<const uint4 *>(v);
                    }
                }
            }
        }
        // Level 1: XC / 2 coarse nodes x CPN chunks, XC * CPN / 64 groups of 32.
#pragma unroll
        for (int gi = w; gi < CPN * XC / 64; gi += 8) {
            const int j = (gi / CB) * NG + lane / G, c = (gi % CB) * G + lane % G;
            if (j < cn) {
                const int dxn = min(2, W - (x0 + 2 * j));
                alignas(16) T acc[E];
#pragma unroll
                for (int e = 0; e < E; ++e) {
                    acc[e] = T(0);
#pragma unroll
                    for (int r = 0; r < 2; ++r)
#pragma unroll
                        for (int dx = 0; dx < 2; ++dx)
                            if (r < rows && dx < dxn) acc[e] += tile[(r * LP + 4 * c + e) * S + 2 * j + dx];
                }
                *reinterpret_cast<uint4 *>(crec + ((size_t)Y * cW + x0 / 2 + j) * rec_bytes + (size_t)c * 16) =
                    *reinterpret_cast<const uint4 *>(acc);
            }
        }
        __syncthreads();  // the tiles are refilled for the next row pair
    }
}

// HBP pyramid, bp.cc:100-117: D_t(X,Y) = sum of the (up to) four finer nodes,
// accumulated from zero in the finer level's raster order.
template <typename T>
__global__ void k_pyramid(const unsigned char *__restrict__ frec, int fW, int fH, unsigned char *__restrict__ crec,
                          int cW, int cH, int L, int Lp, uint32_t rec_bytes) {
    // One thread per (coarse node of row Y = blockIdx.y, 16-byte label chunk).
    constexpr int E = 16 / sizeof(T);
    const int cpn = Lp / E;
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= cW * cpn) return;
    const int X = q / cpn, l0 = (q - X * cpn) * E;
    for (int Y = blockIdx.y; Y < cH; Y += gridDim.y) {
    alignas(16) T acc[E];
#pragma unroll
    for (int e = 0; e < E; ++e) acc[e] = T(0);
    for (int dy = 0; dy < 2; ++dy) {
        const int y = 2 * Y + dy;
        if (y >= fH) break;
        for (int dx = 0; dx < 2; ++dx) {
            const int x = 2 * X + dx;
            if (x >= fW) break;
            alignas(16) T v[E];
            *reinterpret_cast<uint4 *>(v) = *reinterpret_cast<const uint4 *>(
                frec + ((size_t)y * fW + x) * rec_bytes + (size_t)l0 * sizeof(T));
#pragma unroll
            for (int e = 0; e < E; ++e)
                if (l0 + e < L) acc[e] += v[e];
        }
    }
    *reinterpret_cast<uint4 *>(crec + ((size_t)Y * cW + X) * rec_bytes + (size_t)l0 * sizeof(T)) =
        *reinterpret_cast<const uint4 *>(acc);
    }
}

// Materialised message initialisation of a level (used when a level runs
// fewer than two half-sweeps, so the fused first sweep cannot stand in).
// Reference: msgs_t(x,y,d) = msgs_{t+1}(x/2,y/2,d), stored at the sender
// (bp.cc:129-139).  In the receiver layout the slot in_t(p,d) carries the
// message of q = p + dir(d), i.e. msgs_{t+1}(q/2, OPP(d)), which sits at the
// coarse receiver R = q/2 - dir(d) in slot d.  Border senders (at either
// level) never update, so their messages are zero.  crec == nullptr zeroes
// every slot (the top level).
__global__ void k_init_messages(unsigned char *__restrict__ rec, int W, int H, const unsigned char *__restrict__ crec,
                                int cW, int cH, uint32_t rec_bytes, uint32_t d_bytes, uint32_t m_bytes) {
    const uint32_t chunks = m_bytes / 16;
    const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t total = (size_t)W * H * 4 * chunks;
    if (idx >= total) return;
    const uint32_t c = (uint32_t)(idx % chunks);
    const int d = (int)((idx / chunks) % 4);
    const size_t node = idx / (chunks * 4);
    const int x = (int)(node % W), y = (int)(node / W);
    uint4 v = make_uint4(0, 0, 0, 0);
    const int qx = x + ddx(d), qy = y + ddy(d);
    if (crec && qx >= 0 && qy >= 0 && qx < W && qy < H && !on_border(qx, qy, W, H)) {
        const int Qx = qx >> 1, Qy = qy >> 1;
        if (!on_border(Qx, Qy, cW, cH)) {
            const int Rx = Qx - ddx(d), Ry = Qy - ddy(d);
            v = *reinterpret_cast<const uint4 *>(crec + ((size_t)Ry * cW + Rx) * rec_bytes + d_bytes + d * m_bytes +
                                                 16 * c);
        }
    }
    *reinterpret_cast<uint4 *>(rec + node * rec_bytes + d_bytes + d * m_bytes + 16 * c) = v;
}

__global__ void k_fill_interior(int32_t *labels, int W, int H, int32_t value) {
    const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t n = (size_t)(W - 2) * (H - 2);
    if (idx >= n) return;
    const int x = 1 + (int)(idx % (W - 2)), y = 1 + (int)(idx / (W - 2));
    labels[(size_t)y * W + x] = value;
}

// Fresh beliefs from the final messages (GINF_DECODE_FRESH): argmin over l of
// D + sum of incoming messages, interior nodes, lowest label on ties.
template <typename T, typename M>
__global__ void k_decode_fresh(const unsigned char *__restrict__ rec, int W, int H, int L, uint32_t rec_bytes,
                               uint32_t d_bytes, uint32_t m_bytes, int32_t *labels) {
    const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t n = (size_t)(W - 2) * (H - 2);
    if (idx >= n) return;
    const int x = 1 + (int)(idx % (W - 2)), y = 1 + (int)(idx / (W - 2));
    const unsigned char *r = rec + ((size_t)y * W + x) * rec_bytes;
    const T *D = reinterpret_cast<const T *>(r);
    bool z[4];
    for (int d = 0; d < 4; ++d) z[d] = on_border(x + ddx(d), y + ddy(d), W, H);
    T best = T(0);
    int bl = 0;
    for (int l = 0; l < L; ++l) {
        T v = D[l];
        for (int d = 0; d < 4; ++d) {
            const M *m = reinterpret_cast<const M *>(r + d_bytes + d * m_bytes);
            v = v + (z[d] ? T(0) : (T)msg_to_double(m[l]));
        }
        if (l == 0 || v < best) {
            best = v;
            bl = l;
        }
    }
    labels[(size_t)y * W + x] = bl;
}

// Final level-0 messages into a dense [H][W][4][L] array of T (slot d = from
// the neighbour in direction d; 0 where that neighbour is border or off-grid).
template <typename T, typename M>
__global__ void k_export(const unsigned char *__restrict__ rec, int W, int H, int L, uint32_t rec_bytes,
                         uint32_t d_bytes, uint32_t m_bytes, T *__restrict__ dst) {
    const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t total = (size_t)W * H * 4 * L;
    if (idx >= total) return;
    const int l = (int)(idx % L);
    const int d = (int)((idx / L) % 4);
    const size_t node = idx / ((size_t)L * 4);
    const int x = (int)(node % W), y = (int)(node / W);
    const int qx = x + ddx(d), qy = y + ddy(d);
    T v = T(0);
    if (qx >= 0 && qy >= 0 && qx < W && qy < H && !on_border(qx, qy, W, H)) {
        const M *m = reinterpret_cast<const M *>(rec + node * rec_bytes + d_bytes + d * m_bytes);
        v = (T)msg_to_double(m[l]);
    }
    dst[idx] = v;
}

// One ICM node update, grid.cc:127-136 and icm.cc:10-34: LANES lanes per
// node, lane g taking the 16-byte label chunks g, g+LANES, ...; the cost of
// label l is D + V(l,f_S) + V(l,f_E) + V(l,f_N) + V(l,f_W) in that order,
// with V staged in shared memory row by row (Vs[f*Lp + l] = V(l, f)).  The
// partial first-minima of the lanes are combined by (value, label), which
// reproduces the sequential argmin with strict < (lowest label on ties).
// need == false skips the work (no loads) but still takes part in the lane
// combine, which every lane of the warp must reach.
template <typename T, int LANES>
__device__ __forceinline__ int icm_node(const T *D, int W, int L, int Lp, const T *Vs, const int32_t *lab, int x,
                                        int y, int g, int *status, bool need = true) {
    constexpr int E = 16 / sizeof(T);
    // The first cost chunk is requested before the neighbour labels, whose
    // values the table reads depend on; each later chunk one step ahead.
    int c = need ? g * E : L;
    T dv[E];
    if (c < L) IcmIO<T>::load(D + c, dv);
    int f[4];
#pragma unroll
    for (int d = 0; d < 4; ++d) f[d] = need ? lab[(size_t)(y + ddy(d)) * W + (x + ddx(d))] : 0;
#pragma unroll
    for (int d = 0; d < 4; ++d) {
        if (f[d] < 0 || f[d] >= L) {
            if (status && g == 0) atomicOr(status, DEV_ERR_BOUNDS);
            f[d] = 0;
        }
    }
    T best = T(0);
    int bl = 0x7fffffff;
    for (; c < L; c += LANES * E) {
        T dn[E], v[4][E];
        const int cn = c + LANES * E;
        if (cn < L) IcmIO<T>::load(D + cn, dn);
#pragma unroll
        for (int d = 0; d < 4; ++d) IcmIO<T>::load(Vs + (size_t)f[d] * Lp + c, v[d]);
#pragma unroll
        for (int k = 0; k < E; ++k) {
            const int i = c + k;
            T cost = dv[k];
            cost += v[0][k];
            cost += v[1][k];
            cost += v[2][k];
            cost += v[3][k];
            if (i < L && (bl == 0x7fffffff || cost < best)) {
                best = cost;
                bl = i;
            }
        }
#pragma unroll
        for (int k = 0; k < E; ++k) dv[k] = dn[k];
    }
#pragma unroll
    for (int off = 1; off < LANES; off <<= 1) {
        const T ob = __shfl_xor_sync(0xffffffffu, best, off);
        const int ol = __shfl_xor_sync(0xffffffffu, bl, off);
        if (ol != 0x7fffffff && (bl == 0x7fffffff || ob < best || (!(best < ob) && ol < bl))) {
            best = ob;
            bl = ol;
        }
    }
    return bl;
}

// V (L x L, V(l,f) at l + L*f) into shared memory with row stride Lp.
template <typename T>
__device__ __forceinline__ void stage_table(const T *__restrict__ V, T *Vs, int L, int Lp) {
    for (int i = threadIdx.x; i < L * Lp; i += blockDim.x) {
        const int f = i / Lp, l = i - f * Lp;
        Vs[i] = l < L ? V[l + (size_t)L * f] : T(0);
    }
    __syncthreads();
}

// Jacobi sweep over the interior nodes, LANES lanes per node: few lanes share
// the per-node work (index, neighbour labels, the combine).  Two lanes suit
// cost rows strided inside full BP records, four the packed cost-only
// records.  I is the node-index type (32-bit whenever the node count allows).
// chg_in (NULL on the first sweep) flags the nodes the previous sweep
// changed: a node none of whose four neighbours changed would compute the
// same minimisation as last time, so it keeps its label without reading its
// costs.  chg_out receives this sweep's flags (border entries stay 0).
template <typename T, typename I, int LANES>
__global__ void __launch_bounds__(kThreads, 6)
    k_icm_sync(const unsigned char *__restrict__ rec, int W, int H, int L, int Lp, uint32_t rec_bytes,
               const T *__restrict__ V, const int32_t *__restrict__ old_lab, int32_t *__restrict__ new_lab,
               const uint8_t *__restrict__ chg_in, uint8_t *__restrict__ chg_out, int *status) {
    extern __shared__ __align__(16) unsigned char icm_smem[];
    T *Vs = reinterpret_cast<T *>(icm_smem);
    stage_table(V, Vs, L, Lp);
    const I wi = (I)(W - 2);
    const I n = wi * (I)(H - 2);
    const int g = threadIdx.x & (LANES - 1);
    constexpr int kPerBlock = kThreads / LANES;
    // Node groups are whole lane slices of a warp, so every group either has
    // a node or the whole slice skips it together.
    for (I base = (I)blockIdx.x * kPerBlock; base < n; base += (I)gridDim.x * kPerBlock) {
        const I node = base + (threadIdx.x / LANES);
        const bool act = node < n;
        const I nn = act ? node : 0;
        const I row = nn / wi;
        const int x = 1 + (int)(nn - row * wi), y = 1 + (int)row;
        const size_t i = (size_t)y * W + x;
        const bool need = !chg_in || (chg_in[i - W] | chg_in[i + W] | chg_in[i - 1] | chg_in[i + 1]) != 0;
        const T *D = reinterpret_cast<const T *>(rec + i * rec_bytes);
        // A warp none of whose nodes needs the minimisation skips it whole
        // (the test is warp-uniform, so the lane combine stays convergent).
        int bl = 0;
        if (__any_sync(0xffffffffu, need)) bl = icm_node<T, LANES>(D, W, L, Lp, Vs, old_lab, x, y, g, status, need);
        if (act && g == 0) {
            const int prev = old_lab[i];
            if (!need) bl = prev;
            new_lab[i] = bl;
            chg_out[i] = bl != prev ? 1 : 0;
        }
    }
}

template <typename T, typename I, int LANES>
cudaError_t launch_icm_sync_t(const RecordFormat &f, const unsigned char *rec, int W, int H, const void *V,
                              const int32_t *old_labels, int32_t *new_labels, const uint8_t *chg_in, uint8_t *chg_out,
                              int *status, size_t blocks, size_t smem, cudaStream_t s) {
    auto kern = k_icm_sync<T, I, LANES>;
    static SmemLimit limit;
    cudaError_t e = limit.ensure(kern, smem);
    if (e != cudaSuccess) return e;
    kern<<<(unsigned)blocks, kThreads, smem, s>>>(rec, W, H, f.L, f.Lp, f.rec_bytes, static_cast<const T *>(V),
                                                   old_labels, new_labels, chg_in, chg_out, status);
    return cudaGetLastError();
}

// Raster Gauss-Seidel (icm.cc:40-67) as an exact wavefront: on anti-diagonal
// s = x + y every node's west and north neighbours (diagonal s-1) are already
// updated and its east and south neighbours (s+1) are not, exactly as in the
// raster order, and nodes of one diagonal are never adjacent.
template <typename T>
__global__ void k_icm_diag(const unsigned char *__restrict__ rec, int W, int H, int L, int Lp, uint32_t rec_bytes,
                           const T *__restrict__ V, int32_t *lab, int s, int *status) {
    extern __shared__ __align__(16) unsigned char icm_smem[];
    T *Vs = reinterpret_cast<T *>(icm_smem);
    stage_table(V, Vs, L, Lp);
    const int ylo = max(1, s - (W - 2)), yhi = min(H - 2, s - 1);
    const int idx = blockIdx.x * (blockDim.x / 8) + (threadIdx.x >> 3);
    const bool act = ylo + idx <= yhi;
    const int y = act ? ylo + idx : ylo, x = s - y;
    const T *D = reinterpret_cast<const T *>(rec + ((size_t)y * W + x) * rec_bytes);
    const int bl = icm_node<T, 8>(D, W, L, Lp, Vs, lab, x, y, threadIdx.x & 7, status);
    if (act && (threadIdx.x & 7) == 0) lab[(size_t)y * W + x] = bl;
}

// Energy, grid.cc:102-125, in FP64: block partial sums over a fixed
// grid-stride assignment, then one block adds the partials in a fixed tree,
// so the result is identical from run to run.
// a + b as the unevaluated pair (s, e): s = fl(a + b) and e its rounding
// error, exactly (Knuth's TwoSum; the _rn intrinsics keep the compiler from
// contracting or reordering it).
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// Energy accumulators: FP32 terms as a double-float pair (about 48 bits;
// GB300's FP64 pipe is too slow for one FP64 addition per term), int32 terms
// exactly in int64, FP64 terms in FP64.  value() gives the FP64 sum.
template <typename T>
struct EnergyAcc {
    double v = 0.0;
    __device__ void add(T x) { v += (double)x; }
    __device__ void add(const EnergyAcc &o) { v += o.v; }
    __device__ EnergyAcc shfl_xor(int off) const {
        EnergyAcc r;
        r.v = __shfl_xor_sync(0xffffffffu, v, off);
        return r;
    }
    __device__ double value() const { return v; }
};
template <>
struct EnergyAcc<int> {
    long long v = 0;
    __device__ void add(int x) { v += x; }
    __device__ void add(const EnergyAcc &o) { v += o.v; }
    __device__ EnergyAcc shfl_xor(int off) const {
        EnergyAcc r;
        r.v = __shfl_xor_sync(0xffffffffu, v, off);
        return r;
    }
    __device__ double value() const { return (double)v; }
};
template <>
struct EnergyAcc<float> {
    float hi = 0.f, lo = 0.f;
    __device__ void add(float x) {
        float s, e;
        two_sum(hi, x, s, e);
        two_sum(s, __fadd_rn(e, lo), hi, lo);
    }
    __device__ void add(const EnergyAcc &o) {
        float s, e;
        two_sum(hi, o.hi, s, e);
        two_sum(s, __fadd_rn(e, __fadd_rn(lo, o.lo)), hi, lo);
    }
    __device__ EnergyAcc shfl_xor(int off) const {
        EnergyAcc r;
        r.hi = __shfl_xor_sync(0xffffffffu, hi, off);
        r.lo = __shfl_xor_sync(0xffffffffu, lo, off);
        return r;
    }
    __device__ double value() const { return (double)hi + (double)lo; }
};

// Energy partial sums (grid.cc:102-125): per interior node its data cost at
// its label plus the smoothness of its N and E edges.  Nodes are dealt to
// threads in a fixed pattern and reduced in a fixed order, so the result is
// reproducible; each block's sum goes to partials[blockIdx.x].
template <typename T, typename I>
__global__ void k_energy_partial(const T *__restrict__ costs, size_t node_stride, size_t label_stride, int W, int H,
                                 int L, const T *__restrict__ V, const int32_t *__restrict__ f, double *partials,
                                 int *status) {
    const I wi = (I)(W - 2);
    const I n = wi * (I)(H - 2);
    EnergyAcc<T> acc;
    for (I i = (I)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (I)gridDim.x * blockDim.x) {
        const I row = i / wi;
        const int x = 1 + (int)(i - row * wi), y = 1 + (int)row;
        const int fl = f[(size_t)y * W + x];
        const int fn = f[(size_t)(y - 1) * W + x];
        const int fe = f[(size_t)y * W + x + 1];
        if (fl < 0 || fl >= L || fn < 0 || fn >= L || fe < 0 || fe >= L) {
            atomicOr(status, DEV_ERR_BOUNDS);
            continue;
        }
        acc.add(costs[((size_t)y * W + x) * node_stride + (size_t)fl * label_stride]);
        acc.add(V[fl + (size_t)L * fn]);
        acc.add(V[fl + (size_t)L * fe]);
    }
    for (int off = 16; off > 0; off >>= 1) acc.add(acc.shfl_xor(off));
    __shared__ double red[kThreads / 32];
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc.value();
    __syncthreads();
    if (threadIdx.x == 0) {
        double v = 0.0;
        for (int k = 0; k < kThreads / 32; ++k) v += red[k];
        partials[blockIdx.x] = v;
    }
}

__global__ void k_energy_final(const double *partials, int n, double *out) {
    __shared__ double red[kThreads];
    double acc = 0.0;
    for (int i = threadIdx.x; i < n; i += kThreads) acc += partials[i];
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int w = kThreads / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = red[0];
}

template <typename Ts, typename Td>
__global__ void k_convert(const Ts *src, Td *dst, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = (Td)src[i];
}

// D(x,y,d) = coef * min(|left(x,y) - right(max(x-d,0),y)|, cap), label-planar;
// the operation sequence matches the numpy generator bit for bit.
__global__ void k_stereo_costs(int W, int H, int L, const float *__restrict__ left, const float *__restrict__ right,
                               float coef, float cap, float *__restrict__ costs) {
    const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t total = (size_t)W * H * L;
    if (idx >= total) return;
    const int x = (int)(idx % W);
    const int y = (int)((idx / W) % H);
    const int d = (int)(idx / ((size_t)W * H));
    const float a = left[(size_t)y * W + x];
    const float b = right[(size_t)y * W + max(x - d, 0)];
    costs[idx] = coef * fminf(fabsf(a - b), cap);
}

// The reference example's integer recipe (examples/stereo/stereo.cc:28-34):
// for x >= L-1, D(x, y, k) = min(|left(x,y) - right(x-k,y)|, cap) on 8-bit
// grey images; the columns x < L-1 keep zero cost (the Grid constructor's
// zero fill, src/matrix.cc:21-27).  One thread per cost element, label-planar.
__global__ void k_stereo_costs_u8(int W, int H, int L, const uint8_t *__restrict__ left,
                                  const uint8_t *__restrict__ right, int cap, int32_t *__restrict__ costs) {
    const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t total = (size_t)W * H * L;
    if (idx >= total) return;
    const int x = (int)(idx % W);
    const int y = (int)((idx / W) % H);
    const int k = (int)(idx / ((size_t)W * H));
    int c = 0;
    if (x >= L - 1) {
        const int a = left[(size_t)y * W + x];
        const int b = right[(size_t)y * W + x - k];
        c = min(abs(a - b), cap);
    }
    costs[idx] = c;
}

// Level-t inputs and targets of the warm-start network (FP32 records):
// costs and beliefs per fine node, i.e. divided by scale = 4^t.
__global__ void k_level_x(const unsigned char *__restrict__ rec, int W, int H, int L, uint32_t rec_bytes, float scale,
                          float *__restrict__ out) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (size_t)W * H * L) return;
    const size_t node = i / L;
    const int l = (int)(i - node * L);
    out[i] = reinterpret_cast<const float *>(rec + node * rec_bytes)[l] / scale;
}

__global__ void k_level_beliefs(const unsigned char *__restrict__ rec, int W, int H, int L, uint32_t rec_bytes,
                                uint32_t d_bytes, uint32_t m_bytes, float scale, float *__restrict__ out) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (size_t)W * H * L) return;
    const size_t node = i / L;
    const int l = (int)(i - node * L);
    const int x = (int)(node % W), y = (int)(node / W);
    const unsigned char *r = rec + node * rec_bytes;
    float v = reinterpret_cast<const float *>(r)[l];
    for (int d = 0; d < 4; ++d) {
        const int qx = x + ddx(d), qy = y + ddy(d);
        if (qx < 0 || qy < 0 || qx >= W || qy >= H || on_border(qx, qy, W, H)) continue;
        v += reinterpret_cast<const float *>(r + d_bytes + d * m_bytes)[l];
    }
    out[i] = v / scale;
}

// Fine-level target of the warm start: for each node of level t, its costs
// plus the mean over its fine block (2^t x 2^t level-0 nodes, clipped at the
// grid edge) of the level-0 incoming-message sums, divided by 4^t.
__global__ void k_project_fine(const unsigned char *__restrict__ rec0, int W0, int H0,
                               const unsigned char *__restrict__ rect, int Wt, int Ht, int t, int L,
                               uint32_t rec_bytes, uint32_t d_bytes, uint32_t m_bytes, float *__restrict__ out) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (size_t)Wt * Ht * L) return;
    const size_t node = i / L;
    const int l = (int)(i - node * L);
    const int X = (int)(node % Wt), Y = (int)(node / Wt);
    const int bs = 1 << t;
    float sum = 0.f;
    int count = 0;
    for (int y = Y * bs; y < min(H0, (Y + 1) * bs); ++y)
        for (int x = X * bs; x < min(W0, (X + 1) * bs); ++x) {
            const unsigned char *r = rec0 + ((size_t)y * W0 + x) * rec_bytes + d_bytes;
            for (int d = 0; d < 4; ++d) {
                const int qx = x + ddx(d), qy = y + ddy(d);
                if (qx < 0 || qy < 0 || qx >= W0 || qy >= H0 || on_border(qx, qy, W0, H0)) continue;
                sum += reinterpret_cast<const float *>(r + d * m_bytes)[l];
            }
            ++count;
        }
    const float D = reinterpret_cast<const float *>(rect + node * rec_bytes)[l];
    out[i] = (D + sum / (float)max(count, 1)) / (float)(bs * bs);
}

// Labelling that level t hands to the fine level: per node the lowest label
// minimising D_t / 4^t + (sum of incoming messages), i.e. the block mean of
// the beliefs the level-0 nodes start from after the coarse-to-fine copies.
// One warp per node, labels strided over the lanes, FP32 native records.
__global__ void k_level_labels_fine(const unsigned char *__restrict__ rec, int W, int H, int L, uint32_t rec_bytes,
                                    uint32_t d_bytes, uint32_t m_bytes, float inv_scale, int32_t *__restrict__ lab) {
    const size_t node = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (node >= (size_t)W * H) return;
    const int x = (int)(node % W), y = (int)(node / W);
    const unsigned char *r = rec + node * rec_bytes;
    float best = INFINITY;
    int arg = 0x7fffffff;
    for (int l = lane; l < L; l += 32) {
        float v = reinterpret_cast<const float *>(r)[l] * inv_scale;
        for (int d = 0; d < 4; ++d) {
            const int qx = x + ddx(d), qy = y + ddy(d);
            if (qx < 0 || qy < 0 || qx >= W || qy >= H || on_border(qx, qy, W, H)) continue;
            v += reinterpret_cast<const float *>(r + d_bytes + d * m_bytes)[l];
        }
        if (v < best) { best = v; arg = l; }
    }
    for (int o = 16; o > 0; o >>= 1) {
        const float ob = __shfl_xor_sync(0xffffffffu, best, o);
        const int oa = __shfl_xor_sync(0xffffffffu, arg, o);
        if (ob < best || (ob == best && oa < arg)) { best = ob; arg = oa; }
    }
    if (lane == 0) lab[node] = arg == 0x7fffffff ? 0 : arg;
}

// Level-0 labelling that gives every node its level-t block's label.
__global__ void k_upsample_labels(const int32_t *__restrict__ lab_t, int Wt, int t, int32_t *__restrict__ lab0,
                                  int W0, int H0) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (size_t)W0 * H0) return;
    const int x = (int)(i % W0), y = (int)(i / W0);
    lab0[i] = lab_t[(size_t)(y >> t) * Wt + (x >> t)];
}

// Warm start: every incoming slot of every node of level t holds
// factor * (y - x), a quarter of the predicted message sum (factor = 4^t / 4).
__global__ void k_warm_init(unsigned char *__restrict__ rec, int W, int H, int L, int Lp, uint32_t rec_bytes,
                            uint32_t d_bytes, uint32_t m_bytes, const float *__restrict__ y,
                            const float *__restrict__ x, float factor) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (size_t)W * H * Lp) return;
    const size_t node = i / Lp;
    const int l = (int)(i - node * Lp);
    const float v = l < L ? factor * (y[node * L + l] - x[node * L + l]) : 0.f;
    unsigned char *r = rec + node * rec_bytes + d_bytes;
    for (int d = 0; d < 4; ++d) reinterpret_cast<float *>(r + d * m_bytes)[l] = v;
}

}  // namespace

RecordFormat make_format(int ctype, int store, int L) {
    RecordFormat f;
    f.ctype = ctype;
    f.store = store;
    f.L = L;
    f.Lp = (L + 7) & ~7;
    f.t_size = ctype == CT_F64 ? 8u : 4u;
    f.m_size = store == ST_F16 ? 2u : f.t_size;
    f.d_bytes = (uint32_t)f.Lp * f.t_size;
    f.m_bytes = (uint32_t)f.Lp * f.m_size;
    f.rec_bytes = f.d_bytes + 4 * f.m_bytes;
    // Odd number of 16-byte chunks per shared-memory slot: eight consecutive
    // slots then start in eight different bank groups.
    f.slot_bytes = f.rec_bytes + (((f.rec_bytes / 16) % 2 == 0) ? 16u : 0u);
    return f;
}

#define GINF_DISPATCH_T(f, ...)                                   \
    switch ((f).ctype) {                                          \
        case CT_F32: { using T = float; __VA_ARGS__ } break;      \
        case CT_I32: { using T = int; __VA_ARGS__ } break;        \
        case CT_F64: { using T = double; __VA_ARGS__ } break;     \
        default: return cudaErrorInvalidValue;                    \
    }

#define GINF_DISPATCH_TM(f, ...)                                                        \
    if ((f).store == ST_F16) {                                                          \
        if ((f).ctype != CT_F32) return cudaErrorInvalidValue;                          \
        using T = float; using M = __half; __VA_ARGS__                                  \
    } else {                                                                            \
        GINF_DISPATCH_T(f, using M = T; __VA_ARGS__)                                    \
    }

cudaError_t launch_costs_to_records(const RecordFormat &f, int cost_type, const void *src, int W, int H,
                                    unsigned char *rec, cudaStream_t s) {
    const dim3 grid((W + 31) / 32, (unsigned)std::min(H, 65535)), block(32, 8);
    GINF_DISPATCH_T(f, {
        const size_t smem = (size_t)f.Lp * 33 * sizeof(T);
        if (cost_type == CT_F32)
            k_costs_to_records<float, T><<<grid, block, smem, s>>>(static_cast<const float *>(src), W, H, f.L, f.Lp,
                                                                   rec, f.rec_bytes);
        else
            k_costs_to_records<int, T><<<grid, block, smem, s>>>(static_cast<const int *>(src), W, H, f.L, f.Lp, rec,
                                                                 f.rec_bytes);
    })
    return cudaGetLastError();
}

template <typename Tin, typename T, int LP, int XC>
cudaError_t launch_pyr_lp_t(const Tin *src, int W, int H, int L, unsigned char *rec, unsigned char *crec, int cW,
                            uint32_t rec_bytes, cudaStream_t s) {
    auto kern = k_costs_to_records_pyr_lp<Tin, T, LP, XC>;
    const size_t smem = (size_t)2 * LP * (XC + 1) * sizeof(T);
    static SmemLimit limit;
    cudaError_t e = limit.ensure(kern, smem);
    if (e != cudaSuccess) return e;
    const dim3 grid((W + XC - 1) / XC, (unsigned)std::min((H + 1) / 2, 65535));
    kern<<<grid, 256, smem, s>>>(src, W, H, L, rec, crec, cW, rec_bytes);
    return cudaGetLastError();
}

// The specialised transform where one exists (4-byte elements, Lp of 16, 32,
// 64 or 128); `done` false otherwise.
template <typename Tin, typename T>
cudaError_t launch_pyr_lp(int Lp, const Tin *src, int W, int H, int L, unsigned char *rec, unsigned char *crec, int cW,
                          uint32_t rec_bytes, cudaStream_t s, bool &done) {
    done = false;
    if constexpr (sizeof(T) == 4) {
        done = true;
        switch (Lp) {
        case 16: return launch_pyr_lp_t<Tin, T, 16, 32>(src, W, H, L, rec, crec, cW, rec_bytes, s);
        case 32: return launch_pyr_lp_t<Tin, T, 32, 32>(src, W, H, L, rec, crec, cW, rec_bytes, s);
        case 64: return launch_pyr_lp_t<Tin, T, 64, 32>(src, W, H, L, rec, crec, cW, rec_bytes, s);
        case 128: return launch_pyr_lp_t<Tin, T, 128, 32>(src, W, H, L, rec, crec, cW, rec_bytes, s);
        default: done = false;
        }
    }
    return cudaSuccess;
}

cudaError_t launch_costs_to_records_pyr(const RecordFormat &f, int cost_type, const void *src, int W, int H,
                                        unsigned char *rec, unsigned char *crec, int cW, cudaStream_t s) {
    const dim3 grid((W + 31) / 32, (unsigned)std::min((H + 1) / 2, 65535)), block(32, 8);
    GINF_DISPATCH_T(f, {
        bool done = false;
        const cudaError_t e0 = cost_type == CT_F32
                                   ? launch_pyr_lp<float, T>(f.Lp, static_cast<const float *>(src), W, H, f.L, rec,
                                                             crec, cW, f.rec_bytes, s, done)
                                   : launch_pyr_lp<int, T>(f.Lp, static_cast<const int *>(src), W, H, f.L, rec, crec,
                                                           cW, f.rec_bytes, s, done);
        if (done) return e0;
        const size_t smem = (size_t)2 * f.Lp * 33 * sizeof(T);
        if (smem > 48 * 1024) {
            cudaError_t e = cost_type == CT_F32
                                ? cudaFuncSetAttribute(k_costs_to_records_pyr<float, T>,
                                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)
                                : cudaFuncSetAttribute(k_costs_to_records_pyr<int, T>,
                                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e != cudaSuccess) return e;
        }
        if (cost_type == CT_F32)
            k_costs_to_records_pyr<float, T><<<grid, block, smem, s>>>(static_cast<const float *>(src), W, H, f.L,
                                                                       f.Lp, rec, crec, cW, f.rec_bytes);
        else
            k_costs_to_records_pyr<int, T><<<grid, block, smem, s>>>(static_cast<const int *>(src), W, H, f.L, f.Lp,
                                                                     rec, crec, cW, f.rec_bytes);
    })
    return cudaGetLastError();
}

cudaError_t launch_pyramid(const RecordFormat &f, const unsigned char *frec, int fW, int fH, unsigned char *crec,
                           int cW, int cH, cudaStream_t s) {
    GINF_DISPATCH_T(f, {
        const int cpn = f.Lp / (16 / (int)sizeof(T));
        const dim3 grid(blocks_for((size_t)cW * cpn), (unsigned)std::min(cH, 65535));
        k_pyramid<T><<<grid, kThreads, 0, s>>>(frec, fW, fH, crec, cW, cH, f.L, f.Lp, f.rec_bytes);
    })
    return cudaGetLastError();
}

cudaError_t launch_init_messages(const RecordFormat &f, unsigned char *rec, int W, int H, const unsigned char *crec,
                                 int cW, int cH, cudaStream_t s) {
    const size_t total = (size_t)W * H * 4 * (f.m_bytes / 16);
    k_init_messages<<<blocks_for(total), kThreads, 0, s>>>(rec, W, H, crec, cW, cH, f.rec_bytes, f.d_bytes,
                                                           f.m_bytes);
    return cudaGetLastError();
}

cudaError_t launch_fill_interior(int32_t *labels, int W, int H, int32_t value, cudaStream_t s) {
    if (W < 3 || H < 3) return cudaSuccess;
    const size_t n = (size_t)(W - 2) * (H - 2);
    k_fill_interior<<<blocks_for(n), kThreads, 0, s>>>(labels, W, H, value);
    return cudaGetLastError();
}

cudaError_t launch_decode_fresh(const RecordFormat &f, const unsigned char *rec, int W, int H, int32_t *labels,
                                cudaStream_t s) {
    if (W < 3 || H < 3) return cudaSuccess;
    const size_t n = (size_t)(W - 2) * (H - 2);
    GINF_DISPATCH_TM(f, { k_decode_fresh<T, M><<<blocks_for(n), kThreads, 0, s>>>(rec, W, H, f.L, f.rec_bytes,
                                                                                  f.d_bytes, f.m_bytes, labels); })
    return cudaGetLastError();
}

cudaError_t launch_export_messages(const RecordFormat &f, const unsigned char *rec, int W, int H, void *dst,
                                   cudaStream_t s) {
    const size_t total = (size_t)W * H * 4 * f.L;
    GINF_DISPATCH_TM(f, { k_export<T, M><<<blocks_for(total), kThreads, 0, s>>>(rec, W, H, f.L, f.rec_bytes,
                                                                                f.d_bytes, f.m_bytes,
                                                                                static_cast<T *>(dst)); })
    return cudaGetLastError();
}

// Shared memory for the staged table, raising the kernel's limit once when
// it exceeds the default 48 KB.
template <typename K>
cudaError_t icm_smem_attr(K kern, size_t bytes) {
    static SmemLimit limit;
    return limit.ensure(kern, bytes);
}

// SM count of the current device (memoised per device; a failed query is
// not remembered).
int num_sms() {
    static std::atomic<int> count[kMaxDevices];
    const int dev = current_device();
    int n = count[dev].load(std::memory_order_relaxed);
    if (n > 0) return n;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) {
        cudaGetLastError();
        return 1;
    }
    count[dev].store(n, std::memory_order_relaxed);
    return n;
}

cudaError_t launch_icm_sync(const RecordFormat &f, const unsigned char *rec, int W, int H, const void *V,
                            const int32_t *old_labels, int32_t *new_labels, const uint8_t *chg_in, uint8_t *chg_out,
                            int *status, cudaStream_t s) {
    if (W < 3 || H < 3) return cudaSuccess;
    const size_t n = (size_t)(W - 2) * (H - 2);
    const bool packed = f.rec_bytes == f.d_bytes;
    const size_t per_block = kThreads / (packed ? 4 : 2);
    size_t blocks = (n + per_block - 1) / per_block;
    const size_t cap = (size_t)num_sms() * 6;
    if (blocks > cap) blocks = cap;
    const bool narrow = n + blocks * per_block < 0xffffffffull;
    GINF_DISPATCH_T(f, {
        const size_t smem = (size_t)f.L * f.Lp * sizeof(T);
        if (packed)
            return narrow ? launch_icm_sync_t<T, uint32_t, 4>(f, rec, W, H, V, old_labels, new_labels, chg_in, chg_out,
                                                              status, blocks, smem, s)
                          : launch_icm_sync_t<T, size_t, 4>(f, rec, W, H, V, old_labels, new_labels, chg_in, chg_out,
                                                            status, blocks, smem, s);
        return narrow ? launch_icm_sync_t<T, uint32_t, 2>(f, rec, W, H, V, old_labels, new_labels, chg_in, chg_out,
                                                          status, blocks, smem, s)
                      : launch_icm_sync_t<T, size_t, 2>(f, rec, W, H, V, old_labels, new_labels, chg_in, chg_out,
                                                        status, blocks, smem, s);
    })
    return cudaGetLastError();
}

cudaError_t launch_icm_async_diag(const RecordFormat &f, const unsigned char *rec, int W, int H, const void *V,
                                  int32_t *labels, int diag, int *status, cudaStream_t s) {
    const int ylo = diag - (W - 2) > 1 ? diag - (W - 2) : 1;
    const int yhi = diag - 1 < H - 2 ? diag - 1 : H - 2;
    if (yhi < ylo) return cudaSuccess;
    const size_t n = (size_t)(yhi - ylo + 1);
    GINF_DISPATCH_T(f, {
        const size_t smem = (size_t)f.L * f.Lp * sizeof(T);
        cudaError_t e = icm_smem_attr(k_icm_diag<T>, smem);
        if (e != cudaSuccess) return e;
        k_icm_diag<T><<<blocks_for(n * 8), kThreads, smem, s>>>(rec, W, H, f.L, f.Lp, f.rec_bytes,
                                                                static_cast<const T *>(V), labels, diag, status);
    })
    return cudaGetLastError();
}

int energy_num_partials(int W, int H) {
    const size_t n = (W > 2 && H > 2) ? (size_t)(W - 2) * (H - 2) : 0;
    // About eight nodes per thread.
    size_t b = (n + 8 * kThreads - 1) / (8 * kThreads);
    if (b > 2048) b = 2048;
    if (b < 1) b = 1;
    return (int)b;
}

cudaError_t launch_energy(int ctype, const void *costs, size_t node_stride, size_t label_stride, int W, int H, int L,
                          const void *V, const int32_t *labels, double *partials, int num_partials, double *out,
                          int *status, cudaStream_t s) {
    if (W < 3 || H < 3) {
        return cudaMemsetAsync(out, 0, sizeof(double), s);
    }
    RecordFormat f;
    f.ctype = ctype;
    const bool narrow = (size_t)(W - 2) * (H - 2) + (size_t)num_partials * kThreads < 0xffffffffull;
    GINF_DISPATCH_T(f, {
        if (narrow)
            k_energy_partial<T, uint32_t><<<num_partials, kThreads, 0, s>>>(
                static_cast<const T *>(costs), node_stride, label_stride, W, H, L, static_cast<const T *>(V), labels,
                partials, status);
        else
            k_energy_partial<T, size_t><<<num_partials, kThreads, 0, s>>>(
                static_cast<const T *>(costs), node_stride, label_stride, W, H, L, static_cast<const T *>(V), labels,
                partials, status);
    })
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_energy_final<<<1, kThreads, 0, s>>>(partials, num_partials, out);
    return cudaGetLastError();
}

cudaError_t launch_convert_table(int src_type, int dst_type, const void *src, void *dst, int n, cudaStream_t s) {
    const unsigned b = blocks_for((size_t)n);
    if (src_type == CT_F32 && dst_type == CT_F64)
        k_convert<float, double><<<b, kThreads, 0, s>>>(static_cast<const float *>(src), static_cast<double *>(dst), n);
    else if (src_type == CT_I32 && dst_type == CT_F64)
        k_convert<int, double><<<b, kThreads, 0, s>>>(static_cast<const int *>(src), static_cast<double *>(dst), n);
    else if (src_type == CT_I32 && dst_type == CT_F32)
        k_convert<int, float><<<b, kThreads, 0, s>>>(static_cast<const int *>(src), static_cast<float *>(dst), n);
    else if (src_type == CT_F32 && dst_type == CT_I32)
        k_convert<float, int><<<b, kThreads, 0, s>>>(static_cast<const float *>(src), static_cast<int *>(dst), n);
    else
        return cudaErrorInvalidValue;
    return cudaGetLastError();
}

cudaError_t launch_level_x(const RecordFormat &f, const unsigned char *rec, int W, int H, float scale, float *out,
                           cudaStream_t s) {
    if (f.ctype != CT_F32) return cudaErrorInvalidValue;
    k_level_x<<<blocks_for((size_t)W * H * f.L), kThreads, 0, s>>>(rec, W, H, f.L, f.rec_bytes, scale, out);
    return cudaGetLastError();
}

cudaError_t launch_level_beliefs(const RecordFormat &f, const unsigned char *rec, int W, int H, float scale,
                                 float *out, cudaStream_t s) {
    if (f.ctype != CT_F32 || f.store != ST_NATIVE) return cudaErrorInvalidValue;
    k_level_beliefs<<<blocks_for((size_t)W * H * f.L), kThreads, 0, s>>>(rec, W, H, f.L, f.rec_bytes, f.d_bytes,
                                                                         f.m_bytes, scale, out);
    return cudaGetLastError();
}

cudaError_t launch_fine_labels(const RecordFormat &f, const unsigned char *rect, int Wt, int Ht, int t,
                               int32_t *lab_t, int32_t *lab0, int W0, int H0, cudaStream_t s) {
    if (f.ctype != CT_F32 || f.store != ST_NATIVE) return cudaErrorInvalidValue;
    k_level_labels_fine<<<blocks_for((size_t)Wt * Ht * 32), kThreads, 0, s>>>(
        rect, Wt, Ht, f.L, f.rec_bytes, f.d_bytes, f.m_bytes, 1.f / (float)(1u << (2 * t)), lab_t);
    k_upsample_labels<<<blocks_for((size_t)W0 * H0), kThreads, 0, s>>>(lab_t, Wt, t, lab0, W0, H0);
    return cudaGetLastError();
}

cudaError_t launch_project_fine(const RecordFormat &f, const unsigned char *rec0, int W0, int H0,
                                const unsigned char *rect, int Wt, int Ht, int t, float *out, cudaStream_t s) {
    if (f.ctype != CT_F32 || f.store != ST_NATIVE) return cudaErrorInvalidValue;
    k_project_fine<<<blocks_for((size_t)Wt * Ht * f.L), kThreads, 0, s>>>(rec0, W0, H0, rect, Wt, Ht, t, f.L,
                                                                          f.rec_bytes, f.d_bytes, f.m_bytes, out);
    return cudaGetLastError();
}

cudaError_t launch_warm_init(const RecordFormat &f, unsigned char *rec, int W, int H, const float *y, const float *x,
                             float factor, cudaStream_t s) {
    if (f.ctype != CT_F32 || f.store != ST_NATIVE) return cudaErrorInvalidValue;
    k_warm_init<<<blocks_for((size_t)W * H * f.Lp), kThreads, 0, s>>>(rec, W, H, f.L, f.Lp, f.rec_bytes, f.d_bytes,
                                                                       f.m_bytes, y, x, factor);
    return cudaGetLastError();
}

cudaError_t launch_stereo_costs(int W, int H, int L, const float *left, const float *right, float coef, float cap,
                                float *costs, cudaStream_t s) {
    const size_t total = (size_t)W * H * L;
    k_stereo_costs<<<blocks_for(total), kThreads, 0, s>>>(W, H, L, left, right, coef, cap, costs);
    return cudaGetLastError();
}

cudaError_t launch_stereo_costs_u8(int W, int H, int L, const uint8_t *left, const uint8_t *right, int cap,
                                   int32_t *costs, cudaStream_t s) {
    const size_t total = (size_t)W * H * L;
    k_stereo_costs_u8<<<blocks_for(total), kThreads, 0, s>>>(W, H, L, left, right, cap, costs);
    return cudaGetLastError();
}

}  // namespace ginf_gpu
