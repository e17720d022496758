// sweep_impl.cuh -- the checkerboard half-sweep kernel (one BP "iteration").
//
// Work split: one thread per updated node, NT same-colour nodes of one grid
// row per tile.  Per tile:
//   1. every thread issues one bulk TMA copy of its node's record (costs plus
//      the four incoming messages, rec_bytes contiguous bytes) into its own
//      padded shared-memory slot; completion is counted in bytes on the
//      stage's mbarrier (the slot stride is an odd number of 16-byte chunks,
//      so the 128-bit shared loads below are free of bank conflicts);
//   2. the thread forms the belief from = D + m_S + m_E + m_N + m_W, its
//      argmin (the reference's stale-belief label, bp.cc:65-84), and the four
//      outgoing messages, each written over the incoming slot it replaces;
//   3. four bulk TMA stores move the outgoing messages into the neighbours'
//      records (stored at the receiver, slot OPP(d)).
// With STAGES == 2 the next tile's copies are in flight while the current one
// is computed.  The sequential per-thread update reproduces the reference's
// operation order exactly (src/bp.cc:7-63), so f32 and i32 results are
// bit-identical to the CPU code.
#pragma once

#include <cuda_fp16.h>

#include <type_traits>

#include "ginf_internal.h"
#include "ptx.cuh"

namespace ginf_gpu {

__device__ __forceinline__ int dir_dx(int d) { return d == 1 ? 1 : (d == 3 ? -1 : 0); }  // utils.h:36
__device__ __forceinline__ int dir_dy(int d) { return d == 0 ? 1 : (d == 2 ? -1 : 0); }  // utils.h:37
__device__ __forceinline__ int opp_dir(int d) { return d >= 2 ? d - 2 : d + 2; }          // utils.h:10

// GINF_MIN (utils.h:16): on equal operands the second one is returned.
template <typename T>
__device__ __forceinline__ T rmin(T a, T b) {
    return (a < b) ? a : b;
}

// val /= numLabels in T arithmetic (bp.cc:51): IEEE division for floats,
// truncating division for int.
__device__ __forceinline__ float div_labels(float v, int L) { return __fdiv_rn(v, (float)L); }
__device__ __forceinline__ double div_labels(double v, int L) { return __ddiv_rn(v, (double)L); }
__device__ __forceinline__ int div_labels(int v, int L) { return v / L; }

template <typename T>
__device__ __forceinline__ T pos_inf();
template <>
__device__ __forceinline__ float pos_inf<float>() {
    return __int_as_float(0x7f800000);
}
template <>
__device__ __forceinline__ double pos_inf<double>() {
    return __longlong_as_double(0x7ff0000000000000ll);
}
template <>
__device__ __forceinline__ int pos_inf<int>() {
    return 0x7fffffff;
}

// Message element I/O between shared memory (type M) and arithmetic (type T),
// in blocks of B elements = one 16-byte chunk of M.
template <typename M, typename T>
struct MIO;
template <>
struct MIO<float, float> {
    static constexpr int B = 4;
    __device__ static void load(const unsigned char *p, float *o) {
        const float4 v = *reinterpret_cast<const float4 *>(p);
        o[0] = v.x; o[1] = v.y; o[2] = v.z; o[3] = v.w;
    }
    __device__ static void store(unsigned char *p, const float *o) {
        *reinterpret_cast<float4 *>(p) = make_float4(o[0], o[1], o[2], o[3]);
    }
};
template <>
struct MIO<int, int> {
    static constexpr int B = 4;
    __device__ static void load(const unsigned char *p, int *o) {
        const int4 v = *reinterpret_cast<const int4 *>(p);
        o[0] = v.x; o[1] = v.y; o[2] = v.z; o[3] = v.w;
    }
    __device__ static void store(unsigned char *p, const int *o) {
        *reinterpret_cast<int4 *>(p) = make_int4(o[0], o[1], o[2], o[3]);
    }
};
template <>
struct MIO<double, double> {
    static constexpr int B = 2;
    __device__ static void load(const unsigned char *p, double *o) {
        const double2 v = *reinterpret_cast<const double2 *>(p);
        o[0] = v.x; o[1] = v.y;
    }
    __device__ static void store(unsigned char *p, const double *o) {
        *reinterpret_cast<double2 *>(p) = make_double2(o[0], o[1]);
    }
};
template <>
struct MIO<__half, float> {
    static constexpr int B = 8;
    __device__ static void load(const unsigned char *p, float *o) {
        const uint4 v = *reinterpret_cast<const uint4 *>(p);
        const uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            __half2 h;
            *reinterpret_cast<uint32_t *>(&h) = w[k];
            const float2 f = __half22float2(h);
            o[2 * k] = f.x;
            o[2 * k + 1] = f.y;
        }
    }
    __device__ static void store(unsigned char *p, const float *o) {
        uint32_t w[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const __half2 h = __floats2half2_rn(o[2 * k], o[2 * k + 1]);
            w[k] = *reinterpret_cast<const uint32_t *>(&h);
        }
        *reinterpret_cast<uint4 *>(p) = make_uint4(w[0], w[1], w[2], w[3]);
    }
};

// B consecutive T elements from 16-byte aligned shared memory.
template <typename T, int B>
__device__ __forceinline__ void load_t(const unsigned char *p, T *o) {
    constexpr int E = 16 / sizeof(T);
#pragma unroll
    for (int c = 0; c < B / E; ++c) MIO<T, T>::load(p + 16 * c, o + E * c);
}
template <typename T, int B>
__device__ __forceinline__ void store_t(unsigned char *p, const T *o) {
    constexpr int E = 16 / sizeof(T);
#pragma unroll
    for (int c = 0; c < B / E; ++c) MIO<T, T>::store(p + 16 * c, o + E * c);
}

// Which incoming slots hold a zero message: those whose sender is a border
// node (border nodes never update, so their messages stay 0 at every level,
// bp.cc:129-150) and, for a first sweep fed from the coarser level, those
// whose coarse source node is on the coarse border.
__device__ __forceinline__ unsigned zero_mask(const SweepParams &p, int x, int y) {
    if (p.read_mode == RD_ZERO) return 0xFu;
    unsigned z = 0;
#pragma unroll
    for (int d = 0; d < 4; ++d) {
        const int qx = x + dir_dx(d), qy = y + dir_dy(d);
        bool zero = qx == 0 || qy == 0 || qx == p.W - 1 || qy == p.H - 1;
        if (p.read_mode == RD_COARSE && !zero) {
            const int Qx = qx >> 1, Qy = qy >> 1;
            zero = Qx == 0 || Qy == 0 || Qx == p.cW - 1 || Qy == p.cH - 1;
        }
        z |= (zero ? 1u : 0u) << d;
    }
    return z;
}

// from = D + in_S + in_E + in_N + in_W per label, in the order of bp.cc:10-17,
// plus its first argmin (strict <, bp.cc:74-80).  The belief goes to fr[]
// (registers) when FR_REGS, else over the D region of the slot.
template <typename T, typename M, int LMAX, bool FR_REGS>
__device__ __forceinline__ void collect(const SweepParams &p, unsigned char *slot, unsigned zmask, T *fr, int &label) {
    constexpr int B = MIO<M, T>::B;
    const int L = p.L;
    unsigned char *mb = slot + p.d_bytes;
    T best = T(0);
    int bl = 0;
#pragma unroll
    for (int c = 0; c < LMAX; c += B) {
        if (c < L) {
            T v[B], a[B];
            load_t<T, B>(slot + c * sizeof(T), v);
#pragma unroll
            for (int d = 0; d < 4; ++d) {
                MIO<M, T>::load(mb + d * p.m_bytes + c * sizeof(M), a);
                const bool z = (zmask >> d) & 1u;
#pragma unroll
                for (int k = 0; k < B; ++k) v[k] = v[k] + (z ? T(0) : a[k]);
            }
#pragma unroll
            for (int k = 0; k < B; ++k) {
                const int i = c + k;
                if (i == 0) {
                    best = v[k];
                    bl = 0;
                } else if (i < L && v[k] < best) {
                    best = v[k];
                    bl = i;
                }
            }
            if constexpr (FR_REGS) {
#pragma unroll
                for (int k = 0; k < B; ++k) fr[c + k] = v[k];
            } else {
                store_t<T, B>(slot + c * sizeof(T), v);
            }
        }
    }
    label = bl;
}

// Truncated-linear / Potts messages (bp.cc:26-54), all four directions.
template <typename T, typename M, int LMAX, bool FR_REGS>
__device__ __forceinline__ void messages_linear(const SweepParams &p, unsigned char *slot, unsigned zmask, const T *fr) {
    constexpr int B = MIO<M, T>::B;
    const int L = p.L;
    const T *Vt = static_cast<const T *>(p.V);
    const T scale = __ldg(&Vt[L]), trunc = __ldg(&Vt[(size_t)L * (L - 1)]);  // V(0,1), V(0,L-1): bp.cc:35,43
    unsigned char *mb = slot + p.d_bytes;
#pragma unroll 1
    for (int d = 0; d < 4; ++d) {
        const bool zd = (zmask >> d) & 1u;
        unsigned char *md = mb + d * p.m_bytes;
        T o[LMAX];
#pragma unroll
        for (int c = 0; c < LMAX; c += B) {
            if (c < L) {
                T a[B], f[B];
                MIO<M, T>::load(md + c * sizeof(M), a);
                if constexpr (FR_REGS) {
#pragma unroll
                    for (int k = 0; k < B; ++k) f[k] = fr[c + k];
                } else {
                    load_t<T, B>(slot + c * sizeof(T), f);
                }
#pragma unroll
                for (int k = 0; k < B; ++k) o[c + k] = f[k] - (zd ? T(0) : a[k]);
            }
        }
        T minh = o[0];
#pragma unroll
        for (int i = 1; i < LMAX; ++i)
            if (i < L) minh = rmin(minh, o[i]);
#pragma unroll
        for (int i = 1; i < LMAX; ++i)
            if (i < L) o[i] = rmin(o[i], o[i - 1] + scale);
#pragma unroll
        for (int i = LMAX - 2; i >= 0; --i)
            if (i + 1 < L) o[i] = rmin(o[i], o[i + 1] + scale);
        minh += trunc;
        T val = T(0);
#pragma unroll
        for (int i = 0; i < LMAX; ++i)
            if (i < L) {
                o[i] = rmin(o[i], minh);
                val += o[i];
            }
        if (p.norm_min) {
            val = o[0];
#pragma unroll
            for (int i = 1; i < LMAX; ++i)
                if (i < L) val = rmin(val, o[i]);
        } else {
            val = div_labels(val, L);
        }
#pragma unroll
        for (int c = 0; c < LMAX; c += B) {
            if (c < L) {
                T r[B];
#pragma unroll
                for (int k = 0; k < B; ++k) r[k] = o[c + k] - val;
                MIO<M, T>::store(md + c * sizeof(M), r);
            }
        }
    }
}

// Writes o[0..L) (then padding up to the chunk boundary) into message slot md.
template <typename T, typename M, int LMAX>
__device__ __forceinline__ void store_msg(unsigned char *md, const T *o, int L) {
    constexpr int B = MIO<M, T>::B;
#pragma unroll 1
    for (int c = 0; c < L; c += B) {
        T r[B];
#pragma unroll
        for (int k = 0; k < B; ++k) r[k] = (c + k < L) ? o[c + k] : T(0);
        MIO<M, T>::store(md + c * sizeof(M), r);
    }
}

// h = from - incoming (from over the D region of the slot), into local h[].
template <typename T, typename M, int LMAX>
__device__ __forceinline__ void load_h(const unsigned char *slot, const unsigned char *md, bool zd, int L, T *h) {
    constexpr int B = MIO<M, T>::B;
#pragma unroll 1
    for (int c = 0; c < L; c += B) {
        T a[B], f[B];
        MIO<M, T>::load(md + c * sizeof(M), a);
        load_t<T, B>(slot + c * sizeof(T), f);
#pragma unroll
        for (int k = 0; k < B; ++k)
            if (c + k < LMAX) h[c + k] = f[k] - (zd ? T(0) : a[k]);
    }
}

template <typename T>
__device__ __forceinline__ void normalise(T *o, int L, int norm_min) {
    T val;
    if (norm_min) {
        val = o[0];
        for (int i = 1; i < L; ++i) val = rmin(val, o[i]);
    } else {
        val = T(0);
        for (int i = 0; i < L; ++i) val += o[i];
        val = div_labels(val, L);
    }
    for (int i = 0; i < L; ++i) o[i] -= val;
}

// Reference rule for EXPLICIT / TRUNC_QUAD (bp.cc:55-62): the same vector
// out(i) = min_j V(i,j) + from(j) goes out in all four directions, without
// subtracting the receiver's message and without normalisation.
template <typename T, typename M, int LMAX>
__device__ void messages_ref_minconv(const SweepParams &p, unsigned char *slot) {
    const int L = p.L;
    const T *V = static_cast<const T *>(p.V);
    const T *fr = reinterpret_cast<const T *>(slot);
    T o[LMAX];
#pragma unroll 1
    for (int i = 0; i < L; ++i) {
        T m = __ldg(&V[i]) + fr[0];
#pragma unroll 1
        for (int j = 0; j < L; ++j) m = rmin(m, __ldg(&V[i + (size_t)L * j]) + fr[j]);
        o[i] = m;
    }
    unsigned char *mb = slot + p.d_bytes;
#pragma unroll 1
    for (int d = 0; d < 4; ++d) store_msg<T, M, LMAX>(mb + d * p.m_bytes, o, L);
}

// Standard rule, EXPLICIT model: O(L^2) min-convolution of h = from - in.
template <typename T, typename M, int LMAX>
__device__ void messages_std_minconv(const SweepParams &p, unsigned char *slot, unsigned zmask) {
    const int L = p.L;
    const T *V = static_cast<const T *>(p.V);
    unsigned char *mb = slot + p.d_bytes;
    T h[LMAX], o[LMAX];
#pragma unroll 1
    for (int d = 0; d < 4; ++d) {
        unsigned char *md = mb + d * p.m_bytes;
        load_h<T, M, LMAX>(slot, md, (zmask >> d) & 1u, L, h);
#pragma unroll 1
        for (int i = 0; i < L; ++i) {
            T m = __ldg(&V[i]) + h[0];
#pragma unroll 1
            for (int j = 1; j < L; ++j) m = rmin(m, __ldg(&V[i + (size_t)L * j]) + h[j]);
            o[i] = m;
        }
        normalise(o, L, p.norm_min);
        store_msg<T, M, LMAX>(md, o, L);
    }
}

// Standard rule, truncated quadratic: O(L) lower envelope of parabolas
// (Felzenszwalb & Huttenlocher, "Distance Transforms of Sampled Functions",
// Theory of Computing 8, 2012), then truncation at min(h) + V(0, L-1).
template <typename T, typename M, int LMAX>
__device__ void messages_std_quad(const SweepParams &p, unsigned char *slot, unsigned zmask) {
    if constexpr (std::is_same<T, int>::value) {
        return;  // integer grids use the exact O(L^2) rule instead (host side)
    } else {
        const int L = p.L;
        const T *Vt = static_cast<const T *>(p.V);
        const T s = __ldg(&Vt[L]), trunc = __ldg(&Vt[(size_t)L * (L - 1)]);
        unsigned char *mb = slot + p.d_bytes;
        T h[LMAX], o[LMAX], z[LMAX + 1];
        int v[LMAX];
#pragma unroll 1
        for (int d = 0; d < 4; ++d) {
            unsigned char *md = mb + d * p.m_bytes;
            load_h<T, M, LMAX>(slot, md, (zmask >> d) & 1u, L, h);
            T minh = h[0];
            for (int i = 1; i < L; ++i) minh = h[i] < minh ? h[i] : minh;
            if (!(s > T(0))) {
                for (int i = 0; i < L; ++i) o[i] = minh;
            } else {
                int k = 0;
                v[0] = 0;
                z[0] = -pos_inf<T>();
                z[1] = pos_inf<T>();
#pragma unroll 1
                for (int q = 1; q < L; ++q) {
                    T sq;
                    for (;;) {
                        const int pp = v[k];
                        sq = ((h[q] + s * T(q) * T(q)) - (h[pp] + s * T(pp) * T(pp))) / (T(2) * s * T(q - pp));
                        if (sq <= z[k] && k > 0) {
                            --k;
                            continue;
                        }
                        break;
                    }
                    if (sq <= z[k]) {
                        v[0] = q;
                        z[0] = -pos_inf<T>();
                        z[1] = pos_inf<T>();
                        continue;
                    }
                    ++k;
                    v[k] = q;
                    z[k] = sq;
                    z[k + 1] = pos_inf<T>();
                }
                k = 0;
#pragma unroll 1
                for (int q = 0; q < L; ++q) {
                    while (z[k + 1] < T(q)) ++k;
                    const int pp = v[k];
                    o[q] = s * T(q - pp) * T(q - pp) + h[pp];
                }
            }
            const T cap = minh + trunc;
            for (int i = 0; i < L; ++i) o[i] = rmin(o[i], cap);
            normalise(o, L, p.norm_min);
            store_msg<T, M, LMAX>(md, o, L);
        }
    }
}

// LINEAR_ONLY instantiations carry only the truncated-linear / Potts update
// (the hot path), so their register allocation is not shaped by the
// local-memory arrays of the O(L^2) and lower-envelope rules.
template <typename T, typename M, int LMAX, int NT, int STAGES, bool LINEAR_ONLY>
__global__ void __launch_bounds__(NT) sweep_kernel(const SweepParams p) {
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ uint64_t full_bar[STAGES];
    constexpr bool FR_REGS = LMAX * sizeof(T) <= 256;
    const int tid = threadIdx.x;
    if (tid == 0) {
#pragma unroll
        for (int s = 0; s < STAGES; ++s) mbar_init(&full_bar[s], NT);
        fence_barrier_init();
    }
    __syncthreads();

    auto node_of = [&](int t, int &x, int &y) -> bool {
        y = 1 + t / p.tiles_per_row;
        const int k = (t % p.tiles_per_row) * NT + tid;
        x = ((y + p.iter) & 1) + 1 + 2 * k;
        return x <= p.W - 2;
    };

    auto issue_load = [&](int t, int s) {
        int x, y;
        const bool act = node_of(t, x, y);
        unsigned char *slot = smem + (size_t)(s * NT + tid) * p.slot_bytes;
        const unsigned char *r = p.rec + ((size_t)y * p.W + x) * p.rec_bytes;
        uint32_t bytes = 0;
        unsigned want = 0;  // coarse slots to fetch (RD_COARSE)
        if (act) {
            if (p.read_mode == RD_OWN) {
                bytes = p.rec_bytes;
            } else {
                bytes = p.d_bytes;
                if (p.read_mode == RD_COARSE) {
                    want = ~zero_mask(p, x, y) & 0xFu;
                    bytes += __popc(want) * p.m_bytes;
                }
            }
        }
        mbar_arrive_expect_tx(&full_bar[s], bytes);
        if (act) {
            if (p.read_mode == RD_OWN) {
                bulk_load(slot, r, p.rec_bytes, &full_bar[s]);
            } else {
                bulk_load(slot, r, p.d_bytes, &full_bar[s]);
#pragma unroll
                for (int d = 0; d < 4; ++d) {
                    if ((want >> d) & 1u) {
                        // The coarse node Q = (node + dir(d)) / 2 sent its message
                        // towards -dir(d); it is stored at R = Q - dir(d), slot d.
                        const int Qx = (x + dir_dx(d)) >> 1, Qy = (y + dir_dy(d)) >> 1;
                        const int Rx = Qx - dir_dx(d), Ry = Qy - dir_dy(d);
                        const unsigned char *src =
                            p.crec + ((size_t)Ry * p.cW + Rx) * p.rec_bytes + p.d_bytes + d * p.m_bytes;
                        bulk_load(slot + p.d_bytes + d * p.m_bytes, src, p.m_bytes, &full_bar[s]);
                    }
                }
            }
        }
    };

    const int first = blockIdx.x;
#pragma unroll
    for (int s = 0; s < STAGES; ++s) {
        const int t = first + s * gridDim.x;
        if (t < p.num_tiles) issue_load(t, s);
    }

    bool ok = true;
    for (int j = 0;; ++j) {
        const int t = first + j * gridDim.x;
        if (t >= p.num_tiles) break;
        const int s = j % STAGES;
        const uint32_t parity = (uint32_t)(j / STAGES) & 1u;
        // Every thread's wait is bounded; the vote makes giving up block-uniform
        // so no thread is left behind at a later __syncthreads.
        const bool got = mbar_wait_bounded(&full_bar[s], parity, p.status);
        if (!__syncthreads_and(got)) {
            ok = false;
            break;
        }
        int x, y;
        const bool act = node_of(t, x, y);
        unsigned char *slot = smem + (size_t)(s * NT + tid) * p.slot_bytes;
        if (act) {
            const unsigned zmask = zero_mask(p, x, y);
            T fr[FR_REGS ? LMAX : 1];
            int label = 0;
            if (LINEAR_ONLY || p.mode == MODE_LINEAR) {
                collect<T, M, LMAX, FR_REGS>(p, slot, zmask, fr, label);
                messages_linear<T, M, LMAX, FR_REGS>(p, slot, zmask, fr);
            } else if constexpr (!LINEAR_ONLY) {
                collect<T, M, LMAX, false>(p, slot, zmask, fr, label);
                if (p.mode == MODE_REF_MINCONV) messages_ref_minconv<T, M, LMAX>(p, slot);
                else if (p.mode == MODE_STD_MINCONV) messages_std_minconv<T, M, LMAX>(p, slot, zmask);
                else messages_std_quad<T, M, LMAX>(p, slot, zmask);
            }
            if (p.write_labels) p.labels[(size_t)y * p.W + x] = label;
            fence_proxy_async_shared();
#pragma unroll
            for (int d = 0; d < 4; ++d) {
                const int qx = x + dir_dx(d), qy = y + dir_dy(d);
                unsigned char *dst = p.rec + ((size_t)qy * p.W + qx) * p.rec_bytes + p.d_bytes + opp_dir(d) * p.m_bytes;
                bulk_store(dst, slot + p.d_bytes + d * p.m_bytes, p.m_bytes);
            }
            bulk_commit();
            bulk_wait_read_all();
        }
        __syncthreads();
        const int tn = t + STAGES * gridDim.x;
        if (tn < p.num_tiles) issue_load(tn, s);
    }
    if (!ok) {
        // A copy never completed: leave without touching shared memory again.
        return;
    }
    bulk_wait_all();
}

template <typename T, typename M, int LMAX, int NT, int STAGES, bool LINEAR_ONLY>
cudaError_t launch_one(const SweepParams &p, uint32_t slot_bytes, cudaStream_t s, int num_sms) {
    auto kern = sweep_kernel<T, M, LMAX, NT, STAGES, LINEAR_ONLY>;
    const size_t smem = (size_t)STAGES * NT * slot_bytes;
    static size_t configured = 0;  // largest dynamic smem size set so far for this instantiation
    static int occ_cache_smem = -1, occ_cache = 0;
    if (smem > configured) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        configured = smem;
    }
    int occ = 0;
    if (occ_cache_smem == (int)smem) {
        occ = occ_cache;
    } else {
        cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, NT, smem);
        if (e != cudaSuccess) return e;
        occ_cache_smem = (int)smem;
        occ_cache = occ;
    }
    if (occ < 1) return cudaErrorInvalidConfiguration;
    int grid = occ * num_sms;
    if (grid > p.num_tiles) grid = p.num_tiles;
    kern<<<grid, NT, smem, s>>>(p);
    return cudaGetLastError();
}

// Dispatch on LMAX bucket and (NT, STAGES) for one (T, M) pair.  Variants
// other than (32,1), (32,2), (64,1) fall back to (32,1).
template <typename T, typename M, int LM>
cudaError_t launch_variant(const RecordFormat &f, const SweepConfig &cfg, const SweepParams &p, cudaStream_t s,
                           int num_sms) {
    if (p.mode != MODE_LINEAR) return launch_one<T, M, LM, 32, 1, false>(p, f.slot_bytes, s, num_sms);
    if constexpr (std::is_same<T, float>::value) {
        if (cfg.nt == 64) return launch_one<T, M, LM, 64, 1, true>(p, f.slot_bytes, s, num_sms);
        if (cfg.stages == 2) return launch_one<T, M, LM, 32, 2, true>(p, f.slot_bytes, s, num_sms);
    }
    return launch_one<T, M, LM, 32, 1, true>(p, f.slot_bytes, s, num_sms);
}

// Dispatch on the LMAX bucket and (NT, STAGES) for one (T, M) pair.  Float
// grids have the (32,1), (32,2) and (64,1) variants of the linear kernel;
// everything else runs the (32,1) variant.
template <typename T, typename M>
cudaError_t launch_sweep_tm(const RecordFormat &f, const SweepConfig &cfg, const SweepParams &p, cudaStream_t s,
                            int num_sms) {
    if (f.L <= 16) return launch_variant<T, M, 16>(f, cfg, p, s, num_sms);
    if (f.L <= 32) return launch_variant<T, M, 32>(f, cfg, p, s, num_sms);
    if (f.L <= 64) return launch_variant<T, M, 64>(f, cfg, p, s, num_sms);
    if (f.L <= 128) return launch_variant<T, M, 128>(f, cfg, p, s, num_sms);
    return cudaErrorInvalidValue;
}

}  // namespace ginf_gpu
