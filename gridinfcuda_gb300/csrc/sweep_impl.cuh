// sweep_impl.cuh -- the checkerboard half-sweep kernel (one BP "iteration").
//
// Each message is computed by one thread with the reference's operation
// order (src/bp.cc:7-63): sequential min-plus scans, (a<b)?a:b minima, the
// mean by IEEE division.  FP32 and int32 results are therefore bit-identical
// to the reference's CPU code.  The kernel itself is described above
// sweep_kernel at the end of this file.
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

__device__ __forceinline__ void zero_bytes(unsigned char *p, uint32_t bytes) {
    for (uint32_t o = 0; o < bytes; o += 16) *reinterpret_cast<uint4 *>(p + o) = make_uint4(0, 0, 0, 0);
}

// val / L in T arithmetic.  With L a compile-time power of two the division is
// a multiplication by the exact reciprocal, which rounds identically.
template <typename T, int LMAX, bool EXACT>
__device__ __forceinline__ T mean_of(T sum, int L) {
    if constexpr (EXACT && (LMAX & (LMAX - 1)) == 0 && !std::is_same<T, int>::value) {
        return sum * (T(1) / T(LMAX));
    } else if constexpr (EXACT) {
        return div_labels(sum, LMAX);
    } else {
        return div_labels(sum, L);
    }
}

// Belief of one node, computed by its four lanes together: lane `dir` takes
// the 16-byte message chunks dir, dir+4, dir+8, ...  For each label,
// from = D + in_S + in_E + in_N + in_W in that order (bp.cc:10-17); the sum
// overwrites D in shared memory.  Returns the lane's first minimum (value,
// label); labels are visited in increasing order, so combining the four
// partial results by (value, label) gives the reference's first argmin
// (strict <, bp.cc:74-80).
template <typename T, typename M, int LMAX, bool EXACT>
__device__ __forceinline__ void belief_part(const SweepParams &p, unsigned char *slot, int L, int dir, T &best,
                                            int &bl) {
    constexpr int B = MIO<M, T>::B;
    constexpr int NCH = (LMAX + B - 1) / B;
    const unsigned char *mb = slot + p.d_bytes;
#pragma unroll
    for (int j = 0; j < (NCH + 3) / 4; ++j) {
        const int c = (4 * j + dir) * B;
        if (c < LMAX && (EXACT || c < L)) {
            T v[B], a[B];
            load_t<T, B>(slot + c * sizeof(T), v);
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                MIO<M, T>::load(mb + e * p.m_bytes + c * sizeof(M), a);
#pragma unroll
                for (int kk = 0; kk < B; ++kk) v[kk] = v[kk] + a[kk];
            }
            store_t<T, B>(slot + c * sizeof(T), v);
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

// Combines (value, label) partial minima of the four lanes of a node
// (lanes k, k+8, k+16, k+24): smaller value wins, equal values go to the
// lower label; 0x7fffffff marks an empty partial.
template <typename T>
__device__ __forceinline__ void argmin_combine(T &best, int &bl) {
#pragma unroll
    for (int off = 8; off <= 16; off <<= 1) {
        const T ob = __shfl_xor_sync(0xffffffffu, best, off);
        const int ol = __shfl_xor_sync(0xffffffffu, bl, off);
        const bool take = ol != 0x7fffffff && (bl == 0x7fffffff || ob < best || (!(best < ob) && ol < bl));
        if (take) {
            best = ob;
            bl = ol;
        }
    }
}

// Truncated-linear / Potts message towards `dir` (bp.cc:26-54), one lane:
// h = from - in[dir], min of h, forward and backward min-plus scans with slope
// V(0,1), truncation at min(h) + V(0,L-1), subtraction of the mean (or the
// minimum), written over in[dir].
template <typename T, typename M, int LMAX, bool EXACT>
__device__ __forceinline__ void message_linear(const SweepParams &p, unsigned char *slot, int L, int dir, T scale,
                                               T trunc) {
    constexpr int B = MIO<M, T>::B;
    unsigned char *md = slot + p.d_bytes + dir * p.m_bytes;
    T o[LMAX];
#pragma unroll
    for (int c = 0; c < LMAX; c += B) {
        if (EXACT || c < L) {
            T a[B], f[B];
            MIO<M, T>::load(md + c * sizeof(M), a);
            load_t<T, B>(slot + c * sizeof(T), f);
#pragma unroll
            for (int k = 0; k < B; ++k) o[c + k] = f[k] - a[k];
        }
    }
    T minh = o[0];
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
    T val = T(0);
#pragma unroll
    for (int i = 0; i < LMAX; ++i)
        if (EXACT || i < L) {
            o[i] = rmin(o[i], minh);
            val += o[i];
        }
    if (p.norm_min) {
        val = o[0];
#pragma unroll
        for (int i = 1; i < LMAX; ++i)
            if (EXACT || i < L) val = rmin(val, o[i]);
    } else {
        val = mean_of<T, LMAX, EXACT>(val, L);
    }
#pragma unroll
    for (int c = 0; c < LMAX; c += B) {
        if (EXACT || c < L) {
            T r[B];
#pragma unroll
            for (int k = 0; k < B; ++k) r[k] = o[c + k] - val;
            MIO<M, T>::store(md + c * sizeof(M), r);
        }
    }
}

// h = from - in[dir] into local h[] (from is over the D region of the slot).
template <typename T, typename M, int LMAX>
__device__ __forceinline__ void load_h(const unsigned char *slot, const unsigned char *md, int L, T *h) {
    constexpr int B = MIO<M, T>::B;
#pragma unroll 1
    for (int c = 0; c < L; c += B) {
        T a[B], f[B];
        MIO<M, T>::load(md + c * sizeof(M), a);
        load_t<T, B>(slot + c * sizeof(T), f);
#pragma unroll
        for (int k = 0; k < B; ++k)
            if (c + k < LMAX) h[c + k] = f[k] - a[k];
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

// Writes o[0..L) (zero padding to the chunk boundary) into message slot md.
template <typename T, typename M>
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

// Reference rule for EXPLICIT / TRUNC_QUAD (bp.cc:55-62): the same vector
// out(i) = min_j V(i,j) + from(j) goes out in all four directions, without
// subtracting the receiver's message and without normalisation.  Lane `dir`
// computes the chunks dir, dir+4, ... and writes them into all four slots.
template <typename T, typename M, int LMAX>
__device__ void messages_ref_minconv(const SweepParams &p, unsigned char *slot, int L, int dir) {
    constexpr int B = MIO<M, T>::B;
    const T *V = static_cast<const T *>(p.V);
    const T *fr = reinterpret_cast<const T *>(slot);
    unsigned char *mb = slot + p.d_bytes;
#pragma unroll 1
    for (int c = dir * B; c < L; c += 4 * B) {
        T r[B];
#pragma unroll
        for (int k = 0; k < B; ++k) {
            const int i = c + k;
            T m = T(0);
            if (i < L) {
                m = __ldg(&V[i]) + fr[0];
#pragma unroll 1
                for (int j = 0; j < L; ++j) m = rmin(m, __ldg(&V[i + (size_t)L * j]) + fr[j]);
            }
            r[k] = m;
        }
#pragma unroll 1
        for (int e = 0; e < 4; ++e) MIO<M, T>::store(mb + e * p.m_bytes + c * sizeof(M), r);
    }
}

// Standard rule, EXPLICIT model: O(L^2) min-convolution of h = from - in.
template <typename T, typename M, int LMAX>
__device__ void message_std_minconv(const SweepParams &p, unsigned char *slot, int L, int dir) {
    const T *V = static_cast<const T *>(p.V);
    unsigned char *md = slot + p.d_bytes + dir * p.m_bytes;
    T h[LMAX], o[LMAX];
    load_h<T, M, LMAX>(slot, md, L, h);
#pragma unroll 1
    for (int i = 0; i < L; ++i) {
        T m = __ldg(&V[i]) + h[0];
#pragma unroll 1
        for (int j = 1; j < L; ++j) m = rmin(m, __ldg(&V[i + (size_t)L * j]) + h[j]);
        o[i] = m;
    }
    normalise(o, L, p.norm_min);
    store_msg<T, M>(md, o, L);
}

// Two FP32 additions or subtractions in one instruction (add / sub.rn.f32x2,
// sm_100 and later); each element is rounded exactly as the scalar operation.
__device__ __forceinline__ uint64_t pack_f32x2(float x, float y) {
    uint64_t v;
    asm("mov.b64 %0, {%1, %2};" : "=l"(v) : "f"(x), "f"(y));
    return v;
}
__device__ __forceinline__ float2 unpack_f32x2(uint64_t v) {
    float2 r;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(r.x), "=f"(r.y) : "l"(v));
    return r;
}
__device__ __forceinline__ float2 add_f32x2(float ax, float ay, float bx, float by) {
    uint64_t r;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(pack_f32x2(ax, ay)), "l"(pack_f32x2(bx, by)));
    return unpack_f32x2(r);
}
__device__ __forceinline__ float2 sub_f32x2(float ax, float ay, float bx, float by) {
    uint64_t r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(pack_f32x2(ax, ay)), "l"(pack_f32x2(bx, by)));
    return unpack_f32x2(r);
}

// Minimum of three FP32 values in one instruction (three-input min.f32,
// sm_100 and later); exact, like the two-input minimum.
__device__ __forceinline__ float min3_f32(float a, float b, float c) {
    float r;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}

// The window term of output i at distance k of a quadratic message over
// h[0, N): min(h[i-k], h[i+k]), or the one that exists at the ends.
template <int N>
__device__ __forceinline__ float window_pair(const float *h, int i, int k) {
    const bool lo = i - k >= 0, hi = i + k < N;
    if (lo && hi) return fminf(h[i - k], h[i + k]);
    return lo ? h[i - k] : h[i + k];
}

// Outputs c .. c + B - 1 of the windowed quadratic transform over h[0, N)
// (padded with +inf where the caller has no labels), two at a time: the
// sums h + V(0,k) of a pair of outputs in one f32x2 addition, their minima
// as scalars, the shift subtracted in pairs.  Values are those of the scalar
// form below; sum accumulates the outputs in label order.
template <int N, int QW, int B>
__device__ __forceinline__ void window_outputs(const float *h, int c, const float *vtap, float cap, float shift,
                                               float &sum, float *r) {
#pragma unroll
    for (int k = 0; k < B; k += 2) {
        const int i = c + k;
        const float2 t0 = add_f32x2(h[i], h[i + 1], vtap[0], vtap[0]);
        float a0[QW + 1], a1[QW + 1];
#pragma unroll
        for (int k2 = 1; k2 <= QW; ++k2) {
            const float2 t = add_f32x2(window_pair<N>(h, i, k2), window_pair<N>(h, i + 1, k2), vtap[k2], vtap[k2]);
            a0[k2] = t.x;
            a1[k2] = t.y;
        }
        // The minimum over {cap, h + V(0,0), the QW window terms}, three at a time.
        float m0 = min3_f32(cap, t0.x, a0[1]), m1 = min3_f32(cap, t0.y, a1[1]);
#pragma unroll
        for (int k2 = 2; k2 <= QW; k2 += 2) {
            if (k2 + 1 <= QW) {
                m0 = min3_f32(m0, a0[k2], a0[k2 + 1]);
                m1 = min3_f32(m1, a1[k2], a1[k2 + 1]);
            } else {
                m0 = fminf(m0, a0[k2]);
                m1 = fminf(m1, a1[k2]);
            }
        }
        sum += m0;
        sum += m1;
        const float2 o = sub_f32x2(m0, m1, shift, shift);
        r[k] = o.x;
        r[k + 1] = o.y;
    }
}

// Largest truncation radius of the windowed quadratic transform (kernels are
// compiled for radius 4 and radius 8 windows).
constexpr int kQuadWindow = 8;
constexpr int kQuadWindowSmall = 4;

// Truncation radius r of a truncated-quadratic table: V(0,k) < V(0,L-1) for
// k <= r and V(0,r+1) >= V(0,L-1).  Taps further out are dominated by
// min(h) + V(0,L-1).  Returns kQuadWindow + 1 when r exceeds the window.
template <typename T>
__device__ __forceinline__ int quad_radius(const T *Vt, int L, T trunc) {
    int r = 0;
    T prev = __ldg(&Vt[0]);
    for (int k = 1; k < L && k <= kQuadWindow + 1; ++k) {
        const T v = __ldg(&Vt[(size_t)L * k]);
        if (v < prev) return kQuadWindow + 1;  // not a nondecreasing profile: use the lower envelope
        prev = v;
        if (!(v < trunc)) break;
        r = k;
    }
    // The profile must also start at its minimum and stay below the cap.
    if (!(__ldg(&Vt[0]) <= trunc)) return kQuadWindow + 1;
    return r;
}

// Standard rule, truncated quadratic, windowed exact form:
//   out(i) = min( min_{|k| <= r} h(i+k) + V(0,|k|),  min(h) + V(0,L-1) ),
// which equals the brute-force min_j h(j) + V(i,j) over the whole table
// (taps beyond r cost at least min(h) + V(0,L-1)).  Branch-free, all in
// registers: taps beyond r and labels beyond L get +inf.  With the minimum
// subtracted, that minimum is fl(min(h) + V(0,0)) (the taps are
// nondecreasing from V(0,0) and rounding is monotone), so each message is
// rounded to the store type once; with the mean subtracted (FP32 store only)
// the unnormalised values are stored exactly and corrected in a second pass.
template <typename T, typename M, int LMAX, bool EXACT, int QW>
__device__ __forceinline__ void message_quad_window(const SweepParams &p, unsigned char *slot, int L, int dir,
                                                    const T *vtap, T trunc) {
    constexpr int B = MIO<M, T>::B;
    unsigned char *md = slot + p.d_bytes + dir * p.m_bytes;
    T h[LMAX];
#pragma unroll
    for (int c = 0; c < LMAX; c += B) {
        if (EXACT || c < L) {
            T a[B], f[B];
            MIO<M, T>::load(md + c * sizeof(M), a);
            load_t<T, B>(slot + c * sizeof(T), f);
#pragma unroll
            for (int k = 0; k < B; ++k) h[c + k] = (EXACT || c + k < L) ? f[k] - a[k] : pos_inf<T>();
        } else {
#pragma unroll
            for (int k = 0; k < B; ++k) h[c + k] = pos_inf<T>();
        }
    }
    T minh = h[0];
#pragma unroll
    for (int i = 1; i < LMAX; ++i)
        if (EXACT || i < L) minh = fminf(minh, h[i]);
    const T cap = minh + trunc;
    const bool norm_min = p.norm_min != 0;
    const T shift = norm_min ? minh + vtap[0] : T(0);
    T sum = T(0);
#pragma unroll
    for (int c = 0; c < LMAX; c += B) {
        if constexpr (EXACT && std::is_same<T, float>::value) {
            T r[B];
            window_outputs<LMAX, QW, B>(h, c, vtap, cap, shift, sum, r);
            MIO<M, T>::store(md + c * sizeof(M), r);
        } else if (EXACT || c < L) {
            T r[B];
#pragma unroll
            for (int k = 0; k < B; ++k) {
                const int i = c + k;
                // Symmetric taps share their cost: min(h[i-k], h[i+k]) + V(0,k)
                // rounds exactly like the two separate sums (rounding is monotone).
                T m = fminf(cap, h[i] + vtap[0]);
#pragma unroll
                for (int k2 = 1; k2 <= QW; ++k2) {
                    const bool lo = i - k2 >= 0, hi = i + k2 < LMAX;
                    if (lo && hi) m = fminf(m, fminf(h[i - k2], h[i + k2]) + vtap[k2]);
                    else if (lo) m = fminf(m, h[i - k2] + vtap[k2]);
                    else if (hi) m = fminf(m, h[i + k2] + vtap[k2]);
                }
                if (EXACT || i < L) sum += m;
                r[k] = m - shift;
            }
            MIO<M, T>::store(md + c * sizeof(M), r);
        }
    }
    if (!norm_min) {
        const T val = mean_of<T, LMAX, EXACT>(sum, L);
#pragma unroll
        for (int c = 0; c < LMAX; c += B) {
            if (EXACT || c < L) {
                T r[B];
                MIO<M, T>::load(md + c * sizeof(M), r);
#pragma unroll
                for (int k = 0; k < B; ++k) r[k] -= val;
                MIO<M, T>::store(md + c * sizeof(M), r);
            }
        }
    }
}

// Standard rule, truncated quadratic: O(L) lower envelope of parabolas
// (Felzenszwalb & Huttenlocher, "Distance Transforms of Sampled Functions",
// Theory of Computing 8, 2012), then truncation at min(h) + V(0, L-1).
template <typename T, typename M, int LMAX>
__device__ void message_std_quad(const SweepParams &p, unsigned char *slot, int L, int dir, T s, T trunc) {
    if constexpr (std::is_same<T, int>::value) {
        return;  // integer grids use the exact O(L^2) rule instead (host side)
    } else {
        unsigned char *md = slot + p.d_bytes + dir * p.m_bytes;
        T h[LMAX], o[LMAX], z[LMAX + 1];
        int v[LMAX];
        load_h<T, M, LMAX>(slot, md, L, h);
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
        store_msg<T, M>(md, o, L);
    }
}

// FP16 message store, truncated quadratic table V(0,k) = s k^2 (k <= r <= 4),
// min-normalised: the distance transform as r passes
//   m_j(i) = min(m_{j-1}(i), m_{j-1}(i-1) + s (2j-1), m_{j-1}(i+1) + s (2j-1))
// from m_0 = h.  A path of j steps that moves at k of them pays at least
// s (1 + 3 + ... + (2k-1)) = s k^2, the first k steps, so in exact arithmetic
// m_r(i) = min_{|k| <= r} h(i+k) + s k^2: the window's value, with the sums
// rounded step by step instead of once (this store is checked against the
// FP64 run within a tolerance, not bit for bit).  Per output and pass one
// packed addition for two outputs and one three-input minimum, against the
// window's four pair minima, two three-input minima and the additions.  The
// minimum output stays min(h) exactly (every candidate beside h(i) adds a
// positive increment), so the min-normalised message is 0 at its argmin.
// Passes beyond r get an infinite increment and change nothing.
constexpr int kQuadPasses = 4;
template <typename M, int LMAX, bool EXACT>
__device__ __forceinline__ void message_quad_passes(const SweepParams &p, unsigned char *slot, int L, int dir,
                                                    const float *cpass, float trunc) {
    constexpr int B = MIO<M, float>::B;
    static_assert(LMAX % 2 == 0, "outputs come in pairs");
    const float inf = pos_inf<float>();
    unsigned char *md = slot + p.d_bytes + dir * p.m_bytes;
    float m[LMAX];
#pragma unroll
    for (int c = 0; c < LMAX; c += B) {
        if (EXACT || c < L) {
            float a[B], f[B];
            MIO<M, float>::load(md + c * sizeof(M), a);
            load_t<float, B>(slot + c * sizeof(float), f);
#pragma unroll
            for (int k = 0; k < B; k += 2) {
                const float2 d = sub_f32x2(f[k], f[k + 1], a[k], a[k + 1]);
                m[c + k] = (EXACT || c + k < L) ? d.x : inf;
                m[c + k + 1] = (EXACT || c + k + 1 < L) ? d.y : inf;
            }
        } else {
#pragma unroll
            for (int k = 0; k < B; ++k) m[c + k] = inf;
        }
    }
    // min(h), three values at a time (labels beyond L hold +inf).
    float minh = fminf(m[0], m[1]);
#pragma unroll
    for (int i = 2; i < LMAX; i += 2) minh = min3_f32(minh, m[i], m[i + 1]);
    const float cap = minh + trunc;
#pragma unroll
    for (int j = 0; j < kQuadPasses; ++j) {
        const float c = cpass[j];
        // p(i) = m(i) + c of the previous pass, two outputs per addition:
        // pprev = (p(i-2), p(i-1)), pcur = (p(i), p(i+1)), pnext = (p(i+2), p(i+3)).
        float2 pprev = make_float2(inf, inf);
        float2 pcur = add_f32x2(m[0], m[1], c, c);
#pragma unroll
        for (int i = 0; i < LMAX; i += 2) {
            const float2 pnext = i + 2 < LMAX ? add_f32x2(m[i + 2], m[i + 3], c, c) : make_float2(inf, inf);
            const float n0 = min3_f32(m[i], pprev.y, pcur.y);
            const float n1 = min3_f32(m[i + 1], pcur.x, pnext.x);
            m[i] = n0;
            m[i + 1] = n1;
            pprev = pcur;
            pcur = pnext;
        }
    }
#pragma unroll
    for (int c = 0; c < LMAX; c += B) {
        if (EXACT || c < L) {
            float r[B];
#pragma unroll
            for (int k = 0; k < B; k += 2) {
                const float2 o = sub_f32x2(fminf(m[c + k], cap), fminf(m[c + k + 1], cap), minh, minh);
                r[k] = o.x;
                r[k + 1] = o.y;
            }
            MIO<M, float>::store(md + c * sizeof(M), r);
        }
    }
}

enum { KIND_LINEAR = 0, KIND_QUAD = 1, KIND_GENERAL = 2, KIND_QUAD4 = 3, KIND_QUADPASS = 4 };

// Constants a launch reads from its smoothness table: slope V(0,1) and
// truncation V(0,L-1) (bp.cc:35,43), and for the quadratic kernels the taps
// V(0,k) (+inf beyond the truncation radius) and that radius.
template <typename T>
struct TableConsts {
    T scale, trunc;
    T vtap[kQuadWindow + 1];
    T cpass[kQuadPasses];  // KIND_QUADPASS: increments s (2j-1), +inf beyond the radius
    int qr;
};

template <typename T, int KIND>
__device__ __forceinline__ TableConsts<T> table_consts(const void *V, int L) {
    TableConsts<T> tc;
    const T *Vt = static_cast<const T *>(V);
    tc.scale = __ldg(&Vt[L]);
    tc.trunc = __ldg(&Vt[(size_t)L * (L - 1)]);
    tc.qr = kQuadWindow + 1;
    if constexpr ((KIND == KIND_QUAD || KIND == KIND_QUAD4) && sizeof(T) == 4) {
        tc.qr = quad_radius(Vt, L, tc.trunc);
#pragma unroll
        for (int k = 0; k <= kQuadWindow; ++k) tc.vtap[k] = k <= tc.qr ? __ldg(&Vt[(size_t)L * k]) : pos_inf<T>();
    }
    if constexpr (KIND == KIND_QUADPASS && sizeof(T) == 4) {
        tc.qr = quad_radius(Vt, L, tc.trunc);
#pragma unroll
        for (int j = 0; j < kQuadPasses; ++j) tc.cpass[j] = j < tc.qr ? tc.scale * T(2 * j + 1) : pos_inf<T>();
    }
    return tc;
}

// One tile of one checkerboard half-sweep.  Block = NW warps, tile = 8*NW
// consecutive same-colour nodes of one row; lane = (node k = lane & 7,
// direction dir = lane >> 3).
//   1. lane (k, 0) brings the node's whole record into the node's padded
//      shared-memory slot with one bulk TMA copy (complete_tx on the
//      block's mbarrier; the first sweep of a level fetches D and, per lane,
//      one incoming slot from the coarser level instead);
//   2. incoming slots whose sender is a border node are zeroed;
//   3. the node's four lanes form the belief over D and its first argmin;
//   4. lane (k, dir) forms the message towards dir over its incoming slot;
//   5. lane (k, dir) bulk-stores it into the neighbour's record, slot
//      OPP(dir).
// Lanes 0-7 of a warp are eight different nodes with the same direction; the
// odd slot stride in 16-byte chunks puts their 128-bit shared accesses in
// eight different bank groups.  KIND selects the message rule compiled in:
// the truncated-linear update only (the hot path, with a clean register
// allocation), the standard truncated-quadratic update (window radius 8, or
// 4 for KIND_QUAD4), or every rule.  Returns false, block-uniformly, when the
// bounded wait for the tile's copies gave up.
// SPL warps share each group of eight nodes (1, or 2 for the split kernel:
// warp w serves nodes (w / SPL) * 8 + k).
template <int NW, int SPL = 1>
__device__ __forceinline__ bool tile_node(const SweepParams &p, int t, int &x, int &y) {
    const int node = ((threadIdx.x >> 5) / SPL) * 8 + (threadIdx.x & 7);
    y = 1 + t / p.tiles_per_row;
    x = ((y + p.iter) & 1) + 1 + 2 * ((t % p.tiles_per_row) * (NW / SPL) * 8 + node);
    return x <= p.W - 2;
}

// Phase 1 of a tile: every thread announces the bytes it will receive on the
// block's mbarrier, then lane (k, 0) brings the node's whole record into the
// node's padded shared-memory slot with one bulk TMA copy (the first sweep of
// a level fetches D and, per lane, one incoming slot from the coarser level
// instead).
template <int NW, int SPL = 1>
__device__ __forceinline__ void tile_load(const SweepParams &p, int t, unsigned char *smem, uint64_t *bar) {
    const int dir = (threadIdx.x & 31) >> 3;
    const int node = ((threadIdx.x >> 5) / SPL) * 8 + (threadIdx.x & 7);
    unsigned char *slot = smem + (size_t)node * p.slot_bytes;
    int x, y;
    // With SPL warps per node group only the first of them issues copies;
    // every thread still arrives on the mbarrier.
    const bool act = tile_node<NW, SPL>(p, t, x, y) && ((threadIdx.x >> 5) % SPL) == 0;
    uint32_t bytes = 0;
    bool want = false;
    if (act) {
        if (p.read_mode == RD_OWN) {
            if (dir == 0) bytes = p.rec_bytes;
        } else {
            if (dir == 0) bytes = p.d_bytes;
            if (p.read_mode == RD_COARSE) {
                want = !((zero_mask(p, x, y) >> dir) & 1u);
                if (want) bytes += p.m_bytes;
            }
        }
    }
    mbar_arrive_expect_tx(bar, bytes);
    if (act) {
        const unsigned char *r = p.rec + ((size_t)y * p.W + x) * p.rec_bytes;
        if (p.read_mode == RD_OWN) {
            if (dir == 0) bulk_load(slot, r, p.rec_bytes, bar);
        } else {
            if (dir == 0) bulk_load(slot, r, p.d_bytes, bar);
            if (want) {
                // The coarse node Q = (node + dir) / 2 sent its message towards
                // -dir; it is stored at R = Q - dir, slot dir.
                const int Qx = (x + dir_dx(dir)) >> 1, Qy = (y + dir_dy(dir)) >> 1;
                const int Rx = Qx - dir_dx(dir), Ry = Qy - dir_dy(dir);
                const unsigned char *src = p.crec + ((size_t)Ry * p.cW + Rx) * p.rec_bytes + p.d_bytes + dir * p.m_bytes;
                bulk_load(slot + p.d_bytes + dir * p.m_bytes, src, p.m_bytes, bar);
            }
        }
    }
}

// Phase 2 of a tile (lane = (node k = lane & 7, direction dir = lane >> 3)):
//   wait for the copies (bounded; the vote makes giving up block-uniform, so
//   no thread is left behind at a later barrier -- returns false then);
//   zero incoming slots whose sender is a border node; the node's four lanes
//   form the belief over D and its first argmin; lane (k, dir) forms the
//   message towards dir over its incoming slot and bulk-stores it into the
//   neighbour's record, slot OPP(dir).
// Lanes 0-7 of a warp are eight different nodes with the same direction; the
// odd slot stride in 16-byte chunks puts their 128-bit shared accesses in
// eight different bank groups.  KIND selects the message rule compiled in:
// the truncated-linear update only (the hot path, with a clean register
// allocation), the standard truncated-quadratic update (window radius 8, or
// 4 for KIND_QUAD4), or every rule.
// DIRECT (64-byte messages only): the messages leave through ordinary
// 16-byte stores instead of one bulk copy each, which pays on large launches
// (the copy engine's per-copy cost dominates 64-byte copies) and not on small,
// L2-resident ones.
template <typename T, typename M, int LMAX, bool EXACT, int NW, int KIND, bool DIRECT = false>
__device__ __forceinline__ bool tile_finish(const SweepParams &p, const TableConsts<T> &tc, int t,
                                            unsigned char *smem, uint64_t *bar, uint32_t &parity) {
    const int dir = (threadIdx.x & 31) >> 3;
    const int node = (threadIdx.x >> 5) * 8 + (threadIdx.x & 7);
    const int L = EXACT ? LMAX : p.L;
    unsigned char *slot = smem + (size_t)node * p.slot_bytes;
    const bool got = mbar_wait_bounded(bar, parity, p.status);
    parity ^= 1u;
    if (!__syncthreads_and(got)) return false;
    int x, y;
    const bool act = tile_node<NW>(p, t, x, y);
    if (act && ((zero_mask(p, x, y) >> dir) & 1u)) zero_bytes(slot + p.d_bytes + dir * p.m_bytes, p.m_bytes);
    __syncwarp();
    T best = pos_inf<T>();
    int label = 0x7fffffff;
    if (act) belief_part<T, M, LMAX, EXACT>(p, slot, L, dir, best, label);
    argmin_combine(best, label);
    __syncwarp();
    if (act) {
        if constexpr (KIND == KIND_LINEAR) {
            message_linear<T, M, LMAX, EXACT>(p, slot, L, dir, tc.scale, tc.trunc);
        } else if constexpr (KIND == KIND_QUADPASS) {
            if constexpr (std::is_same<T, float>::value && sizeof(M) == 2)
                message_quad_passes<M, LMAX, EXACT>(p, slot, L, dir, tc.cpass, tc.trunc);
        } else if constexpr (KIND == KIND_QUAD || KIND == KIND_QUAD4) {
            constexpr int QW = KIND == KIND_QUAD4 ? kQuadWindowSmall : kQuadWindow;
            if constexpr (sizeof(T) == 4 && !std::is_same<T, int>::value) {
                if (tc.qr <= QW) message_quad_window<T, M, LMAX, EXACT, QW>(p, slot, L, dir, tc.vtap, tc.trunc);
                else message_std_quad<T, M, LMAX>(p, slot, L, dir, tc.scale, tc.trunc);
            } else {
                message_std_quad<T, M, LMAX>(p, slot, L, dir, tc.scale, tc.trunc);
            }
        } else {
            if (p.mode == MODE_LINEAR) message_linear<T, M, LMAX, EXACT>(p, slot, L, dir, tc.scale, tc.trunc);
            else if (p.mode == MODE_REF_MINCONV) messages_ref_minconv<T, M, LMAX>(p, slot, L, dir);
            else if (p.mode == MODE_STD_MINCONV) message_std_minconv<T, M, LMAX>(p, slot, L, dir);
            else message_std_quad<T, M, LMAX>(p, slot, L, dir, tc.scale, tc.trunc);
        }
    }
    if constexpr (DIRECT) {
        static_assert(EXACT && LMAX * sizeof(M) == 64, "direct stores are for 64-byte messages");
        __syncwarp();
        if (act) {
            if (dir == 0 && p.write_labels) p.labels[(size_t)y * p.W + x] = label;
            const int qx = x + dir_dx(dir), qy = y + dir_dy(dir);
            uint4 *dst = reinterpret_cast<uint4 *>(p.rec + ((size_t)qy * p.W + qx) * p.rec_bytes + p.d_bytes +
                                                   opp_dir(dir) * p.m_bytes);
            const uint4 *src = reinterpret_cast<const uint4 *>(slot + p.d_bytes + dir * p.m_bytes);
#pragma unroll
            for (int c = 0; c < 4; ++c) dst[c] = src[c];
        }
        // The slots just read are refilled by the next tile's bulk copies.
        fence_proxy_async_shared();
    } else {
        // Every lane orders its shared-memory writes before the async-proxy
        // reads of the bulk stores (lanes may store slots other lanes wrote).
        fence_proxy_async_shared();
        __syncwarp();
        if (act) {
            if (dir == 0 && p.write_labels) p.labels[(size_t)y * p.W + x] = label;
            const int qx = x + dir_dx(dir), qy = y + dir_dy(dir);
            unsigned char *dst =
                p.rec + ((size_t)qy * p.W + qx) * p.rec_bytes + p.d_bytes + opp_dir(dir) * p.m_bytes;
            bulk_store(dst, slot + p.d_bytes + dir * p.m_bytes, p.m_bytes);
            bulk_commit();
            bulk_wait_read_all();
        }
    }
    __syncthreads();
    return true;
}

// ---------------------------------------------------------------------------
// Split kernel: FP32 records, L = 128, truncated quadratic with the windowed
// transform (window radius QW).  A lane holding a whole 128-label message
// needs ~235 registers, which leaves 8 warps per SM and the kernel
// latency-bound; here two warps serve each group of eight nodes and a lane
// (k, dir) of warp 2g + hf computes labels [64 hf, 64 hf + 64) of node
// g * 8 + k's message towards dir, with h read over that range plus a QW-label
// halo.  Results are bit-identical to message_quad_window:
//   - min(h) is the fminf of the two halves' minima (fminf is exact);
//   - each output value is the same expression over the same h values (h is
//     +inf outside [0, L), as the single-lane form's missing taps);
//   - the mean's sum stays sequential in label order: half 0 sums its 64
//     outputs from zero, half 1 continues from that partial sum;
//   - the argmin combines the halves' first minima by (value, label).
// Shared words exchanged between the two warps of a group.
template <int NW>
struct SplitXch {
    float minh[NW][32];      // lane's minimum of h over its own half
    float sum[NW / 2][32];   // half 0's sequential partial sum of its outputs
    float mean[NW / 2][32];  // the finished mean, from half 1
    float best[NW][8];       // node's belief minimum over the warp's half
    int label[NW][8];        // and its first label
};

// Belief over labels [base, base + 64) of one node by its four lanes of one
// warp (chunks base + 4 (4 j + dir)); see belief_part.
__device__ __forceinline__ void belief_half(const SweepParams &p, unsigned char *slot, int dir, int base, float &best,
                                            int &bl) {
    const unsigned char *mb = slot + p.d_bytes;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const int c = base + (4 * j + dir) * 4;
        float v[4], a[4];
        load_t<float, 4>(slot + c * sizeof(float), v);
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            MIO<float, float>::load(mb + e * p.m_bytes + c * sizeof(float), a);
#pragma unroll
            for (int kk = 0; kk < 4; ++kk) v[kk] = v[kk] + a[kk];
        }
        store_t<float, 4>(slot + c * sizeof(float), v);
#pragma unroll
        for (int kk = 0; kk < 4; ++kk) {
            if (bl == 0x7fffffff || v[kk] < best) {
                best = v[kk];
                bl = c + kk;
            }
        }
    }
}

// One tile of the split kernel (8 * NW / 2 nodes).  Block barriers: after the
// beliefs (the halo of h reads the other half's), after h is loaded (the
// outgoing messages overwrite the incoming slots), after half 0's partial
// sum, and after half 1's mean.  Each half bulk-stores its own 256 bytes.
template <int NW, int QW>
__device__ __forceinline__ bool tile_finish_split(const SweepParams &p, const TableConsts<float> &tc, int t,
                                                  unsigned char *smem, uint64_t *bar, uint32_t &parity,
                                                  SplitXch<NW> &xs) {
    constexpr int L = 128, HL = 64, NH = HL + 2 * QW;
    static_assert(QW % 4 == 0, "the halo is whole 16-byte chunks");
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int hf = w & 1, g = w >> 1;
    const int dir = lane >> 3, k = lane & 7;
    const int base = hf * HL;
    unsigned char *slot = smem + (size_t)(g * 8 + k) * p.slot_bytes;
    unsigned char *md = slot + p.d_bytes + dir * p.m_bytes;
    const bool got = mbar_wait_bounded(bar, parity, p.status);
    parity ^= 1u;
    if (!__syncthreads_and(got)) return false;
    int x, y;
    const bool act = tile_node<NW, 2>(p, t, x, y);
    // Each half zeroes, then sums, only its own labels of the incoming slots.
    if (act && ((zero_mask(p, x, y) >> dir) & 1u)) zero_bytes(md + base * sizeof(float), HL * sizeof(float));
    __syncwarp();
    float best = pos_inf<float>();
    int label = 0x7fffffff;
    if (act) belief_half(p, slot, dir, base, best, label);
    argmin_combine(best, label);
    if (dir == 0) {
        xs.best[w][k] = best;
        xs.label[w][k] = label;
    }
    __syncthreads();
    {
        const float ob = xs.best[w ^ 1][k];
        const int ol = xs.label[w ^ 1][k];
        if (ol != 0x7fffffff && (label == 0x7fffffff || ob < best || (!(best < ob) && ol < label))) label = ol;
    }
    float h[NH];
    float mloc = pos_inf<float>();
    if (act) {
#pragma unroll
        for (int c = 0; c < NH; c += 4) {
            // Chunk labels base - QW + c .. +3: below 0 only for half 0's
            // leading halo, at or above L only for half 1's trailing halo.
            const bool in = (c >= QW || hf == 1) && (c < HL + QW || hf == 0);
            if (in) {
                const int j0 = base - QW + c;
                float a[4], f[4];
                MIO<float, float>::load(md + j0 * sizeof(float), a);
                load_t<float, 4>(slot + j0 * sizeof(float), f);
#pragma unroll
                for (int kk = 0; kk < 4; ++kk) h[c + kk] = f[kk] - a[kk];
            } else {
#pragma unroll
                for (int kk = 0; kk < 4; ++kk) h[c + kk] = pos_inf<float>();
            }
        }
#pragma unroll
        for (int i = QW; i < QW + HL; ++i) mloc = fminf(mloc, h[i]);
    }
    xs.minh[w][lane] = mloc;
    __syncthreads();
    // Outputs go straight into the lane's half of the incoming slot: final
    // with the minimum subtracted, unnormalised (and corrected below) with
    // the mean subtracted.
    const bool norm_min = p.norm_min != 0;
    unsigned char *mh = md + base * sizeof(float);
    if (act) {
        const float minh = hf == 0 ? fminf(mloc, xs.minh[w ^ 1][lane]) : fminf(xs.minh[w ^ 1][lane], mloc);
        const float cap = minh + tc.trunc;
        const float shift = norm_min ? minh + tc.vtap[0] : 0.f;
        float sum = 0.f;
#pragma unroll
        for (int c = 0; c < HL; c += 4) {
            // h[QW .. QW + HL) are this half's labels; the halo (+inf off the
            // grid of labels) lies on both sides, so no output is at an end.
            float r[4];
            window_outputs<NH, QW, 4>(h, c + QW, tc.vtap, cap, shift, sum, r);
            MIO<float, float>::store(mh + c * sizeof(float), r);
        }
        if (hf == 0) xs.sum[g][lane] = sum;
    }
    if (!norm_min) {
        __syncthreads();
        if (act && hf == 1) {
            float s = xs.sum[g][lane];
#pragma unroll
            for (int c = 0; c < HL; c += 4) {
                float r[4];
                MIO<float, float>::load(mh + c * sizeof(float), r);
#pragma unroll
                for (int kk = 0; kk < 4; ++kk) s += r[kk];
            }
            xs.mean[g][lane] = mean_of<float, L, true>(s, L);
        }
        __syncthreads();
        if (act) {
            const float val = xs.mean[g][lane];
#pragma unroll
            for (int c = 0; c < HL; c += 4) {
                float r[4];
                MIO<float, float>::load(mh + c * sizeof(float), r);
#pragma unroll
                for (int kk = 0; kk < 4; ++kk) r[kk] -= val;
                MIO<float, float>::store(mh + c * sizeof(float), r);
            }
        }
    }
    // Each lane stores only what it wrote itself.
    fence_proxy_async_shared();
    if (act) {
        if (hf == 0 && dir == 0 && p.write_labels) p.labels[(size_t)y * p.W + x] = label;
        const int qx = x + dir_dx(dir), qy = y + dir_dy(dir);
        unsigned char *dst = p.rec + ((size_t)qy * p.W + qx) * p.rec_bytes + p.d_bytes + opp_dir(dir) * p.m_bytes;
        bulk_store(dst + base * sizeof(float), mh, HL * sizeof(float));
        bulk_commit();
        bulk_wait_read_all();
    }
    __syncthreads();
    return true;
}

template <int NW, int QW>
__global__ void __launch_bounds__(NW * 32, 5) sweep_kernel_split(const SweepParams p) {
    static_assert(NW % 2 == 0, "warps come in pairs");
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ uint64_t full_bar;
    __shared__ SplitXch<NW> xs;
    launch_dependents();
    const TableConsts<float> tc = table_consts<float, KIND_QUAD>(p.V, 128);
    if (threadIdx.x == 0) {
        mbar_init(&full_bar, NW * 32);
        fence_barrier_init();
    }
    __syncthreads();
    grid_dependency_wait();
    int t = blockIdx.x;
    if (t < p.num_tiles) tile_load<NW, 2>(p, t, smem, &full_bar);
    uint32_t parity = 0;
    for (; t < p.num_tiles; t += gridDim.x) {
        if (!tile_finish_split<NW, QW>(p, tc, t, smem, &full_bar, parity, xs)) return;
        const int tn = t + gridDim.x;
        if (tn < p.num_tiles) tile_load<NW, 2>(p, tn, smem, &full_bar);
    }
    bulk_wait_all();
}

// One checkerboard half-sweep of one level: blocks take tiles in turn, each
// issuing the copies of its next tile as soon as the current one is done.
template <typename T, typename M, int LMAX, bool EXACT, int NW, int KIND, bool DIRECT>
__device__ __forceinline__ void sweep_body(const SweepParams &p) {
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ uint64_t full_bar;
    // The next half-sweep may be launched now; its blocks take SM slots as
    // these retire and wait below before touching any record.
    launch_dependents();
    const TableConsts<T> tc = table_consts<T, KIND>(p.V, EXACT ? LMAX : p.L);
    if (threadIdx.x == 0) {
        mbar_init(&full_bar, NW * 32);
        fence_barrier_init();
    }
    __syncthreads();
    // Records (and labels) are written by the previous kernel in the stream.
    grid_dependency_wait();
    int t = blockIdx.x;
    if (t < p.num_tiles) tile_load<NW>(p, t, smem, &full_bar);
    uint32_t parity = 0;
    for (; t < p.num_tiles; t += gridDim.x) {
        if (!tile_finish<T, M, LMAX, EXACT, NW, KIND, DIRECT>(p, tc, t, smem, &full_bar, parity)) return;
        const int tn = t + gridDim.x;
        if (tn < p.num_tiles) tile_load<NW>(p, tn, smem, &full_bar);
    }
    bulk_wait_all();
}

template <typename T, typename M, int LMAX, bool EXACT, int NW, int KIND, bool DIRECT = false>
__global__ void __launch_bounds__(NW * 32) sweep_kernel(const SweepParams p) {
    sweep_body<T, M, LMAX, EXACT, NW, KIND, DIRECT>(p);
}

// The same kernel with room for MINB blocks per SM in the register
// allocation.  The L = 128 quadratic kernels with FP16 messages use it with
// six (168 registers): their packed window form would otherwise take every
// register.  (Any explicit bound, even one block, changes the allocation, so
// the other kernels have none.)
template <typename T, typename M, int LMAX, bool EXACT, int NW, int KIND, int MINB>
__global__ void __launch_bounds__(NW * 32, MINB) sweep_kernel_bounded(const SweepParams p) {
    sweep_body<T, M, LMAX, EXACT, NW, KIND, false>(p);
}

// Per-kernel launch state (one per kernel instantiation, in static storage).
struct LaunchCache {
    SmemLimit smem;
    OccupancyMemo occ;
};

// Launches one half-sweep kernel over tiles of `nodes` nodes, NW warps per
// block, one block per resident slot of every SM (fewer if there are fewer
// tiles).
template <typename K>
cudaError_t launch_tiles(K kern, LaunchCache &lc_state, int NW, int nodes, const SweepParams &params,
                         uint32_t slot_bytes, cudaStream_t s, int num_sms) {
    // The tiling follows the variant actually launched.
    SweepParams p = params;
    const int n1 = p.W >= 3 ? (p.W - 3) / 2 + 1 : 0;
    p.tiles_per_row = (n1 + nodes - 1) / nodes;
    p.num_tiles = p.H >= 3 ? (p.H - 2) * p.tiles_per_row : 0;
    if (p.num_tiles <= 0) return cudaSuccess;
    const size_t smem = (size_t)nodes * slot_bytes;
    cudaError_t e = lc_state.smem.ensure(kern, smem);
    if (e != cudaSuccess) return e;
    int occ = 0;
    e = lc_state.occ.blocks(kern, NW * 32, smem, occ);
    if (e != cudaSuccess) return e;
    if (occ < 1) return cudaErrorInvalidConfiguration;
    int grid = occ * num_sms;
    if (grid > p.num_tiles) grid = p.num_tiles;
    // Programmatic stream serialisation: this launch may begin while the
    // previous kernel of the stream finishes (the kernel waits for it before
    // reading records).
    cudaLaunchConfig_t lc = {};
    lc.gridDim = dim3(grid);
    lc.blockDim = dim3(NW * 32);
    lc.dynamicSmemBytes = smem;
    lc.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    lc.attrs = attr;
    lc.numAttrs = 1;
    return cudaLaunchKernelEx(&lc, kern, p);
}

template <typename T, typename M, int LMAX, bool EXACT, int NW, int KIND, bool DIRECT = false>
cudaError_t launch_one(const SweepParams &params, uint32_t slot_bytes, cudaStream_t s, int num_sms) {
    static LaunchCache cache;
    if constexpr ((KIND == KIND_QUAD || KIND == KIND_QUAD4 || KIND == KIND_QUADPASS) && sizeof(M) == 2 &&
                  LMAX == 128 && !DIRECT) {
        return launch_tiles(sweep_kernel_bounded<T, M, LMAX, EXACT, NW, KIND, 6>, cache, NW, NW * 8, params,
                            slot_bytes, s, num_sms);
    } else {
        return launch_tiles(sweep_kernel<T, M, LMAX, EXACT, NW, KIND, DIRECT>, cache, NW, NW * 8, params, slot_bytes,
                            s, num_sms);
    }
}

template <int NW, int QW>
cudaError_t launch_split(const SweepParams &params, uint32_t slot_bytes, cudaStream_t s, int num_sms) {
    static LaunchCache cache;
    return launch_tiles(sweep_kernel_split<NW, QW>, cache, NW, NW / 2 * 8, params, slot_bytes, s, num_sms);
}

template <typename T, typename M, int LM>
cudaError_t launch_variant(const RecordFormat &f, const SweepConfig &cfg, const SweepParams &p, cudaStream_t s,
                           int num_sms) {
    const bool exact = f.L == LM;
    if (p.mode == MODE_STD_QUAD) {
        // The host measured the truncation radius (quad_radius_host); radius-4
        // windows run the cheaper 9-tap kernel.
        if constexpr (std::is_same<T, float>::value && std::is_same<M, float>::value && LM == 128) {
            // FP32 records at L = 128: two warps per eight nodes (register relief).
            if (exact && p.quad_radius <= kQuadWindowSmall) return launch_split<4, 4>(p, f.slot_bytes, s, num_sms);
            if (exact && p.quad_radius <= kQuadWindow) return launch_split<4, 8>(p, f.slot_bytes, s, num_sms);
        }
        if constexpr (std::is_same<T, float>::value && sizeof(M) == 2) {
            // FP16 store and an exactly quadratic table: the pass form.
            if (p.quad_exact && p.quad_radius <= kQuadPasses) {
                if (exact) return launch_one<T, M, LM, true, 2, KIND_QUADPASS>(p, f.slot_bytes, s, num_sms);
                return launch_one<T, M, LM, false, 2, KIND_QUADPASS>(p, f.slot_bytes, s, num_sms);
            }
        }
        if (p.quad_radius <= kQuadWindowSmall) {
            if (exact) return launch_one<T, M, LM, true, 2, KIND_QUAD4>(p, f.slot_bytes, s, num_sms);
            return launch_one<T, M, LM, false, 2, KIND_QUAD4>(p, f.slot_bytes, s, num_sms);
        }
        if (exact) return launch_one<T, M, LM, true, 2, KIND_QUAD>(p, f.slot_bytes, s, num_sms);
        return launch_one<T, M, LM, false, 2, KIND_QUAD>(p, f.slot_bytes, s, num_sms);
    }
    if (p.mode != MODE_LINEAR) return launch_one<T, M, LM, false, 2, KIND_GENERAL>(p, f.slot_bytes, s, num_sms);
    if (!exact) return launch_one<T, M, LM, false, 2, KIND_LINEAR>(p, f.slot_bytes, s, num_sms);
    if constexpr (std::is_same<T, float>::value) {
        if (cfg.nt == 8) return launch_one<T, M, LM, true, 1, KIND_LINEAR>(p, f.slot_bytes, s, num_sms);
        if (cfg.nt == 32) return launch_one<T, M, LM, true, 4, KIND_LINEAR>(p, f.slot_bytes, s, num_sms);
        if constexpr (LM * sizeof(M) == 64) {
            const int n1 = p.W >= 3 ? (p.W - 3) / 2 + 1 : 0;
            const long tiles = p.H >= 3 ? (long)(p.H - 2) * ((n1 + 15) / 16) : 0;
            if (tiles >= kDirectStoreTiles)
                return launch_one<T, M, LM, true, 2, KIND_LINEAR, true>(p, f.slot_bytes, s, num_sms);
        }
    }
    return launch_one<T, M, LM, true, 2, KIND_LINEAR>(p, f.slot_bytes, s, num_sms);
}

// Dispatch on the LMAX bucket for one (T, M) pair.  L equal to the bucket
// runs a kernel specialised for that L; float grids have 8-, 16- and 32-node
// tile variants of it, everything else 16-node tiles.
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
