// warmnet.cu -- the learned warm start: a small convolutional network that
// maps the costs of a pyramid level to the messages its nodes should start
// from (on the beliefs' scale), with
// hand-written tensor-core kernels -- the forward, data-gradient and
// weight-gradient convolutions on tcgen05 with tensor-memory accumulators
// (conv_tc.cu) -- the loss, ReLU, bias-gradient and Adam kernels, and a
// checkpoint format.
//
// Network (L labels, h hidden channels): conv3x3(L->h) ReLU, conv3x3(h->h)
// ReLU, conv3x3(h->h) ReLU, conv3x3(h->L); zero padding; activations NHWC.
// Input x = D_t / 4^t (the level's costs per fine node), output
// y = x + net(x), trained towards (D_t + m) / 4^t, m the message sums of a
// long hierarchical BP run (the finest level's, averaged per block, or the
// level's own).  Rounding points (mirrored by oracle/warmnet_ref.py):
// x, weights and hidden activations in BF16; sums in FP32; the output and
// every gradient in FP32, rounded to BF16 where they feed a tensor-core
// product.  The reference has no learned component: this whole file is new.
#include <cuda_bf16.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "ginf_gb300.h"
#include "ginf_internal.h"

namespace ginf_gpu {

cudaError_t conv_fwd_tc(int cin, int cout, bool relu, bool out_f32, const __nv_bfloat16 *in, const __nv_bfloat16 *w,
                        const float *bias, int nimg, int h, int wd, void *out, const float *res, int *status,
                        cudaStream_t s);
cudaError_t conv_wgrad_tc(int cin, int cout, const __nv_bfloat16 *dout, const __nv_bfloat16 *in, int nimg, int h,
                          int wd, float *partials, int max_parts, int *parts, int *status, cudaStream_t s);

namespace {

constexpr int kThreads = 256;

inline unsigned nblocks(size_t n, int per = kThreads) { return (unsigned)((n + per - 1) / per); }

__device__ __forceinline__ uint32_t pack_bf16(__nv_bfloat16 lo, __nv_bfloat16 hi) {
    return (uint32_t)__bfloat16_as_ushort(lo) | ((uint32_t)__bfloat16_as_ushort(hi) << 16);
}


struct Geo {
    int n, h, w;  // images, rows, columns
};

// Pixels per bias-gradient partial sum, added in a fixed order by
// k_reduce_partials.
constexpr int kChunk = 1024;

// Bias gradient partials: sum over a chunk of pixels of g[p][c] (FP32).
// 256 threads = 256 / C groups of C channels (C divides 256); group k sums
// the chunk's pixels k, k + groups, ..., then the groups are added in order.
__global__ void __launch_bounds__(256) k_bias_partials(const float *__restrict__ g, int npix, int C,
                                                        float *__restrict__ partials) {
    __shared__ float red[256];
    const int groups = (int)blockDim.x / C, c = (int)threadIdx.x % C, grp = (int)threadIdx.x / C;
    const int pbeg = blockIdx.x * kChunk, pend = min(npix, pbeg + kChunk);
    float s = 0.f;
#pragma unroll 8
    for (int p = pbeg + grp; p < pend; p += groups) s += g[(size_t)p * C + c];
    red[threadIdx.x] = s;
    __syncthreads();
    if ((int)threadIdx.x < C) {
        float tot = 0.f;
        for (int k = 0; k < groups; ++k) tot += red[k * C + threadIdx.x];
        partials[(size_t)blockIdx.x * C + threadIdx.x] = tot;
    }
}

// out[i] = sum over chunks k of partials[k][i], in chunk order; eight
// partials loaded ahead of their additions.
__global__ void k_reduce_partials(const float *__restrict__ partials, int chunks, int n, float *__restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float s = 0.f;
    int k = 0;
    for (; k + 8 <= chunks; k += 8) {
        float v[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) v[j] = partials[(size_t)(k + j) * n + i];
#pragma unroll
        for (int j = 0; j < 8; ++j) s += v[j];
    }
    for (; k < chunks; ++k) s += partials[(size_t)k * n + i];
    out[i] = s;
}

// Flipped, transposed weights for the data gradient:
// wf[ci][tap'][co] = w[co][8 - tap'][ci].
__global__ void k_flip_weights(const __nv_bfloat16 *__restrict__ w, int cin, int cout, __nv_bfloat16 *__restrict__ wf) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= cin * 9 * cout) return;
    const int co = i % cout, tap = (i / cout) % 9, ci = i / (cout * 9);
    wf[i] = w[((size_t)co * 9 + (8 - tap)) * cin + ci];
}

// Round to BF16, eight values per thread (two 16-byte loads, one 16-byte
// store) when both buffers are 16-byte aligned, grid-stride, scalar tail.
__global__ void k_f32_to_bf16(const float *__restrict__ a, __nv_bfloat16 *__restrict__ b, size_t n) {
    const size_t n8 = (((uintptr_t)a | (uintptr_t)b) & 15) == 0 ? n / 8 : 0;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    for (size_t i = t; i < n8; i += stride) {
        const float4 lo = reinterpret_cast<const float4 *>(a)[2 * i], hi = reinterpret_cast<const float4 *>(a)[2 * i + 1];
        reinterpret_cast<uint4 *>(b)[i] =
            make_uint4(pack_bf16(__float2bfloat16_rn(lo.x), __float2bfloat16_rn(lo.y)),
                       pack_bf16(__float2bfloat16_rn(lo.z), __float2bfloat16_rn(lo.w)),
                       pack_bf16(__float2bfloat16_rn(hi.x), __float2bfloat16_rn(hi.y)),
                       pack_bf16(__float2bfloat16_rn(hi.z), __float2bfloat16_rn(hi.w)));
    }
    for (size_t i = n8 * 8 + t; i < n; i += stride) b[i] = __float2bfloat16_rn(a[i]);
}

void f32_to_bf16(const float *a, __nv_bfloat16 *b, size_t n, cudaStream_t s) {
    const size_t blocks = (n / 8 + kThreads - 1) / kThreads;
    k_f32_to_bf16<<<(unsigned)(blocks < 1 ? 1 : (blocks > 4096 ? 4096 : blocks)), kThreads, 0, s>>>(a, b, n);
}

// Loss = mean((y - t)^2) (per-block double partials), dy = 2 (y - t) / n.
// Four values per thread and step (16-byte accesses) when the buffers are
// 16-byte aligned; each four squares are summed in FP32 before the FP64
// accumulation (a quarter of the FP64 additions).
__global__ void k_mse(const float *__restrict__ y, const float *__restrict__ t, size_t n, float *__restrict__ dy,
                      double *__restrict__ partials) {
    double s = 0.0;
    const float scale = 2.f / (float)n;
    const size_t n4 = (((uintptr_t)y | (uintptr_t)t | (uintptr_t)dy) & 15) == 0 ? n / 4 : 0;
    const size_t stride = (size_t)gridDim.x * blockDim.x, t0 = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    for (size_t i = t0; i < n4; i += stride) {
        const float4 a = reinterpret_cast<const float4 *>(y)[i], b = reinterpret_cast<const float4 *>(t)[i];
        const float d0 = a.x - b.x, d1 = a.y - b.y, d2 = a.z - b.z, d3 = a.w - b.w;
        reinterpret_cast<float4 *>(dy)[i] = make_float4(scale * d0, scale * d1, scale * d2, scale * d3);
        s += (double)(d0 * d0 + d1 * d1 + d2 * d2 + d3 * d3);
    }
    for (size_t i = n4 * 4 + t0; i < n; i += stride) {
        const float d = y[i] - t[i];
        s += (double)d * d;
        dy[i] = scale * d;
    }
    __shared__ double red[kThreads];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int w = kThreads / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) partials[blockIdx.x] = red[0];
}

// One warp: lane l sums p[l], p[l + 32], ..., then the lanes combine in a
// fixed shuffle order (lane 0's total is the result).
__global__ void k_sum_double(const double *p, int n, double denom, float *out) {
    double s = 0.0;
    for (int i = threadIdx.x; i < n; i += 32) s += p[i];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (threadIdx.x == 0) *out = (float)(s / denom);
}

// g = grad of a ReLU output times (activation > 0), FP32 and a BF16 copy.
__global__ void k_relu_bwd(const float *__restrict__ grad, const __nv_bfloat16 *__restrict__ act, size_t n,
                           float *__restrict__ g, __nv_bfloat16 *__restrict__ gb) {
    // Eight values per thread (16-byte accesses) when every buffer is
    // 16-byte aligned, grid-stride, scalar tail.
    const size_t n8 = (((uintptr_t)grad | (uintptr_t)act | (uintptr_t)g | (uintptr_t)gb) & 15) == 0 ? n / 8 : 0;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    for (size_t i = t; i < n8; i += stride) {
        const float4 g0 = reinterpret_cast<const float4 *>(grad)[2 * i], g1 = reinterpret_cast<const float4 *>(grad)[2 * i + 1];
        const uint4 a = reinterpret_cast<const uint4 *>(act)[i];
        const float gv[8] = {g0.x, g0.y, g0.z, g0.w, g1.x, g1.y, g1.z, g1.w};
        const uint32_t aw[4] = {a.x, a.y, a.z, a.w};
        float o[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const uint16_t bits = (uint16_t)(aw[j / 2] >> (16 * (j & 1)));
            o[j] = __bfloat162float(__ushort_as_bfloat16(bits)) > 0.f ? gv[j] : 0.f;
        }
        reinterpret_cast<float4 *>(g)[2 * i] = make_float4(o[0], o[1], o[2], o[3]);
        reinterpret_cast<float4 *>(g)[2 * i + 1] = make_float4(o[4], o[5], o[6], o[7]);
        reinterpret_cast<uint4 *>(gb)[i] = make_uint4(pack_bf16(__float2bfloat16_rn(o[0]), __float2bfloat16_rn(o[1])),
                                                      pack_bf16(__float2bfloat16_rn(o[2]), __float2bfloat16_rn(o[3])),
                                                      pack_bf16(__float2bfloat16_rn(o[4]), __float2bfloat16_rn(o[5])),
                                                      pack_bf16(__float2bfloat16_rn(o[6]), __float2bfloat16_rn(o[7])));
    }
    for (size_t i = n8 * 8 + t; i < n; i += stride) {
        const float v = __bfloat162float(act[i]) > 0.f ? grad[i] : 0.f;
        g[i] = v;
        gb[i] = __float2bfloat16_rn(v);
    }
}

// Adam (bias-corrected) on FP32 master weights, refreshing the BF16 copy.
__global__ void k_adam(float *__restrict__ p, const float *__restrict__ g, float *__restrict__ m, float *__restrict__ v,
                       int n, float lr, float b1, float b2, float eps, float c1, float c2,
                       __nv_bfloat16 *__restrict__ pb) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float upd = lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    const float np = p[i] - upd;
    p[i] = np;
    if (pb) pb[i] = __float2bfloat16_rn(np);
}

uint64_t splitmix(uint64_t &s) {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

uint64_t fnv1a(const void *data, size_t n, uint64_t h = 1469598103934665603ull) {
    const unsigned char *p = static_cast<const unsigned char *>(data);
    for (size_t i = 0; i < n; ++i) {
        h ^= p[i];
        h *= 1099511628211ull;
    }
    return h;
}

}  // namespace

}  // namespace ginf_gpu

using namespace ginf_gpu;

// ---------------------------------------------------------------------------
// The network object.

struct ginf_warmnet {
    int device = -1;  // the device its parameters and buffers live on
    int L = 0, hidden = 0;
    int cin[4], cout[4];
    size_t woff[4], boff[4], nparams = 0;  // offsets into the flat FP32 parameter vector
    float *params = nullptr;               // FP32 master weights and biases (device)
    float *adam_m = nullptr, *adam_v = nullptr;
    float *grads = nullptr;
    __nv_bfloat16 *wbf = nullptr;  // BF16 copy of the weights (same offsets)
    int64_t step = 0;
    // activations / gradients, grown to the largest batch seen
    size_t cap_pix = 0;
    __nv_bfloat16 *a[4] = {};  // a[0] = x (L ch), a[1..3] hidden
    float *y = nullptr;        // output (L ch)
    float *gy = nullptr;       // dLoss/dy
    float *g32 = nullptr;      // FP32 gradient scratch (max channels)
    float *gtmp = nullptr;     // data gradient before the ReLU mask
    __nv_bfloat16 *gb = nullptr;
    __nv_bfloat16 *wflip = nullptr;
    float *partials = nullptr;
    size_t cap_partials = 0;
    double *loss_part = nullptr;
    float *loss_dev = nullptr;
    int *status = nullptr;  // device word: DEV_ERR_* from the convolution kernels' bounded waits
};

namespace {

ginf_status wfail(ginf_status s, const std::string &m) {
    ginf_gpu::set_last_error(m.c_str());
    return s;
}

#define GINF_WCK(call)                                                                       \
    do {                                                                                     \
        cudaError_t e_ = (call);                                                             \
        if (e_ != cudaSuccess) {                                                             \
            cudaGetLastError();                                                              \
            return wfail(GINF_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
        }                                                                                    \
    } while (0)

void layout(ginf_warmnet *n) {
    const int ch[5] = {n->L, n->hidden, n->hidden, n->hidden, n->L};
    size_t off = 0;
    for (int l = 0; l < 4; ++l) {
        n->cin[l] = ch[l];
        n->cout[l] = ch[l + 1];
        n->woff[l] = off;
        off += (size_t)n->cout[l] * 9 * n->cin[l];
        n->boff[l] = off;
        off += n->cout[l];
    }
    n->nparams = off;
}

ginf_status alloc_params(ginf_warmnet *n) {
    GINF_WCK(cudaMalloc(&n->params, n->nparams * sizeof(float)));
    GINF_WCK(cudaMalloc(&n->adam_m, n->nparams * sizeof(float)));
    GINF_WCK(cudaMalloc(&n->adam_v, n->nparams * sizeof(float)));
    GINF_WCK(cudaMalloc(&n->grads, n->nparams * sizeof(float)));
    GINF_WCK(cudaMalloc(&n->wbf, n->nparams * sizeof(__nv_bfloat16)));
    GINF_WCK(cudaMemset(n->adam_m, 0, n->nparams * sizeof(float)));
    GINF_WCK(cudaMemset(n->adam_v, 0, n->nparams * sizeof(float)));
    GINF_WCK(cudaMemset(n->grads, 0, n->nparams * sizeof(float)));
    size_t wf = 0;
    for (int l = 0; l < 4; ++l) wf = std::max(wf, (size_t)n->cout[l] * 9 * n->cin[l]);
    GINF_WCK(cudaMalloc(&n->wflip, wf * sizeof(__nv_bfloat16)));
    GINF_WCK(cudaMalloc(&n->loss_part, 1024 * sizeof(double)));
    GINF_WCK(cudaMalloc(&n->loss_dev, sizeof(float)));
    GINF_WCK(cudaMalloc(&n->status, sizeof(int)));
    GINF_WCK(cudaMemset(n->status, 0, sizeof(int)));
    return GINF_OK;
}

// After a synchronisation: a wait in a convolution kernel that ran out.
ginf_status check_status(ginf_warmnet *n) {
    int st = 0;
    GINF_WCK(cudaMemcpy(&st, n->status, sizeof(int), cudaMemcpyDeviceToHost));
    if (st == 0) return GINF_OK;
    GINF_WCK(cudaMemset(n->status, 0, sizeof(int)));
    return wfail(GINF_ERR_TIMEOUT, "warm-start convolution: a device wait ran out (status " + std::to_string(st) + ")");
}

ginf_status refresh_bf16(ginf_warmnet *n, cudaStream_t s) {
    f32_to_bf16(n->params, n->wbf, n->nparams, s);
    GINF_WCK(cudaGetLastError());
    return GINF_OK;
}

ginf_status ensure_batch(ginf_warmnet *n, size_t pix) {
    if (pix <= n->cap_pix) return GINF_OK;
    for (int l = 0; l < 4; ++l) cudaFree(n->a[l]);
    cudaFree(n->y);
    cudaFree(n->gy);
    cudaFree(n->g32);
    cudaFree(n->gtmp);
    cudaFree(n->gb);
    const size_t cmax = (size_t)std::max(n->L, n->hidden);
    GINF_WCK(cudaMalloc(&n->a[0], pix * n->L * sizeof(__nv_bfloat16)));
    for (int l = 1; l < 4; ++l) GINF_WCK(cudaMalloc(&n->a[l], pix * n->hidden * sizeof(__nv_bfloat16)));
    GINF_WCK(cudaMalloc(&n->y, pix * n->L * sizeof(float)));
    GINF_WCK(cudaMalloc(&n->gy, pix * n->L * sizeof(float)));
    GINF_WCK(cudaMalloc(&n->g32, pix * cmax * sizeof(float)));
    GINF_WCK(cudaMalloc(&n->gtmp, pix * cmax * sizeof(float)));
    GINF_WCK(cudaMalloc(&n->gb, pix * cmax * sizeof(__nv_bfloat16)));
    n->cap_pix = pix;
    // Partial sums: one per bias chunk of pixels, and one per CTA of the
    // weight gradient (up to two per SM).
    const size_t chunks = (pix + kChunk - 1) / kChunk;
    int sms = 0;
    GINF_WCK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, n->device));
    size_t need = chunks * cmax;
    for (int l = 0; l < 4; ++l) need = std::max(need, (size_t)2 * sms * n->cout[l] * 9 * n->cin[l]);
    if (need > n->cap_partials) {
        cudaFree(n->partials);
        GINF_WCK(cudaMalloc(&n->partials, need * sizeof(float)));
        n->cap_partials = need;
    }
    return GINF_OK;
}

// 3x3 convolution on the tcgen05 path for the supported (cin, cout) pairs.
cudaError_t conv_fwd(int cin, int cout, bool relu, bool out_f32, const __nv_bfloat16 *in, const __nv_bfloat16 *w,
                     const float *bias, Geo g, void *out, const float *res, int *status, cudaStream_t s) {
    return conv_fwd_tc(cin, cout, relu, out_f32, in, w, bias, g.n, g.h, g.w, out, res, status, s);
}

// Weight gradient on the tcgen05 path: per-CTA partial sums, then their sum
// in CTA order (deterministic).
cudaError_t conv_wgrad(int cin, int cout, const __nv_bfloat16 *dout, const __nv_bfloat16 *in, Geo g, float *part,
                       size_t part_cap, float *dw, int *status, cudaStream_t s) {
    const size_t nw = (size_t)cout * 9 * cin;
    const size_t cap = part_cap / nw;
    int parts = 0;
    cudaError_t e = conv_wgrad_tc(cin, cout, dout, in, g.n, g.h, g.w, part, cap > 0x7fffffff ? 0x7fffffff : (int)cap,
                                  &parts, status, s);
    if (e != cudaSuccess) return e;
    k_reduce_partials<<<nblocks(nw), kThreads, 0, s>>>(part, parts, (int)nw, dw);
    return cudaGetLastError();
}

// y = x + net(x) into y_out (the network's own buffer when null); the last
// layer reads x itself as its residual.
ginf_status forward(ginf_warmnet *n, const float *x, Geo g, int *status, cudaStream_t s, float *y_out = nullptr) {
    const size_t pix = (size_t)g.n * g.h * g.w;
    ginf_status st = ensure_batch(n, pix);
    if (st != GINF_OK) return st;
    f32_to_bf16(x, n->a[0], pix * n->L, s);
    GINF_WCK(cudaGetLastError());
    for (int l = 0; l < 3; ++l)
        GINF_WCK(conv_fwd(n->cin[l], n->cout[l], true, false, n->a[l], n->wbf + n->woff[l], n->params + n->boff[l], g,
                          n->a[l + 1], nullptr, status, s));
    GINF_WCK(conv_fwd(n->cin[3], n->cout[3], false, true, n->a[3], n->wbf + n->woff[3], n->params + n->boff[3], g,
                      y_out ? y_out : n->y, x, status, s));
    return GINF_OK;
}

// Loss and every parameter gradient (into n->grads) for one batch.
ginf_status backward(ginf_warmnet *n, const float *target, Geo g, cudaStream_t s) {
    const size_t pix = (size_t)g.n * g.h * g.w;
    const size_t ny = pix * n->L;
    int blocks = (int)std::min<size_t>(1024, nblocks(ny));
    k_mse<<<blocks, kThreads, 0, s>>>(n->y, target, ny, n->gy, n->loss_part);
    k_sum_double<<<1, 32, 0, s>>>(n->loss_part, blocks, (double)ny, n->loss_dev);
    GINF_WCK(cudaGetLastError());
    const int chunks = (int)((pix + kChunk - 1) / kChunk);
    // Layer 4 (linear output): g = dy.
    const float *gl = n->gy;
    f32_to_bf16(n->gy, n->gb, ny, s);
    GINF_WCK(cudaGetLastError());
    for (int l = 3; l >= 0; --l) {
        const int ci = n->cin[l], co = n->cout[l];
        // bias gradient
        k_bias_partials<<<chunks, 256, 0, s>>>(gl, (int)pix, co, n->partials);
        k_reduce_partials<<<nblocks(co), kThreads, 0, s>>>(n->partials, chunks, co, n->grads + n->boff[l]);
        GINF_WCK(cudaGetLastError());
        // weight gradient
        GINF_WCK(conv_wgrad(ci, co, n->gb, n->a[l], g, n->partials, n->cap_partials, n->grads + n->woff[l], n->status,
                            s));
        if (l == 0) break;
        // data gradient: conv of the (BF16) output gradient with the flipped weights
        k_flip_weights<<<nblocks((size_t)ci * 9 * co), kThreads, 0, s>>>(n->wbf + n->woff[l], ci, co, n->wflip);
        GINF_WCK(cudaGetLastError());
        GINF_WCK(conv_fwd(co, ci, false, true, n->gb, n->wflip, nullptr, g, n->gtmp, nullptr, n->status, s));
        // through the ReLU of layer l-1's output
        k_relu_bwd<<<(unsigned)std::min<size_t>(4096, std::max<size_t>(1, nblocks(pix * ci / 8))), kThreads, 0, s>>>(
            n->gtmp, n->a[l], pix * ci, n->g32, n->gb);
        GINF_WCK(cudaGetLastError());
        gl = n->g32;
    }
    return GINF_OK;
}

ginf_status check_geo(const ginf_warmnet *n, int nimg, int h, int w) {
    if (!n) return wfail(GINF_ERR_INVALID_ARGUMENT, "warmnet is NULL");
    if (nimg < 1 || h < 1 || w < 1) return wfail(GINF_ERR_INVALID_ARGUMENT, "bad batch geometry");
    int dev = 0;
    GINF_WCK(cudaGetDevice(&dev));
    if (dev != n->device)
        return wfail(GINF_ERR_INVALID_ARGUMENT, "network was created on device " + std::to_string(n->device) +
                                                    ", the calling thread's current device is " + std::to_string(dev));
    return GINF_OK;
}

const char kMagic[8] = {'G', 'I', 'N', 'F', 'W', 'N', 'E', 'T'};
constexpr uint32_t kVersion = 1;

}  // namespace

namespace ginf_gpu {
// Used by the learned HBP solve in capi.cu: forward pass on level-t inputs.
// Device waits that run out are recorded in `status` (the network's own
// word when null).
ginf_status warmnet_forward(ginf_warmnet *n, const float *x, int nimg, int h, int w, float **y_out, int *status,
                            cudaStream_t s) {
    ginf_status st = check_geo(n, nimg, h, w);
    if (st != GINF_OK) return st;
    Geo g{nimg, h, w};
    st = forward(n, x, g, status ? status : n->status, s);
    if (st != GINF_OK) return st;
    *y_out = n->y;
    return GINF_OK;
}

// The C-ABI forward: the last layer writes the caller's buffer.
ginf_status warmnet_forward_into(ginf_warmnet *n, const float *x, int nimg, int h, int w, float *out, cudaStream_t s) {
    ginf_status st = check_geo(n, nimg, h, w);
    if (st != GINF_OK) return st;
    Geo g{nimg, h, w};
    return forward(n, x, g, n->status, s, out);
}
int warmnet_labels(const ginf_warmnet *n) { return n ? n->L : 0; }
}  // namespace ginf_gpu

extern "C" {

ginf_status ginf_warmnet_create(ginf_warmnet **out, int32_t num_labels, int32_t hidden, uint64_t seed) {
    ginf_gpu::set_last_error("");
    if (!out) return wfail(GINF_ERR_INVALID_ARGUMENT, "out is NULL");
    if ((num_labels != 16 && num_labels != 32 && num_labels != 64) || hidden != 32)
        return wfail(GINF_ERR_UNSUPPORTED, "the warm-start network is compiled for L in {16, 32, 64} and 32 hidden channels");
    ginf_warmnet *n = new ginf_warmnet();
    n->L = num_labels;
    n->hidden = hidden;
    layout(n);
    ginf_status st = cudaGetDevice(&n->device) == cudaSuccess ? alloc_params(n)
                                                               : wfail(GINF_ERR_NO_DEVICE, "no current CUDA device");
    if (st != GINF_OK) {
        ginf_warmnet_destroy(n);
        return st;
    }
    // He-uniform weights (last layer scaled by 0.1), zero biases.
    std::vector<float> p(n->nparams, 0.f);
    uint64_t s = seed * 0x9E3779B97F4A7C15ull + 12345;
    for (int l = 0; l < 4; ++l) {
        const float bound = std::sqrt(6.f / (9.f * n->cin[l])) * (l == 3 ? 0.1f : 1.f);
        for (size_t i = 0; i < (size_t)n->cout[l] * 9 * n->cin[l]; ++i) {
            const double u = (double)(splitmix(s) >> 11) * (1.0 / 9007199254740992.0);
            p[n->woff[l] + i] = (float)((2.0 * u - 1.0) * bound);
        }
    }
    if (cudaMemcpy(n->params, p.data(), p.size() * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess ||
        refresh_bf16(n, nullptr) != GINF_OK || cudaDeviceSynchronize() != cudaSuccess) {
        cudaGetLastError();
        ginf_warmnet_destroy(n);
        return wfail(GINF_ERR_CUDA, "warmnet initialisation failed");
    }
    *out = n;
    return GINF_OK;
}

ginf_status ginf_warmnet_destroy(ginf_warmnet *n) {
    if (!n) return GINF_OK;
    cudaFree(n->params);
    cudaFree(n->adam_m);
    cudaFree(n->adam_v);
    cudaFree(n->grads);
    cudaFree(n->wbf);
    cudaFree(n->wflip);
    for (int l = 0; l < 4; ++l) cudaFree(n->a[l]);
    cudaFree(n->y);
    cudaFree(n->gy);
    cudaFree(n->g32);
    cudaFree(n->gtmp);
    cudaFree(n->gb);
    cudaFree(n->partials);
    cudaFree(n->loss_part);
    cudaFree(n->loss_dev);
    cudaFree(n->status);
    delete n;
    return GINF_OK;
}

ginf_status ginf_warmnet_num_params(const ginf_warmnet *n, int64_t *count) {
    if (!n || !count) return wfail(GINF_ERR_INVALID_ARGUMENT, "NULL argument");
    *count = (int64_t)n->nparams;
    return GINF_OK;
}

ginf_status ginf_warmnet_get_params(const ginf_warmnet *n, float *host) {
    if (!n || !host) return wfail(GINF_ERR_INVALID_ARGUMENT, "NULL argument");
    GINF_WCK(cudaMemcpy(host, n->params, n->nparams * sizeof(float), cudaMemcpyDeviceToHost));
    return GINF_OK;
}

ginf_status ginf_warmnet_set_params(ginf_warmnet *n, const float *host) {
    if (!n || !host) return wfail(GINF_ERR_INVALID_ARGUMENT, "NULL argument");
    GINF_WCK(cudaMemcpy(n->params, host, n->nparams * sizeof(float), cudaMemcpyHostToDevice));
    ginf_status st = refresh_bf16(n, nullptr);
    if (st != GINF_OK) return st;
    GINF_WCK(cudaDeviceSynchronize());
    return GINF_OK;
}

ginf_status ginf_warmnet_forward(ginf_warmnet *n, const float *x, int32_t nimg, int32_t h, int32_t w, float *out,
                                 void *stream) {
    ginf_gpu::set_last_error("");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    ginf_status st = warmnet_forward_into(n, x, nimg, h, w, out, s);
    if (st != GINF_OK) return st;
    GINF_WCK(cudaStreamSynchronize(s));
    return check_status(n);
}

ginf_status ginf_warmnet_gradients(ginf_warmnet *n, const float *x, const float *target, int32_t nimg, int32_t h,
                                   int32_t w, float *loss, float *grads_host, void *stream) {
    ginf_gpu::set_last_error("");
    ginf_status st = check_geo(n, nimg, h, w);
    if (st != GINF_OK) return st;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    Geo g{nimg, h, w};
    if ((st = forward(n, x, g, n->status, s)) != GINF_OK) return st;
    if ((st = backward(n, target, g, s)) != GINF_OK) return st;
    if (loss) GINF_WCK(cudaMemcpyAsync(loss, n->loss_dev, sizeof(float), cudaMemcpyDeviceToHost, s));
    if (grads_host)
        GINF_WCK(cudaMemcpyAsync(grads_host, n->grads, n->nparams * sizeof(float), cudaMemcpyDeviceToHost, s));
    GINF_WCK(cudaStreamSynchronize(s));
    return check_status(n);
}

ginf_status ginf_warmnet_train_step(ginf_warmnet *n, const float *x, const float *target, int32_t nimg, int32_t h,
                                    int32_t w, float lr, float *loss, void *stream) {
    ginf_gpu::set_last_error("");
    ginf_status st = check_geo(n, nimg, h, w);
    if (st != GINF_OK) return st;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    Geo g{nimg, h, w};
    if ((st = forward(n, x, g, n->status, s)) != GINF_OK) return st;
    if ((st = backward(n, target, g, s)) != GINF_OK) return st;
    n->step += 1;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.f - std::pow(b1, (float)n->step), c2 = 1.f - std::pow(b2, (float)n->step);
    k_adam<<<nblocks(n->nparams), kThreads, 0, s>>>(n->params, n->grads, n->adam_m, n->adam_v, (int)n->nparams, lr,
                                                    b1, b2, 1e-8f, c1, c2, n->wbf);
    GINF_WCK(cudaGetLastError());
    if (loss) GINF_WCK(cudaMemcpyAsync(loss, n->loss_dev, sizeof(float), cudaMemcpyDeviceToHost, s));
    GINF_WCK(cudaStreamSynchronize(s));
    return check_status(n);
}

// Checkpoint: magic "GINFWNET", u32 version, u32 L, u32 hidden, i64 Adam step,
// u64 parameter count, then parameters, Adam m and Adam v as FP32, then the
// FNV-1a 64 checksum of everything before it.
ginf_status ginf_warmnet_save(const ginf_warmnet *n, const char *path) {
    if (!n || !path) return wfail(GINF_ERR_INVALID_ARGUMENT, "NULL argument");
    std::vector<unsigned char> buf;
    auto put = [&](const void *p, size_t k) {
        const unsigned char *c = static_cast<const unsigned char *>(p);
        buf.insert(buf.end(), c, c + k);
    };
    const uint32_t ver = kVersion, L = (uint32_t)n->L, hid = (uint32_t)n->hidden;
    const uint64_t np = n->nparams;
    put(kMagic, 8);
    put(&ver, 4);
    put(&L, 4);
    put(&hid, 4);
    put(&n->step, 8);
    put(&np, 8);
    std::vector<float> tmp(np);
    for (float *src : {n->params, n->adam_m, n->adam_v}) {
        GINF_WCK(cudaMemcpy(tmp.data(), src, np * sizeof(float), cudaMemcpyDeviceToHost));
        put(tmp.data(), np * sizeof(float));
    }
    const uint64_t sum = fnv1a(buf.data(), buf.size());
    put(&sum, 8);
    FILE *f = std::fopen(path, "wb");
    if (!f) return wfail(GINF_ERR_INVALID_ARGUMENT, std::string("cannot write ") + path);
    const bool ok = std::fwrite(buf.data(), 1, buf.size(), f) == buf.size();
    std::fclose(f);
    if (!ok) return wfail(GINF_ERR_INVALID_ARGUMENT, std::string("short write to ") + path);
    return GINF_OK;
}

ginf_status ginf_warmnet_load(ginf_warmnet **out, const char *path) {
    ginf_gpu::set_last_error("");
    if (!out || !path) return wfail(GINF_ERR_INVALID_ARGUMENT, "NULL argument");
    FILE *f = std::fopen(path, "rb");
    if (!f) return wfail(GINF_ERR_INVALID_ARGUMENT, std::string("cannot read ") + path);
    std::vector<unsigned char> buf;
    unsigned char tmp[65536];
    size_t k;
    while ((k = std::fread(tmp, 1, sizeof(tmp), f)) > 0) buf.insert(buf.end(), tmp, tmp + k);
    std::fclose(f);
    const size_t head = 8 + 4 + 4 + 4 + 8 + 8;
    if (buf.size() < head + 8 || std::memcmp(buf.data(), kMagic, 8) != 0)
        return wfail(GINF_ERR_INVALID_ARGUMENT, "not a warm-start network file");
    uint64_t sum;
    std::memcpy(&sum, buf.data() + buf.size() - 8, 8);
    if (sum != fnv1a(buf.data(), buf.size() - 8))
        return wfail(GINF_ERR_INVALID_ARGUMENT, "warm-start network file: checksum mismatch");
    uint32_t ver, L, hid;
    int64_t step;
    uint64_t np;
    std::memcpy(&ver, buf.data() + 8, 4);
    std::memcpy(&L, buf.data() + 12, 4);
    std::memcpy(&hid, buf.data() + 16, 4);
    std::memcpy(&step, buf.data() + 20, 8);
    std::memcpy(&np, buf.data() + 28, 8);
    if (ver != kVersion) return wfail(GINF_ERR_UNSUPPORTED, "warm-start network file: unknown version");
    ginf_warmnet *n = nullptr;
    ginf_status st = ginf_warmnet_create(&n, (int32_t)L, (int32_t)hid, 0);
    if (st != GINF_OK) return st;
    if (np != n->nparams || buf.size() != head + 3 * np * sizeof(float) + 8) {
        ginf_warmnet_destroy(n);
        return wfail(GINF_ERR_INVALID_ARGUMENT, "warm-start network file: size mismatch");
    }
    const unsigned char *p = buf.data() + head;
    float *dst[3] = {n->params, n->adam_m, n->adam_v};
    for (int i = 0; i < 3; ++i) {
        if (cudaMemcpy(dst[i], p + (size_t)i * np * sizeof(float), np * sizeof(float), cudaMemcpyHostToDevice) !=
            cudaSuccess) {
            cudaGetLastError();
            ginf_warmnet_destroy(n);
            return wfail(GINF_ERR_CUDA, "warm-start network upload failed");
        }
    }
    n->step = step;
    if ((st = refresh_bf16(n, nullptr)) != GINF_OK || cudaDeviceSynchronize() != cudaSuccess) {
        ginf_warmnet_destroy(n);
        return st != GINF_OK ? st : wfail(GINF_ERR_CUDA, "warm-start network upload failed");
    }
    *out = n;
    return GINF_OK;
}

}  // extern "C"
