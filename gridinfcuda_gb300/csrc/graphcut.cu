// graphcut.cu -- alpha-beta swap (src/graphcut.cc:9-279, decodeAlphaBeta) on
// the GPU, with the reference's exact results.
//
// The reference solves each label pair's min cut by push-relabel in which
// every push and relabel runs in raster order and sees the effect of the ones
// before it (Gauss-Seidel): a node's push reads the excess its west and north
// neighbours just pushed into it.  Processing the grid as anti-diagonal
// wavefronts (x + y = k, k = 0, 1, ...) keeps exactly those dependencies --
// a node's raster-earlier neighbours lie on diagonal k-1, its raster-later
// ones on k+1, and no two nodes of one diagonal are neighbours -- so each
// sweep gives the raster sweep's values (two nodes of a diagonal may add
// flow into the same neighbour's excess, which is integer and commutes).
// The global relabel (breadth-first distances to the sink) and the final
// reachability (nodes that reach the sink over residual edges) are sets and
// distances that do not depend on the search order; they run as frontier
// searches.  Everything the reference carries from one label pair to the
// next -- the excess, heights and residues of nodes outside the current
// partition -- lives in device memory and is carried the same way.
//
// A pair's work is a chain of dependent sweeps (a round is one global
// relabel and ten push and relabel wavefronts of W + H - 1 diagonals each),
// so one CTA of 1024 threads runs the whole solve, every pair and iteration,
// with block barriers between diagonals (grid-wide barriers would cost
// microseconds each).  Residues are stored slot-major as the reference's
// Matrix(3, W, H, 6): four directions, the (unused) source slot, the sink.
// The solve gives up after kAlphaBetaLimitNs of device time, records
// DEV_ERR_TIMEOUT and returns (the reference would run on).
#include <cstdint>

#include "ginf_internal.h"
#include "ptx.cuh"

namespace ginf_gpu {

namespace {

constexpr int kThreadsAB = 1024;
constexpr int kSink = 5;
constexpr int kItersPerRelabel = 10;  // GINF_GRAPHCUT_NUM_ITERS_PER_GLOBAL_RELABEL, graphcut.h:8
constexpr uint64_t kAlphaBetaLimitNs = 60ull * 1000000000ull;

__device__ __forceinline__ int gdx(int d) { return d == 1 ? 1 : (d == 3 ? -1 : 0); }  // utils.h:36
__device__ __forceinline__ int gdy(int d) { return d == 0 ? 1 : (d == 2 ? -1 : 0); }  // utils.h:37
__device__ __forceinline__ int gopp(int d) { return d >= 2 ? d - 2 : d + 2; }          // utils.h:10

// Diagonals a sweep must visit, one bit each, for grids with W + H - 1 up to
// kDiagBits (larger grids visit every diagonal of the active range).
constexpr int kDiagBits = 65536;

struct Shared {
    int red[kThreadsAB / 32];
    int count;      // active nodes / queue tail
    int tail;       // next frontier's size
    int min_cost;
    int success;
    int stop;
    int kmin, kmax;  // diagonals holding active nodes
    unsigned diag[kDiagBits / 32];  // diagonals holding active nodes or receiving flow
};

__device__ __forceinline__ bool diag_visit(const Shared &sh, int k, bool bits) {
    return !bits || ((sh.diag[k >> 5] >> (k & 31)) & 1u);
}

// Active nodes (non-zero excess, height below N + 2) as the range of
// diagonals x + y that hold them: kmin > kmax when there are none.
__device__ void active_diagonals(const AlphaBetaParams &p, Shared &sh) {
    const int W = p.W;
    const size_t N = (size_t)W * p.H;
    const int32_t NP2 = (int32_t)N + 2;
    const int nd = W + p.H - 1;
    const bool bits = nd <= kDiagBits;
    if (threadIdx.x == 0) {
        sh.kmin = 0x7fffffff;
        sh.kmax = -1;
    }
    if (bits)
        for (int w = threadIdx.x; w < (nd + 31) / 32; w += blockDim.x) sh.diag[w] = 0u;
    __syncthreads();
    int lo = 0x7fffffff, hi = -1;
    // Four nodes per thread and step, their loads issued together.
    for (size_t i0 = threadIdx.x; i0 < N; i0 += 4 * (size_t)blockDim.x) {
        int32_t ev[4], hv[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const size_t i = i0 + u * (size_t)blockDim.x;
            ev[u] = i < N ? p.excess[i] : 0;
            hv[u] = i < N ? p.height[i] : NP2;
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            if (!(ev[u] && hv[u] < NP2)) continue;
            const size_t i = i0 + u * (size_t)blockDim.x;
            const int k = (int)(i % W) + (int)(i / W);
            lo = min(lo, k);
            hi = max(hi, k);
            if (bits) atomicOr(&sh.diag[k >> 5], 1u << (k & 31));
        }
    }
    if (hi >= 0) {
        atomicMin(&sh.kmin, lo);
        atomicMax(&sh.kmax, hi);
    }
    __syncthreads();
}

// Barrier 1 over the block's first `n` threads (a multiple of 32).
__device__ __forceinline__ void bar_sync_first(int n) { asm volatile("bar.sync 1, %0;" ::"r"(n) : "memory"); }

// Sum of v over the block, in int32 (wrapping, as the reference's int sums).
__device__ int block_sum(int v, Shared &sh) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __syncthreads();
    if (lane == 0) sh.red[w] = v;
    __syncthreads();
    int t = 0;
    if (threadIdx.x < 32) {
        t = threadIdx.x < (int)(blockDim.x >> 5) ? sh.red[threadIdx.x] : 0;
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
        if (threadIdx.x == 0) sh.red[0] = t;
    }
    __syncthreads();
    t = sh.red[0];
    __syncthreads();
    return t;
}

// getLabelingCost(f), src/grid.cc:102-125, in int32.
__device__ int energy_i32(const AlphaBetaParams &p, const int32_t *f, Shared &sh) {
    const int W = p.W, H = p.H, L = p.L;
    const size_t N = (size_t)W * H;
    int acc = 0;
    // Four nodes per thread and step: their labels, then their cost and
    // table entries, each group of loads issued together (the int32 sum is
    // order-independent).
    for (size_t i0 = threadIdx.x; i0 < N; i0 += 4 * (size_t)blockDim.x) {
        int fl[4], fn[4], fe[4];
        bool in[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const size_t i = i0 + u * (size_t)blockDim.x;
            const int x = i < N ? (int)(i % W) : 0, y = i < N ? (int)(i / W) : 0;
            in[u] = i < N && x >= 1 && y >= 1 && x <= W - 2 && y <= H - 2;
            fl[u] = in[u] ? f[i] : 0;
            fn[u] = in[u] ? f[i - W] : 0;
            fe[u] = in[u] ? f[i + 1] : 0;
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            if (!in[u]) continue;
            const size_t i = i0 + u * (size_t)blockDim.x;
            acc += p.D[i + N * fl[u]];
            acc += p.V[fl[u] + (size_t)L * fn[u]];
            acc += p.V[fl[u] + (size_t)L * fe[u]];
        }
    }
    return block_sum(acc, sh);
}

// Frontier search from every node with sink residue over residual edges
// q -> p (residue of q towards p non-zero): dist[] gets breadth-first
// distances (1 at the sink-adjacent nodes), 0 where unreachable.
__device__ void sink_search(const AlphaBetaParams &p, int32_t *dist, Shared &sh) {
    const int W = p.W, H = p.H;
    const size_t N = (size_t)W * H;
    const int32_t *res = p.res;
    if (threadIdx.x == 0) sh.count = 0;
    __syncthreads();
    // Four nodes per thread and step, their loads issued together (the
    // order of a frontier does not matter to the distances).
    for (size_t i0 = threadIdx.x; i0 < N; i0 += 4 * (size_t)blockDim.x) {
        int32_t rv[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const size_t i = i0 + u * (size_t)blockDim.x;
            rv[u] = i < N ? res[kSink * N + i] : 0;
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const size_t i = i0 + u * (size_t)blockDim.x;
            if (i >= N) break;
            dist[i] = rv[u] ? 1 : 0;
            if (rv[u]) p.q0[atomicAdd(&sh.count, 1)] = (int32_t)i;
        }
    }
    __syncthreads();
    int32_t *cur = p.q0, *nxt = p.q1;
    int n = sh.count;
    int level = 1;
    while (n > 0) {
        if (threadIdx.x == 0) sh.tail = 0;
        __syncthreads();
        for (int j = threadIdx.x; j < n; j += blockDim.x) {
            const int32_t v = cur[j];
            const int x = v % W, y = v / W;
            for (int d = 0; d < 4; ++d) {
                const int nx = x + gdx(d), ny = y + gdy(d);
                if (nx < 0 || ny < 0 || nx >= W || ny >= H) continue;
                const size_t q = (size_t)ny * W + nx;
                if (res[gopp(d) * N + q] && atomicCAS(&dist[q], 0, level + 1) == 0) nxt[atomicAdd(&sh.tail, 1)] = (int32_t)q;
            }
        }
        __syncthreads();
        n = sh.tail;
        int32_t *t = cur;
        cur = nxt;
        nxt = t;
        ++level;
        __syncthreads();
    }
}

__global__ void __launch_bounds__(kThreadsAB, 1) k_alpha_beta(const AlphaBetaParams p) {
    __shared__ Shared sh;
    const int W = p.W, H = p.H, L = p.L;
    const size_t N = (size_t)W * H;
    const int32_t NP2 = (int32_t)N + 2;
    int32_t *f = p.result, *nf = p.newr, *ex = p.excess, *ht = p.height, *res = p.res;
    const uint64_t t0 = global_timer_ns();
    // Threads taking part in the wavefronts: enough whole warps for the
    // longest diagonal, min(W, H) nodes.
    const int mwh = W < H ? W : H;
    const int nwave = mwh >= (int)blockDim.x ? (int)blockDim.x : (mwh + 31) / 32 * 32;
    // result and newResult start as the initial labelling (graphcut.cc:205, 215).
    for (size_t i = threadIdx.x; i < N; i += blockDim.x) nf[i] = f[i];
    const int c0 = energy_i32(p, f, sh);
    if (threadIdx.x == 0) {
        sh.min_cost = c0;
        sh.success = 1;
        sh.stop = 0;
    }
    __syncthreads();
    for (int t = 0; t < p.iters && sh.success && !sh.stop; ++t) {
        __syncthreads();
        if (threadIdx.x == 0) sh.success = 0;
        for (int alpha = 0; alpha < L && !sh.stop; ++alpha) {
            for (int beta = alpha + 1; beta < L && !sh.stop; ++beta) {
                // graphCutConstructGraph (graphcut.cc:10-45): partition nodes only.
                for (size_t i = threadIdx.x; i < N; i += blockDim.x) {
                    const int fl = f[i];
                    if (fl != alpha && fl != beta) continue;
                    const int x = (int)(i % W), y = (int)(i / W);
                    int ac = 0, bc = 0;
                    for (int d = 0; d < 4; ++d) {
                        const int nx = x + gdx(d), ny = y + gdy(d);
                        int cap = 0;
                        if (nx >= 0 && ny >= 0 && nx < W && ny < H) {
                            const int fn = f[(size_t)ny * W + nx];
                            if (fn == alpha || fn == beta) {
                                cap = p.V[alpha + (size_t)L * beta];
                            } else {
                                ac += p.V[alpha + (size_t)L * fn];
                                bc += p.V[beta + (size_t)L * fn];
                            }
                        }
                        res[d * N + i] = cap;
                    }
                    ex[i] = p.D[i + N * alpha] + ac;
                    res[kSink * N + i] = p.D[i + N * beta] + bc;
                    ht[i] = 0;
                }
                __syncthreads();
                for (;;) {
                    // graphCutCountActive (graphcut.cc:75-88).
                    int act = 0;
                    for (size_t i0 = threadIdx.x; i0 < N; i0 += 4 * (size_t)blockDim.x) {
                        int32_t ev[4], hv[4];
#pragma unroll
                        for (int u = 0; u < 4; ++u) {
                            const size_t i = i0 + u * (size_t)blockDim.x;
                            ev[u] = i < N ? ex[i] : 0;
                            hv[u] = i < N ? ht[i] : NP2;
                        }
#pragma unroll
                        for (int u = 0; u < 4; ++u) act += (ev[u] && hv[u] < NP2) ? 1 : 0;
                    }
                    act = block_sum(act, sh);
                    if (act == 0) break;
                    if (threadIdx.x == 0 && global_timer_ns() - t0 > kAlphaBetaLimitNs) {
                        atomicOr(p.status, DEV_ERR_TIMEOUT);
                        sh.stop = 1;
                    }
                    __syncthreads();
                    if (sh.stop) break;
                    // graphCutGlobalRelabel (graphcut.cc:91-140).
                    sink_search(p, p.dist, sh);
                    for (size_t i0 = threadIdx.x; i0 < N; i0 += 4 * (size_t)blockDim.x) {
                        int32_t dv[4], hv[4];
#pragma unroll
                        for (int u = 0; u < 4; ++u) {
                            const size_t i = i0 + u * (size_t)blockDim.x;
                            dv[u] = i < N ? p.dist[i] : 0;
                            hv[u] = i < N ? ht[i] : 0;
                        }
#pragma unroll
                        for (int u = 0; u < 4; ++u) {
                            const size_t i = i0 + u * (size_t)blockDim.x;
                            if (i < N) ht[i] = dv[u] != 0 ? dv[u] : (hv[u] > NP2 ? hv[u] : NP2);
                        }
                    }
                    __syncthreads();
                    const bool bits = W + H - 1 <= kDiagBits;
                    for (int r = 0; r < kItersPerRelabel; ++r) {
                        // A sweep changes only active nodes and the nodes they
                        // push into, so it visits only the diagonals that hold
                        // an active node or have received flow from the one
                        // before (the bitmap, read by every thread after the
                        // last barrier, so the skips are uniform); with no
                        // active node the rest of the ten sweeps change nothing
                        // and are left out.
                        active_diagonals(p, sh);
                        if (sh.kmin > sh.kmax) break;
                        // Pushes (graphcut.cc:143-177), raster order as wavefronts,
                        // on the warps that can hold a diagonal's nodes; the
                        // others wait at the end of the sweep.
                        if ((int)threadIdx.x < nwave)
                        for (int k = sh.kmin; k <= sh.kmax; ++k) {
                            if (!diag_visit(sh, k, bits)) continue;
                            const int xlo = k - (H - 1) > 0 ? k - (H - 1) : 0;
                            const int xhi = k < W - 1 ? k : W - 1;
                            for (int x = xlo + (int)threadIdx.x; x <= xhi; x += nwave) {
                                const int y = k - x;
                                const size_t i = (size_t)y * W + x;
                                // Everything this push reads, loaded at once: no
                                // other node touches it while this diagonal runs
                                // (neighbours lie on diagonals k - 1 and k + 1),
                                // and its own pushes change distinct slots.
                                int e = ex[i];
                                const int h = ht[i];
                                int rs = res[kSink * N + i];
                                int rd[4], hq[4];
#pragma unroll
                                for (int d = 0; d < 4; ++d) {
                                    rd[d] = res[d * N + i];
                                    const int nx = x + gdx(d), ny = y + gdy(d);
                                    hq[d] = (nx >= 0 && ny >= 0 && nx < W && ny < H) ? ht[(size_t)ny * W + nx] : 0;
                                }
                                if (!(e && h < NP2)) continue;
                                if (rs && h == 1) {
                                    const int fl = min(rs, e);
                                    e -= fl;
                                    res[kSink * N + i] = rs - fl;
                                }
#pragma unroll
                                for (int d = 0; d < 4; ++d) {
                                    // A non-zero residue only ever points at a node
                                    // inside the grid (graphcut.cc:18-33).
                                    if (!rd[d] || h != hq[d] + 1) continue;
                                    const size_t q = (size_t)(y + gdy(d)) * W + x + gdx(d);
                                    const int fl = min(rd[d], e);
                                    e -= fl;
                                    atomicAdd(&ex[q], fl);
                                    res[d * N + i] = rd[d] - fl;
                                    // Only this node writes its neighbour's slot
                                    // towards it during this diagonal.
                                    atomicAdd(&res[gopp(d) * N + q], fl);
                                    // South and east neighbours lie on the next
                                    // diagonal, which this sweep reaches later.
                                    if (d <= 1) {
                                        atomicMax(&sh.kmax, k + 1);
                                        if (bits) atomicOr(&sh.diag[(k + 1) >> 5], 1u << ((k + 1) & 31));
                                    }
                                }
                                ex[i] = e;
                            }
                            bar_sync_first(nwave);
                        }
                        __syncthreads();
                        // Relabels (graphcut.cc:180-195), raster order as
                        // wavefronts: they change only active nodes' heights and
                        // no excess, so the active diagonals bound them.
                        active_diagonals(p, sh);
                        if ((int)threadIdx.x < nwave)
                        for (int k = sh.kmin; k <= sh.kmax; ++k) {
                            if (!diag_visit(sh, k, bits)) continue;
                            const int xlo = k - (H - 1) > 0 ? k - (H - 1) : 0;
                            const int xhi = k < W - 1 ? k : W - 1;
                            for (int x = xlo + (int)threadIdx.x; x <= xhi; x += nwave) {
                                const int y = k - x;
                                const size_t i = (size_t)y * W + x;
                                // Loaded at once: the west and north neighbours'
                                // heights were relabelled on diagonal k - 1, the
                                // others are untouched until later.
                                const int e = ex[i], h = ht[i], rs = res[kSink * N + i];
                                int rd[4], hq[4];
#pragma unroll
                                for (int d = 0; d < 4; ++d) {
                                    rd[d] = res[d * N + i];
                                    const int nx = x + gdx(d), ny = y + gdy(d);
                                    hq[d] = (nx >= 0 && ny >= 0 && nx < W && ny < H) ? ht[(size_t)ny * W + nx] : 0;
                                }
                                if (!(e && h < NP2)) continue;
                                if (rs) {
                                    ht[i] = 1;
                                } else {
                                    int mh = NP2;
#pragma unroll
                                    for (int d = 0; d < 4; ++d)
                                        if (rd[d]) mh = min(mh, hq[d]);
                                    ht[i] = mh + 1;
                                }
                            }
                            bar_sync_first(nwave);
                        }
                        __syncthreads();
                    }
                }
                if (sh.stop) break;
                // Nodes that reach the sink take alpha, the rest of the
                // partition beta (graphcut.cc:253-263, 60-72).
                sink_search(p, p.dist, sh);
                for (size_t i0 = threadIdx.x; i0 < N; i0 += 4 * (size_t)blockDim.x) {
                    int fl[4], dv[4];
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        const size_t i = i0 + u * (size_t)blockDim.x;
                        fl[u] = i < N ? nf[i] : -1;
                        dv[u] = i < N ? p.dist[i] : 0;
                    }
#pragma unroll
                    for (int u = 0; u < 4; ++u)
                        if (fl[u] == alpha || fl[u] == beta) nf[i0 + u * (size_t)blockDim.x] = dv[u] != 0 ? alpha : beta;
                }
                __syncthreads();
                const int cost = energy_i32(p, nf, sh);
                const bool better = cost < sh.min_cost;
                __syncthreads();
                if (better) {
                    for (size_t i = threadIdx.x; i < N; i += blockDim.x) f[i] = nf[i];
                    if (threadIdx.x == 0) {
                        sh.min_cost = cost;
                        sh.success = 1;
                    }
                } else {
                    for (size_t i = threadIdx.x; i < N; i += blockDim.x) nf[i] = f[i];
                }
                __syncthreads();
            }
        }
        __syncthreads();
    }
}

}  // namespace

cudaError_t launch_alpha_beta(const AlphaBetaParams &p, cudaStream_t s) {
    k_alpha_beta<<<1, kThreadsAB, 0, s>>>(p);
    return cudaGetLastError();
}

}  // namespace ginf_gpu
