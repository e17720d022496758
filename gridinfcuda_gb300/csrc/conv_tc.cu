// conv_tc.cu -- the warm-start network's 3x3 convolutions (the forward pass,
// the data gradient as a forward convolution with flipped weights, and the
// weight gradient) on the fifth-generation tensor cores: tcgen05.mma with the
// accumulator in tensor memory, both operands read from shared memory by
// matrix descriptors, the input rows brought in by TMA tensor copies.
//
// Implicit GEMM.  A tile is M = 128 consecutive pixels of one image row,
// N = COUT output channels, K = 9 taps x CIN input channels, BF16 operands,
// FP32 accumulation.  Activations are NHWC BF16.  A CTA owns a strip of
// tiles going down one 128-pixel column band of an image, so each input row
// is loaded once (plus one halo row above and below the strip): a row
// arrives as one TMA tensor copy of 130 pixels x CIN channels (the band plus
// one pixel either side; pixels and rows outside the image read as zero,
// which is the convolution's zero padding) into a 1024-byte aligned buffer,
// swizzled by the copy (128-, 64- or 32-byte swizzle for CIN = 64, 32, 16:
// one pixel's channels per swizzle row), which is the canonical K-major
// layout the tensor cores read: 8-pixel groups SBO = 8 rows apart.  The
// swizzle is a function of the absolute shared-memory address, so the A
// operand of tap (dy, dx) is the buffer of row y + dy read from pixel dx + 1
// on, a descriptor whose start is one swizzle row further per pixel -- the
// nine taps are nine descriptors over three row buffers, nothing is copied
// per tap.
//
// The weights, [dx][8-channel chunk][j * COUT + co][8] in the canonical
// layout without swizzle, stack the three row offsets dy = j - 1 along N, so
// one MMA (N = 3 * COUT) applies an input row r to the accumulators of output
// rows r + 1, r and r - 1 at once; those live in a descending ring of
// tensor-memory slots (adjacent unless the ring wraps, when the run splits in
// two), and the first block into a fresh slot overwrites it.
//
// Roles (192 threads): warp 4 lane 0 issues the row copies into a ring of
// RING buffers; warp 5 lane 0 issues, per input row, 3 * CIN / 16 steps of
// one or two MMAs (descriptors formed once per row, compile-time step
// offsets) and commits them to mbarriers (a row buffer is free after its own
// MMAs; an output row's accumulator is full after input row r + 1); warps 0-3
// read the accumulator back (warp w owns lanes 32w..32w+31, i.e. pixels 32w..
// of the tile), add the bias, apply ReLU, stage the warp's 32 pixels in
// shared memory and store them 512 bytes per instruction, adding the
// residual in that pass.  Every wait is bounded (DEV_ERR_TIMEOUT in the
// status word), and the tensor memory is released on every path.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <atomic>
#include <mutex>

#include "ginf_internal.h"
#include "ptx.cuh"

namespace ginf_gpu {

struct ConvTcParams {
    const __nv_bfloat16 *wt;  // [COUT][9][CIN], tap = (dy + 1) * 3 + dx + 1
    const float *bias;       // COUT, or null
    const float *res;        // FP32 residual [pixel][COUT] added after the activation, or null
    void *out;               // [pixel][COUT], FP32 or BF16
    int n, h, w;             // images, rows, columns
    int bands, chunks, rows_per_chunk, items;
    int *status;
};

namespace {

constexpr int kTileM = 128;            // pixels per tile (MMA M)
constexpr int kSlab = kTileM + 2;      // pixels per row copy: the band and one either side
constexpr int kThreadsTc = 192;        // warps 0-3 epilogue, 4 copies, 5 MMA
constexpr int kCopyWarp = 4, kMmaWarp = 5;

__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
    asm volatile("mbarrier.arrive.release.cta.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}

// One box of the 4-D row map (channels, x, row, image): a row of the band.
__device__ __forceinline__ void tma_load_row(uint32_t dst, const CUtensorMap *map, int x, int row, int img,
                                             uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
        "[%6];" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(0), "r"(x), "r"(row), "r"(img), "r"(smem_addr(bar))
        : "memory");
}

// Shared-memory matrix descriptor: start address, leading byte offset
// (between core matrices adjacent in K; unused when a swizzle row holds the
// instruction's K), stride byte offset (between 8-row groups in M or N),
// version 1, swizzle mode (0 none, 2 128-byte, 4 64-byte, 6 32-byte).
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo, uint32_t swizzle = 0) {
    return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)(lbo >> 4) << 16) | ((uint64_t)(sbo >> 4) << 32) |
           (1ull << 46) | ((uint64_t)swizzle << 61);
}

// Instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both
// K-major, M = 128, N = n.
__host__ __device__ constexpr uint32_t instr_desc_bf16(int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(kTileM >> 4) << 24);
}

__device__ __forceinline__ void umma_bf16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(acc)
        : "memory");
}

// Arrives on bar once every tcgen05 operation this thread issued before is done.
__device__ __forceinline__ void umma_commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_addr(bar))
                 : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// 16 consecutive FP32 columns of this warp's 32 lanes (one lane per thread),
// waited for before returning.
__device__ __forceinline__ void tmem_load16(uint32_t taddr, float *v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15}, [%16];\n\t"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

struct Item {
    int img, x0, y0, rows;
};

// Work item: (image, 128-pixel band, chunk of rows_per_chunk rows), chunks
// of one band adjacent so that neighbouring CTAs share halo rows in L2.
__device__ __forceinline__ Item item_of(const ConvTcParams &p, int it) {
    Item r;
    const int chunk = it % p.chunks, rest = it / p.chunks;
    r.x0 = (rest % p.bands) * kTileM;
    r.img = rest / p.bands;
    r.y0 = chunk * p.rows_per_chunk;
    r.rows = min(p.rows_per_chunk, p.h - r.y0);
    return r;
}

template <int CIN, int COUT, bool OUT_F32, int RING>
struct TcLayout {
    static constexpr int kChunks = CIN / 8;
    static constexpr int kPixBytes = CIN * 2;                          // one pixel: one swizzle row
    static constexpr uint32_t kSwizzle = CIN == 64 ? 2 : (CIN == 32 ? 4 : 6);
    static constexpr int kCopyBytes = kSlab * kPixBytes;               // what one row's copy writes
    static constexpr int kRowBytes = (kCopyBytes + 1023) / 1024 * 1024;  // one row buffer, 1024-byte aligned
    static constexpr int kWBytes = 9 * CIN * COUT * 2;      // [tap][chunk][co][16 B]
    static constexpr int kRows = 0;
    static constexpr int kW = kRows + RING * kRowBytes;
    static constexpr int kBias = kW + kWBytes;
    static constexpr int kOutBytes = COUT * (OUT_F32 ? 4 : 2);  // one pixel's outputs
    static constexpr int kChunksOut = kOutBytes / 16;
    static constexpr int kStagePitch = kOutBytes + 16;
    static constexpr int kStage = (kBias + COUT * 4 + 15) / 16 * 16;  // 4 warps x 32 pixel rows
    static constexpr int kBars = kStage + 4 * 32 * kStagePitch;
    static constexpr int kAcc = COUT == 64 ? 4 : 8;  // accumulator slots in tensor memory
    static constexpr int kNumBars = 2 * RING + 2 * kAcc + 1;  // full, empty, acc_full, acc_empty, done
    static constexpr int kTmemSlot = kBars + kNumBars * 8;
    static constexpr int kAbort = kTmemSlot + 4;
    static constexpr int kBytes = kAbort + 4;
    static constexpr uint32_t kCols = kAcc * COUT;  // 128 or 256 columns: two CTAs fit an SM's 512
    static_assert((kCols & (kCols - 1)) == 0 && kCols >= 32, "tensor-memory allocation is a power of two");
};

// Tensor-memory column of output row (tile) t's accumulator: slots run
// downwards, so the accumulators of rows r + 1, r, r - 1 -- the three an
// input row r feeds -- are adjacent and ascending unless the ring wraps.
template <int COUT, int ACC>
__device__ __forceinline__ uint32_t acc_col(uint32_t t) {
    return (uint32_t)(ACC - 1 - (int)(t % ACC)) * COUT;
}

template <int CIN, int COUT, bool RELU, bool OUT_F32, int RING>
__global__ void __launch_bounds__(kThreadsTc, 2)
    k_conv_tc(const __grid_constant__ CUtensorMap rows_map, const ConvTcParams p) {
    using Lay = TcLayout<CIN, COUT, OUT_F32, RING>;
    static_assert((CIN == 16 || CIN == 32 || CIN == 64) && COUT % 16 == 0 && COUT <= 256, "tile shape");
    extern __shared__ __align__(1024) unsigned char sm[];
    uint64_t *bars = reinterpret_cast<uint64_t *>(sm + Lay::kBars);
    uint64_t *full = bars, *empty = bars + RING, *acc_full = bars + 2 * RING, *acc_empty = acc_full + Lay::kAcc,
             *done = acc_empty + Lay::kAcc;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(sm + Lay::kTmemSlot);
    volatile int *abort_flag = reinterpret_cast<volatile int *>(sm + Lay::kAbort);
    float *bias = reinterpret_cast<float *>(sm + Lay::kBias);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    unsigned char *stage = sm + Lay::kStage + (warp & 3) * 32 * Lay::kStagePitch;

    // Weights into [dx][chunk][j * COUT + co][8 channels]: for one column
    // offset dx the three row offsets dy = j - 1 stacked along N, so one MMA
    // applies all three to an input row.  The bias (zero without one).
    for (int e = threadIdx.x; e < 9 * Lay::kChunks * COUT; e += blockDim.x) {
        const int n = e % (3 * COUT), t = e / (3 * COUT), c8 = t % Lay::kChunks, dx = t / Lay::kChunks;
        const int j = n / COUT, co = n % COUT;
        *reinterpret_cast<uint4 *>(sm + Lay::kW + (size_t)e * 16) =
            *reinterpret_cast<const uint4 *>(p.wt + ((size_t)co * 9 + j * 3 + dx) * CIN + c8 * 8);
    }
    for (int c = threadIdx.x; c < COUT; c += blockDim.x) bias[c] = p.bias ? p.bias[c] : 0.f;
    if (threadIdx.x == 0) {
        for (int i = 0; i < RING; ++i) {
            mbar_init(&full[i], 1);
            mbar_init(&empty[i], 1);
        }
        for (int i = 0; i < Lay::kAcc; ++i) {
            mbar_init(&acc_full[i], 1);
            mbar_init(&acc_empty[i], 4 * 32);
        }
        mbar_init(done, 1);
        *abort_flag = 0;
        fence_barrier_init();
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(tmem_slot)),
                     "r"(Lay::kCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    fence_proxy_async_shared();  // the weights, written by threads, are read by the tensor cores
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    if (smem_addr(sm) & 1023u) {  // swizzled row buffers start on 1024-byte boundaries
        if (threadIdx.x == 0 && p.status) atomicOr(p.status, DEV_ERR_BOUNDS);
        *abort_flag = 1;
    }
    __syncthreads();

    if (warp == kCopyWarp) {
        if (lane == 0) {
            uint32_t ld = 0;
            for (int it = blockIdx.x; it < p.items && !*abort_flag; it += gridDim.x) {
                const Item t = item_of(p, it);
                for (int r = t.y0 - 1; r <= t.y0 + t.rows; ++r, ++ld) {
                    const int slot = (int)(ld % RING);
                    if (!mbar_wait_bounded(&empty[slot], ((ld / RING) & 1u) ^ 1u, p.status)) {
                        *abort_flag = 1;
                        break;
                    }
                    mbar_arrive_expect_tx(&full[slot], Lay::kCopyBytes);
                    tma_load_row(smem_addr(sm + Lay::kRows + slot * Lay::kRowBytes), &rows_map, t.x0 - 1, r, t.img,
                                 &full[slot]);
                }
            }
            // Copies still in flight land before the CTA's shared memory goes.
            for (uint32_t q = ld > RING ? ld - RING : 0; q < ld; ++q)
                mbar_wait_bounded(&full[q % RING], (q / RING) & 1u, nullptr);
        }
        __syncwarp();
    } else if (warp == kMmaWarp) {
        if (lane == 0) {
            constexpr int ACC = Lay::kAcc;
            const uint32_t rbase = smem_addr(sm + Lay::kRows);
            // Weights: [dx][chunk][3 * COUT rows][16 B], K-adjacent chunks 3 * COUT * 16 bytes apart.
            const uint64_t bdesc = smem_desc(smem_addr(sm + Lay::kW), 3 * COUT * 16, 128);
            uint32_t ld = 0, tile = 0;
            bool ok = true;
            for (int it = blockIdx.x; it < p.items && ok && !*abort_flag; it += gridDim.x) {
                const Item t = item_of(p, it);
                // Input row r = y0 - 1 + i feeds output rows y = r + 1 - j
                // (dy = j - 1), j in [jlo, jhi] within the strip; output row
                // y0 + m is tile `tile + m`.
                for (int i = 0; i < t.rows + 2 && ok; ++i, ++ld) {
                    const int jlo = i - (t.rows - 1) > 0 ? i - (t.rows - 1) : 0, jhi = i < 2 ? i : 2;
                    ok = mbar_wait_bounded(&full[ld % RING], (ld / RING) & 1u, p.status);
                    // Block j = 0 starts row y0 + i's accumulator: its slot must be read out.
                    if (ok && jlo == 0) {
                        const uint32_t tn = tile + i;
                        ok = mbar_wait_bounded(&acc_empty[tn % ACC], ((tn / ACC) & 1u) ^ 1u, p.status);
                    }
                    if (!ok) break;
                    tc_fence_after();
                    // The blocks j in [jlo, jhi] as at most two runs with
                    // adjacent accumulators (the ring wraps at most once),
                    // fixed for the row; every step then issues one MMA per
                    // run, its descriptors the row's plus constant offsets.
                    int k0 = jlo;
                    while (k0 < jhi && (tile + i - k0) % ACC != 0) ++k0;
                    const int n0 = k0 - jlo + 1, n1 = jhi - k0;  // blocks in run 0, run 1
                    const uint32_t d0 = tmem + acc_col<COUT, ACC>(tile + i - jlo);
                    const uint32_t d1 = tmem + acc_col<COUT, ACC>(tile + i - k0 - 1);
                    const uint32_t i0 = instr_desc_bf16(n0 * COUT), i1 = instr_desc_bf16(n1 > 0 ? n1 * COUT : 16);
                    const uint64_t a0 = smem_desc(rbase + (ld % RING) * Lay::kRowBytes, 16, 8 * Lay::kPixBytes,
                                                  Lay::kSwizzle);
                    const uint64_t b0 = bdesc + (uint64_t)(jlo * COUT), b1 = bdesc + (uint64_t)((k0 + 1) * COUT);
#pragma unroll
                    for (int dx = 0; dx < 3; ++dx)
#pragma unroll
                        for (int ks = 0; ks < CIN / 16; ++ks) {
                            // Offsets in 16-byte units of the descriptors' address fields.
                            const uint64_t ao = (uint64_t)((dx * Lay::kPixBytes + ks * 32) >> 4);
                            const uint64_t bo = (uint64_t)((dx * Lay::kChunks + 2 * ks) * 3 * COUT);
                            if (dx == 0 && ks == 0 && jlo == 0) {
                                // Block 0 starts output row y0 + i: overwrite.
                                umma_bf16(d0, a0, b0, instr_desc_bf16(COUT), 0u);
                                if (n0 > 1)
                                    umma_bf16(d0 + COUT, a0, b0 + (uint64_t)COUT, instr_desc_bf16((n0 - 1) * COUT), 1u);
                            } else {
                                umma_bf16(d0, a0 + ao, b0 + bo, i0, 1u);
                            }
                            if (n1 > 0) umma_bf16(d1, a0 + ao, b1 + bo, i1, 1u);
                        }
                    umma_commit(&empty[ld % RING]);  // the row's only MMAs are these
                    if (jhi == 2) umma_commit(&acc_full[(tile + i - 2) % ACC]);  // row y0 + i - 2 is done
                }
                tile += t.rows;
            }
            if (!ok) *abort_flag = 1;
            umma_commit(done);
            mbar_wait_bounded(done, 0, nullptr);
        }
        __syncwarp();
    } else {
        // Epilogue: warp w reads lanes 32w..32w+31 of the accumulator.
        uint32_t tile = 0;
        const uint32_t lane_base = (uint32_t)(warp * 32) << 16;
        // The tensor-memory loads are warp-collective: every decision to stop
        // is taken by the whole warp.
        for (int it = blockIdx.x; it < p.items && !__any_sync(~0u, *abort_flag); it += gridDim.x) {
            const Item t = item_of(p, it);
            for (int j = 0; j < t.rows; ++j, ++tile) {
                const uint32_t acc = tile % Lay::kAcc;
                if (!__all_sync(~0u, mbar_wait_bounded(&acc_full[acc], (tile / Lay::kAcc) & 1u, p.status))) {
                    *abort_flag = 1;
                    break;
                }
                tc_fence_after();
                float v[COUT];
#pragma unroll
                for (int c = 0; c < COUT; c += 16)
                    tmem_load16(tmem + lane_base + acc_col<COUT, Lay::kAcc>(tile) + c, v + c);
                tc_fence_before();
                mbar_arrive(&acc_empty[acc]);
#pragma unroll
                for (int c = 0; c < COUT; ++c) {
                    v[c] += bias[c];
                    if (RELU) v[c] = fmaxf(v[c], 0.f);
                }
                // This lane's pixel into the warp's staging rows (a pitch of
                // one 16-byte chunk more than a pixel's outputs keeps eight
                // consecutive lanes on distinct banks) ...
                unsigned char *row = stage + lane * Lay::kStagePitch;
#pragma unroll
                for (int c = 0; c < Lay::kChunksOut; ++c) {
                    uint4 q;
                    if (OUT_F32) {
                        q = make_uint4(__float_as_uint(v[4 * c]), __float_as_uint(v[4 * c + 1]),
                                       __float_as_uint(v[4 * c + 2]), __float_as_uint(v[4 * c + 3]));
                    } else {
                        uint32_t w4[4];
#pragma unroll
                        for (int k = 0; k < 4; ++k)
                            w4[k] = (uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(v[8 * c + 2 * k])) |
                                    ((uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(v[8 * c + 2 * k + 1])) << 16);
                        q = make_uint4(w4[0], w4[1], w4[2], w4[3]);
                    }
                    *reinterpret_cast<uint4 *>(row + c * 16) = q;
                }
                __syncwarp();
                // ... then the warp's 32 pixels, contiguous in the output,
                // written 512 bytes per instruction (the residual read the
                // same way).
                const int x = t.x0 + warp * 32;
                const int valid = p.w - x < 32 ? p.w - x : 32;
                const size_t pix = ((size_t)t.img * p.h + t.y0 + j) * p.w + x;
                uint4 *o = reinterpret_cast<uint4 *>(static_cast<unsigned char *>(p.out) + pix * Lay::kOutBytes);
                const uint4 *rs = OUT_F32 && p.res ? reinterpret_cast<const uint4 *>(p.res + pix * COUT) : nullptr;
                const int nq = valid * Lay::kChunksOut;
                uint4 r[Lay::kChunksOut];  // all residual loads in flight before the first store
                if (OUT_F32 && rs) {
#pragma unroll
                    for (int i = 0; i < Lay::kChunksOut; ++i)
                        if (lane + 32 * i < nq) r[i] = rs[lane + 32 * i];
                }
#pragma unroll
                for (int i = 0; i < Lay::kChunksOut; ++i) {
                    const int q = lane + 32 * i;
                    if (q >= nq) break;
                    uint4 val = *reinterpret_cast<const uint4 *>(stage + (q / Lay::kChunksOut) * Lay::kStagePitch +
                                                                 (q % Lay::kChunksOut) * 16);
                    if (OUT_F32 && rs)
                        val = make_uint4(__float_as_uint(__uint_as_float(val.x) + __uint_as_float(r[i].x)),
                                         __float_as_uint(__uint_as_float(val.y) + __uint_as_float(r[i].y)),
                                         __float_as_uint(__uint_as_float(val.z) + __uint_as_float(r[i].z)),
                                         __float_as_uint(__uint_as_float(val.w) + __uint_as_float(r[i].w)));
                    o[q] = val;
                }
                __syncwarp();
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(Lay::kCols) : "memory");
    }
}

// Per device, once: the kernel's dynamic shared-memory limit and a
// preference for the largest shared-memory split (without it the driver may
// pick a split that holds one of these CTAs per SM, not two).
struct TcKernelSetup {
    SmemLimit smem;
    std::atomic<bool> carveout[kMaxDevices];
    template <typename K>
    cudaError_t ensure(K kern, int bytes) {
        cudaError_t e = smem.ensure(kern, (size_t)bytes);
        if (e != cudaSuccess) return e;
        std::atomic<bool> &c = carveout[current_device()];
        if (c.load(std::memory_order_acquire)) return cudaSuccess;
        e = cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout,
                                 (int)cudaSharedmemCarveoutMaxShared);
        if (e == cudaSuccess) c.store(true, std::memory_order_release);
        return e;
    }
};

PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f);
        cudaGetLastError();
    });
    return fn;
}

// Rows map over an NHWC BF16 tensor (channels, x, row, image), box of `box_px`
// pixels, swizzled by a pixel's bytes (C = 16, 32 or 64).
bool encode_rows_map(CUtensorMap *map, const void *base, int C, int n, int h, int w, int box_px) {
    PFN_cuTensorMapEncodeTiled_v12000 encode = tensor_map_encoder();
    if (!encode) return false;
    const cuuint64_t dims[4] = {(cuuint64_t)C, (cuuint64_t)w, (cuuint64_t)h, (cuuint64_t)n};
    const cuuint64_t strides[3] = {(cuuint64_t)C * 2, (cuuint64_t)w * C * 2, (cuuint64_t)h * w * C * 2};
    const cuuint32_t box[4] = {(cuuint32_t)C, (cuuint32_t)box_px, 1, 1};
    const cuuint32_t estr[4] = {1, 1, 1, 1};
    const CUtensorMapSwizzle swz =
        C == 64 ? CU_TENSOR_MAP_SWIZZLE_128B : (C == 32 ? CU_TENSOR_MAP_SWIZZLE_64B : CU_TENSOR_MAP_SWIZZLE_32B);
    return encode(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<void *>(base), dims, strides, box, estr,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, swz, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// CTA slots of a kernel with `smem` bytes of shared memory: two per SM at most.
cudaError_t cta_slots(int smem, int *slots) {
    int dev = 0, sms = 0, smem_sm = 0, reserved = 0;
    cudaError_t e;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
    if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
    if ((e = cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev)) != cudaSuccess)
        return e;
    if ((e = cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev)) != cudaSuccess)
        return e;
    int per_sm = smem_sm / (smem + reserved);
    per_sm = per_sm < 1 ? 1 : (per_sm > 2 ? 2 : per_sm);
    *slots = sms * per_sm;
    return cudaSuccess;
}

// Work items for `slots` CTAs: each band's rows split into chunks so that the
// items about fill the GPU once, at least four rows per chunk (two halo rows
// per chunk).  False when there is nothing to do or too much to count.
struct ItemPlan {
    int bands, rows_per_chunk, chunks, items, grid;
};

bool plan_items(int n, int h, int w, int slots, ItemPlan &pl) {
    if (n < 1 || h < 1 || w < 1 || slots < 1) return false;
    pl.bands = (w + kTileM - 1) / kTileM;
    const long long strips = (long long)n * pl.bands;
    long long rpc = (strips * h + slots - 1) / slots;
    rpc = rpc < 4 ? 4 : (rpc > h ? h : rpc);
    pl.rows_per_chunk = (int)rpc;
    pl.chunks = (h + pl.rows_per_chunk - 1) / pl.rows_per_chunk;
    const long long items = strips * pl.chunks;
    if (items > 0x7fffffffLL) return false;
    pl.items = (int)items;
    pl.grid = pl.items < slots ? pl.items : slots;
    return true;
}

template <int CIN, int COUT, bool RELU, bool OUT_F32>
cudaError_t launch_conv_tc(const __nv_bfloat16 *in, ConvTcParams p, cudaStream_t s) {
    // The deepest ring of row buffers (3 to 8) that leaves room for two CTAs
    // per SM (228 KB of shared memory, 1 KB of it reserved per CTA).
    constexpr int kBudget = 113 * 1024;
    constexpr int kFixed = TcLayout<CIN, COUT, OUT_F32, 8>::kBytes - 8 * TcLayout<CIN, COUT, OUT_F32, 8>::kRowBytes;
    constexpr int kFit = (kBudget - kFixed) / TcLayout<CIN, COUT, OUT_F32, 8>::kRowBytes;
    constexpr int RING = kFit < 3 ? 3 : (kFit > 8 ? 8 : kFit);
    using Lay = TcLayout<CIN, COUT, OUT_F32, RING>;
    // At least 80 KB, so that no more than two CTAs share an SM's 512
    // tensor-memory columns (a third would wait in its allocation).
    constexpr int kSmem = Lay::kBytes < 80 * 1024 ? 80 * 1024 : Lay::kBytes;
    auto kern = k_conv_tc<CIN, COUT, RELU, OUT_F32, RING>;
    static TcKernelSetup setup;
    cudaError_t attr_err = setup.ensure(kern, kSmem);
    if (attr_err != cudaSuccess) return attr_err;
    alignas(64) CUtensorMap map;
    if (!tensor_map_encoder()) return cudaErrorNotSupported;
    if (!encode_rows_map(&map, in, CIN, p.n, p.h, p.w, kSlab)) return cudaErrorInvalidValue;
    int slots = 0;
    cudaError_t e = cta_slots(kSmem, &slots);
    if (e != cudaSuccess) return e;
    ItemPlan pl;
    if (!plan_items(p.n, p.h, p.w, slots, pl)) return cudaErrorInvalidValue;
    p.bands = pl.bands;
    p.rows_per_chunk = pl.rows_per_chunk;
    p.chunks = pl.chunks;
    p.items = pl.items;
    kern<<<pl.grid, kThreadsTc, kSmem, s>>>(map, p);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Weight gradient: dW[co][tap][ci] = sum over pixels p of dout[p][co] *
// in[p shifted by tap][ci], a GEMM with the pixels as K.  Both operands are
// read MN-major (channels contiguous per pixel) from the same swizzled row
// buffers the forward pass uses: A = input rows, M = taps x CIN, where one
// M = 128 tile holds 128 / CIN taps of one row offset dy as MN atoms one
// pixel apart (LBO = a pixel's bytes; the taps past dx = +1 are computed and
// dropped); B = the output-gradient row [128 pixels][COUT], N = COUT.  Each
// CTA accumulates in tensor memory over all of its rows (K steps of 16
// pixels) and writes one partial sum; the caller adds the partials in a
// fixed order, so the result is deterministic.

struct WgradParams {
    float *partials;  // [CTA][COUT][9][CIN]
    int n, h, w;
    int bands, chunks, rows_per_chunk, items;
    int *status;
};

template <int CIN, int COUT, int RING>
struct WgLayout {
    static constexpr int kInPix = CIN * 2, kOutPix = COUT * 2;  // bytes per pixel = one swizzle row
    static constexpr uint32_t kSwIn = CIN == 64 ? 2 : (CIN == 32 ? 4 : 6);
    static constexpr uint32_t kSwOut = COUT == 64 ? 2 : (COUT == 32 ? 4 : 6);
    static constexpr int kInCopy = kSlab * kInPix, kInRow = (kInCopy + 1023) / 1024 * 1024;
    static constexpr int kOutCopy = kTileM * kOutPix, kOutRow = (kOutCopy + 1023) / 1024 * 1024;
    static constexpr int kTaps = 128 / CIN;                // taps per M tile
    static constexpr int kMT = (3 + kTaps - 1) / kTaps;    // M tiles per row offset
    static constexpr int kAcc = 3 * kMT;                   // accumulators of COUT columns
    static constexpr int kIn = 0;
    static constexpr int kOut = kIn + RING * kInRow;
    // Operand reads of the dropped taps run up to 8 pixels past a row
    // buffer's copy; every buffer is padded to 136 pixels or more, and 4 KB
    // of slack follow the last one.
    static constexpr int kBars = kOut + RING * kOutRow + 4096;
    static constexpr int kNumBars = 4 * RING + 1;  // in full / empty, out full / empty, done
    static constexpr int kTmemSlot = kBars + kNumBars * 8;
    static constexpr int kAbort = kTmemSlot + 4;
    static constexpr int kBytes = kAbort + 4;
    static constexpr uint32_t kCols = kAcc * COUT <= 32 ? 32 : (kAcc * COUT <= 64 ? 64 : (kAcc * COUT <= 128 ? 128 : 256));
};

// Instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both
// MN-major, M = 128, N = n.
__host__ __device__ constexpr uint32_t instr_desc_bf16_mn(int n) {
    return instr_desc_bf16(n) | (1u << 15) | (1u << 16);
}

template <int CIN, int COUT, int RING>
__global__ void __launch_bounds__(kThreadsTc, 2)
    k_conv_wgrad_tc(const __grid_constant__ CUtensorMap in_map, const __grid_constant__ CUtensorMap out_map,
                    const WgradParams p) {
    using Lay = WgLayout<CIN, COUT, RING>;
    static_assert((CIN == 16 || CIN == 32 || CIN == 64) && (COUT == 16 || COUT == 32 || COUT == 64), "shape");
    extern __shared__ __align__(1024) unsigned char sm[];
    uint64_t *bars = reinterpret_cast<uint64_t *>(sm + Lay::kBars);
    uint64_t *in_full = bars, *in_empty = bars + RING, *out_full = bars + 2 * RING, *out_empty = bars + 3 * RING,
             *done = bars + 4 * RING;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(sm + Lay::kTmemSlot);
    volatile int *abort_flag = reinterpret_cast<volatile int *>(sm + Lay::kAbort);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x == 0) {
        for (int i = 0; i < RING; ++i) {
            mbar_init(&in_full[i], 1);
            mbar_init(&in_empty[i], 1);
            mbar_init(&out_full[i], 1);
            mbar_init(&out_empty[i], 1);
        }
        mbar_init(done, 1);
        *abort_flag = 0;
        fence_barrier_init();
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(tmem_slot)),
                     "r"(Lay::kCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    if (smem_addr(sm) & 1023u) {
        if (threadIdx.x == 0 && p.status) atomicOr(p.status, DEV_ERR_BOUNDS);
        *abort_flag = 1;
    }
    __syncthreads();
    // Items as in the forward pass: a 128-pixel band of one image, a chunk of
    // its rows.
    ConvTcParams ip{};
    ip.n = p.n;
    ip.h = p.h;
    ip.w = p.w;
    ip.bands = p.bands;
    ip.chunks = p.chunks;
    ip.rows_per_chunk = p.rows_per_chunk;

    if (warp == kCopyWarp) {
        if (lane == 0) {
            uint32_t li = 0, lo = 0;  // input rows, output-gradient rows issued
            auto in_row = [&](int r, const Item &t) {
                const int slot = (int)(li % RING);
                if (!mbar_wait_bounded(&in_empty[slot], ((li / RING) & 1u) ^ 1u, p.status)) return false;
                mbar_arrive_expect_tx(&in_full[slot], Lay::kInCopy);
                tma_load_row(smem_addr(sm + Lay::kIn + slot * Lay::kInRow), &in_map, t.x0 - 1, r, t.img, &in_full[slot]);
                ++li;
                return true;
            };
            auto out_row = [&](int r, const Item &t) {
                const int slot = (int)(lo % RING);
                if (!mbar_wait_bounded(&out_empty[slot], ((lo / RING) & 1u) ^ 1u, p.status)) return false;
                mbar_arrive_expect_tx(&out_full[slot], Lay::kOutCopy);
                tma_load_row(smem_addr(sm + Lay::kOut + slot * Lay::kOutRow), &out_map, t.x0, r, t.img, &out_full[slot]);
                ++lo;
                return true;
            };
            bool ok = true;
            for (int it = blockIdx.x; it < p.items && ok && !*abort_flag; it += gridDim.x) {
                const Item t = item_of(ip, it);
                ok = in_row(t.y0 - 1, t) && in_row(t.y0, t);
                for (int j = 0; j < t.rows && ok; ++j) ok = in_row(t.y0 + j + 1, t) && out_row(t.y0 + j, t);
            }
            if (!ok) *abort_flag = 1;
            for (uint32_t q = li > RING ? li - RING : 0; q < li; ++q)
                mbar_wait_bounded(&in_full[q % RING], (q / RING) & 1u, nullptr);
            for (uint32_t q = lo > RING ? lo - RING : 0; q < lo; ++q)
                mbar_wait_bounded(&out_full[q % RING], (q / RING) & 1u, nullptr);
        }
        __syncwarp();
    } else if (warp == kMmaWarp) {
        if (lane == 0) {
            constexpr uint32_t idesc = instr_desc_bf16_mn(COUT);
            const uint32_t ibase = smem_addr(sm + Lay::kIn), obase = smem_addr(sm + Lay::kOut);
            uint32_t li = 0, lo = 0;
            bool ok = true, fresh = true;
            for (int it = blockIdx.x; it < p.items && ok && !*abort_flag; it += gridDim.x) {
                const Item t = item_of(ip, it);
                const uint32_t base = li;
                for (int j = 0; j < t.rows && ok; ++j, ++lo) {
                    // Input rows y - 1, y, y + 1 of output-gradient row y = y0 + j.
                    for (uint32_t q = j == 0 ? base : base + j + 2; q <= base + j + 2 && ok; ++q)
                        ok = mbar_wait_bounded(&in_full[q % RING], (q / RING) & 1u, p.status);
                    if (ok) ok = mbar_wait_bounded(&out_full[lo % RING], (lo / RING) & 1u, p.status);
                    if (!ok) break;
                    tc_fence_after();
                    const uint64_t b0 = smem_desc(obase + (lo % RING) * Lay::kOutRow, 16, 8 * Lay::kOutPix, Lay::kSwOut);
#pragma unroll
                    for (int dy = 0; dy < 3; ++dy) {
                        const uint64_t a0 = smem_desc(ibase + ((base + j + dy) % RING) * Lay::kInRow, Lay::kInPix,
                                                      8 * Lay::kInPix, Lay::kSwIn);
#pragma unroll
                        for (int mt = 0; mt < Lay::kMT; ++mt)
#pragma unroll
                            for (int ks = 0; ks < kTileM / 16; ++ks) {
                                // Offsets in 16-byte units: tap block mt starts
                                // mt * kTaps pixels in, K step ks 16 pixels on.
                                const uint64_t ao = (uint64_t)((mt * Lay::kTaps + 16 * ks) * Lay::kInPix >> 4);
                                const uint64_t bo = (uint64_t)(16 * ks * Lay::kOutPix >> 4);
                                umma_bf16(tmem + (dy * Lay::kMT + mt) * COUT, a0 + ao, b0 + bo, idesc,
                                          fresh && ks == 0 ? 0u : 1u);
                            }
                    }
                    fresh = false;
                    umma_commit(&out_empty[lo % RING]);
                    umma_commit(&in_empty[(base + j) % RING]);
                    if (j == t.rows - 1) {
                        umma_commit(&in_empty[(base + j + 1) % RING]);
                        umma_commit(&in_empty[(base + j + 2) % RING]);
                    }
                }
                li = base + t.rows + 2;
            }
            if (!ok) *abort_flag = 1;
            umma_commit(done);
        }
        __syncwarp();
    } else {
        // Epilogue, once: accumulator (dy, mt), lane m = 32 * warp + lane is
        // tap dx = mt * kTaps + m / CIN, channel m % CIN.
        const bool ok = __all_sync(~0u, mbar_wait_bounded(done, 0, p.status));
        if (ok && !__any_sync(~0u, *abort_flag)) {
            tc_fence_after();
            const int m = warp * 32 + lane, ci = m % CIN;
            float *part = p.partials + (size_t)blockIdx.x * COUT * 9 * CIN;
#pragma unroll 1
            for (int a = 0; a < Lay::kAcc; ++a) {
                const int dy = a / Lay::kMT, dx = (a % Lay::kMT) * Lay::kTaps + m / CIN;
                float v[COUT];
#pragma unroll
                for (int c = 0; c < COUT; c += 16)
                    tmem_load16(tmem + ((uint32_t)(warp * 32) << 16) + a * COUT + c, v + c);
                if (dx < 3) {
#pragma unroll
                    for (int co = 0; co < COUT; ++co) part[((size_t)co * 9 + dy * 3 + dx) * CIN + ci] = v[co];
                }
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(Lay::kCols) : "memory");
    }
}

template <int CIN, int COUT>
cudaError_t launch_wgrad_tc(const __nv_bfloat16 *dout, const __nv_bfloat16 *in, WgradParams p, int max_parts,
                            int *parts, cudaStream_t s) {
    constexpr int kBudget = 113 * 1024;
    constexpr int kFixed = WgLayout<CIN, COUT, 8>::kBytes - 8 * (WgLayout<CIN, COUT, 8>::kInRow + WgLayout<CIN, COUT, 8>::kOutRow);
    constexpr int kFit = (kBudget - kFixed) / (WgLayout<CIN, COUT, 8>::kInRow + WgLayout<CIN, COUT, 8>::kOutRow);
    constexpr int RING = kFit < 3 ? 3 : (kFit > 8 ? 8 : kFit);
    using Lay = WgLayout<CIN, COUT, RING>;
    constexpr int kSmem = Lay::kBytes < 80 * 1024 ? 80 * 1024 : Lay::kBytes;
    auto kern = k_conv_wgrad_tc<CIN, COUT, RING>;
    static TcKernelSetup setup;
    cudaError_t attr_err = setup.ensure(kern, kSmem);
    if (attr_err != cudaSuccess) return attr_err;
    alignas(64) CUtensorMap in_map, out_map;
    if (!encode_rows_map(&in_map, in, CIN, p.n, p.h, p.w, kSlab) ||
        !encode_rows_map(&out_map, dout, COUT, p.n, p.h, p.w, kTileM))
        return cudaErrorInvalidValue;
    int slots = 0;
    cudaError_t e = cta_slots(kSmem, &slots);
    if (e != cudaSuccess) return e;
    if (slots > max_parts) slots = max_parts;
    ItemPlan pl;
    if (!plan_items(p.n, p.h, p.w, slots, pl)) return cudaErrorInvalidValue;
    p.bands = pl.bands;
    p.rows_per_chunk = pl.rows_per_chunk;
    p.chunks = pl.chunks;
    p.items = pl.items;
    kern<<<pl.grid, kThreadsTc, kSmem, s>>>(in_map, out_map, p);
    *parts = pl.grid;
    return cudaGetLastError();
}

}  // namespace

// 3x3 convolution of NHWC BF16 input with weights [COUT][9][CIN] on the
// tcgen05 path; cudaErrorInvalidValue for a channel pair it is not built for.
cudaError_t conv_fwd_tc(int cin, int cout, bool relu, bool out_f32, const __nv_bfloat16 *in, const __nv_bfloat16 *w,
                        const float *bias, int nimg, int h, int wd, void *out, const float *res, int *status,
                        cudaStream_t s) {
    if (((uintptr_t)in | (uintptr_t)w | (uintptr_t)out | (uintptr_t)res) & 15) return cudaErrorMisalignedAddress;
    ConvTcParams p{};
    p.wt = w;
    p.bias = bias;
    p.res = res;
    p.out = out;
    p.n = nimg;
    p.h = h;
    p.w = wd;
    p.status = status;
#define GINF_TC_CASE(CI, CO)                                                                    \
    if (cin == CI && cout == CO) {                                                              \
        if (out_f32) return relu ? cudaErrorInvalidValue : launch_conv_tc<CI, CO, false, true>(in, p, s); \
        return relu ? launch_conv_tc<CI, CO, true, false>(in, p, s)                             \
                    : launch_conv_tc<CI, CO, false, false>(in, p, s);                           \
    }
    GINF_TC_CASE(16, 32)
    GINF_TC_CASE(32, 32)
    GINF_TC_CASE(64, 32)
    GINF_TC_CASE(32, 16)
    GINF_TC_CASE(32, 64)
#undef GINF_TC_CASE
    return cudaErrorInvalidValue;
}

// Weight gradient of the 3x3 convolution on the tcgen05 path: per-CTA
// partial sums [parts][COUT][9][CIN] into `partials` (room for max_parts),
// their count in *parts; cudaErrorInvalidValue for a channel pair it is not
// built for.
cudaError_t conv_wgrad_tc(int cin, int cout, const __nv_bfloat16 *dout, const __nv_bfloat16 *in, int nimg, int h,
                          int wd, float *partials, int max_parts, int *parts, int *status, cudaStream_t s) {
    if (((uintptr_t)dout | (uintptr_t)in) & 15) return cudaErrorMisalignedAddress;
    WgradParams p{};
    p.partials = partials;
    p.n = nimg;
    p.h = h;
    p.w = wd;
    p.status = status;
#define GINF_WG_TC_CASE(CI, CO) \
    if (cin == CI && cout == CO) return launch_wgrad_tc<CI, CO>(dout, in, p, max_parts, parts, s);
    GINF_WG_TC_CASE(16, 32)
    GINF_WG_TC_CASE(32, 32)
    GINF_WG_TC_CASE(64, 32)
    GINF_WG_TC_CASE(32, 16)
    GINF_WG_TC_CASE(32, 64)
#undef GINF_WG_TC_CASE
    return cudaErrorInvalidValue;
}

}  // namespace ginf_gpu
