// ref_bridge.cc -- extern "C" entry points into the reference's own CPU code.
//
// TEST INFRASTRUCTURE ONLY.  oracle/Makefile compiles this file together with
// the reference's unmodified src/{grid,matrix,bp,icm,graphcut}.cc (from the read-only
// reference checkout, never copied) into oracle/_ref/libginf_ref.so.  The
// tests use it to pin the C restatement (ginf_oracle.c) and to write the
// golden fixtures under tests/golden/.
//
// Inputs follow the reference's Matrix layouts: D label-planar
// (x + W*y + W*H*l), V indexed fp + L*fq, labels x + W*y.
#include <cstdint>
#include <cstring>

#include "bp.h"
#include "graphcut.h"
#include "grid.h"
#include "icm.h"
#include "matrix.h"

namespace ginf {
// Defined in src/bp.cc:7-18 and :21-63; emitted there as weak symbols by the
// float / int instantiations of decodeHbp.
template <typename T> void bpCollect(Grid<T> *, Matrix<T> *, Matrix<T> *, Matrix<T> *, int, int);
template <typename T> void bpSendMsg(Grid<T> *, Matrix<T> *, Matrix<T> *, T *, int, int, int);
}  // namespace ginf

namespace {

// Builds a reference Grid the way a user would: data costs through the public
// data pointer, smoothness through the matching useSmoothness* call
// (grid.cc:69-100) or, for model 0, setSmoothnessCost per entry (grid.cc:63).
template <typename T>
ginf::Grid<T> *make_grid(int W, int H, int L, const T *D, int model, T scale, T d, const T *V) {
    auto *g = new ginf::Grid<T>(W, H, L);
    if (D) std::memcpy(g->getDataCosts()->data, D, sizeof(T) * (size_t)W * H * L);
    switch (model) {
        case 1: g->useSmoothnessPotts(scale); break;
        case 2: g->useSmoothnessTruncLinear(scale, d); break;
        case 3: g->useSmoothnessTruncQuad(scale, d); break;
        default:
            for (int fp = 0; fp < L; fp++)
                for (int fq = 0; fq < L; fq++) g->setSmoothnessCost(fp, fq, V[fp + (size_t)L * fq]);
    }
    return g;
}

template <typename T>
int table(int L, int model, T scale, T d, const T *V, T *out) {
    ginf::Grid<T> *g = make_grid<T>(1, 1, L, nullptr, model, scale, d, V);
    std::memcpy(out, g->getSmCosts()->data, sizeof(T) * (size_t)L * L);
    delete g;
    return 0;
}

template <typename T>
int hbp(int W, int H, int L, const T *D, int model, T scale, T d, const T *V, int levels, int iters,
        int32_t *labels) {
    ginf::Grid<T> *g = make_grid<T>(W, H, L, D, model, scale, d, V);
    ginf::Matrix<int> result(2, W, H);
    std::memcpy(result.data, labels, sizeof(int) * (size_t)W * H);
    if (levels == 1) ginf::decodeBp(g, iters, &result);
    else ginf::decodeHbp(g, levels, iters, &result);
    std::memcpy(labels, result.data, sizeof(int) * (size_t)W * H);
    delete g;
    return 0;
}

// Single-level BP driven through the reference's own bpCollect / bpSendMsg,
// on the schedule of bp.cc:147-165, to read out the final messages.  They are
// returned in the receiver layout out[((y*W+x)*4+d)*L+l] = message to (x,y)
// from its neighbour in direction d (0 where that neighbour is off-grid).
template <typename T>
int bp_msgs(int W, int H, int L, const T *D, int model, T scale, T d, const T *V, int iters, T *out) {
    ginf::Grid<T> *g = make_grid<T>(W, H, L, D, model, scale, d, V);
    ginf::Matrix<T> data(3, W, H, L), from(3, W, H, L), msgs(4, W, H, 4, L);
    data.copyFrom(g->getDataCosts());
    T *buf = new T[L];
    for (int it = 0; it < iters; it++)
        for (int y = 1; y < H - 1; y++)
            for (int x = ((y + it) & 1) + 1; x < W - 1; x += 2) {
                ginf::bpCollect(g, &msgs, &from, &data, x, y);
                for (int dir = 0; dir < 4; dir++) {
                    ginf::bpSendMsg(g, &msgs, &from, buf, x, y, dir);
                    for (int j = 0; j < L; j++) msgs.get(x, y, dir, j) = buf[j];
                }
            }
    for (int y = 0; y < H; y++)
        for (int x = 0; x < W; x++)
            for (int dir = 0; dir < 4; dir++) {
                const int nx = x + ginf::dirX[dir], ny = y + ginf::dirY[dir];
                const int back = dir >= 2 ? dir - 2 : dir + 2;
                for (int l = 0; l < L; l++) {
                    T v = 0;
                    if (nx >= 0 && ny >= 0 && nx < W && ny < H) v = msgs.at(nx, ny, back, l);
                    out[(((size_t)y * W + x) * 4 + dir) * L + l] = v;
                }
            }
    delete[] buf;
    delete g;
    return 0;
}

template <typename T>
int icm(int W, int H, int L, const T *D, int model, T scale, T d, const T *V, const int32_t *initial,
        int iters, int32_t *result, bool async) {
    ginf::Grid<T> *g = make_grid<T>(W, H, L, D, model, scale, d, V);
    ginf::Matrix<int> init(2, W, H), res(2, W, H);
    std::memcpy(init.data, initial, sizeof(int) * (size_t)W * H);
    if (async) ginf::decodeIcmAsync(g, &init, iters, &res);
    else ginf::decodeIcmSync(g, &init, iters, &res);
    std::memcpy(result, res.data, sizeof(int) * (size_t)W * H);
    delete g;
    return 0;
}

template <typename T>
T energy(int W, int H, int L, const T *D, int model, T scale, T d, const T *V, const int32_t *labels) {
    ginf::Grid<T> *g = make_grid<T>(W, H, L, D, model, scale, d, V);
    ginf::Matrix<int> f(2, W, H);
    std::memcpy(f.data, labels, sizeof(int) * (size_t)W * H);
    T e = g->getLabelingCost(&f);
    delete g;
    return e;
}

// decodeAlphaBeta (src/graphcut.cc:197-279), instantiated for int only (:281).
int alpha_beta(int W, int H, int L, const int *D, int model, int scale, int d, const int *V, const int32_t *initial,
               int iters, int32_t *result) {
    ginf::Grid<int> *g = make_grid<int>(W, H, L, D, model, scale, d, V);
    ginf::Matrix<int> init(2, W, H), res(2, W, H);
    std::memcpy(init.data, initial, sizeof(int) * (size_t)W * H);
    ginf::decodeAlphaBeta(g, &init, iters, &res);
    std::memcpy(result, res.data, sizeof(int) * (size_t)W * H);
    delete g;
    return 0;
}

}  // namespace

extern "C" {

int ref_table_f32(int L, int model, float scale, float d, const float *V, float *out) {
    return table<float>(L, model, scale, d, V, out);
}
int ref_table_i32(int L, int model, int32_t scale, int32_t d, const int32_t *V, int32_t *out) {
    return table<int>(L, model, scale, d, (const int *)V, (int *)out);
}
int ref_hbp_f32(int W, int H, int L, const float *D, int model, float scale, float d, const float *V,
                int levels, int iters, int32_t *labels) {
    return hbp<float>(W, H, L, D, model, scale, d, V, levels, iters, labels);
}
int ref_hbp_i32(int W, int H, int L, const int32_t *D, int model, int32_t scale, int32_t d,
                const int32_t *V, int levels, int iters, int32_t *labels) {
    return hbp<int>(W, H, L, (const int *)D, model, scale, d, (const int *)V, levels, iters, labels);
}
int ref_bp_msgs_f32(int W, int H, int L, const float *D, int model, float scale, float d, const float *V,
                    int iters, float *out) {
    return bp_msgs<float>(W, H, L, D, model, scale, d, V, iters, out);
}
int ref_bp_msgs_i32(int W, int H, int L, const int32_t *D, int model, int32_t scale, int32_t d,
                    const int32_t *V, int iters, int32_t *out) {
    return bp_msgs<int>(W, H, L, (const int *)D, model, scale, d, (const int *)V, iters, (int *)out);
}
int ref_icm_f32(int W, int H, int L, const float *D, int model, float scale, float d, const float *V,
                const int32_t *initial, int iters, int32_t *result, int async) {
    return icm<float>(W, H, L, D, model, scale, d, V, initial, iters, result, async != 0);
}
int ref_icm_i32(int W, int H, int L, const int32_t *D, int model, int32_t scale, int32_t d,
                const int32_t *V, const int32_t *initial, int iters, int32_t *result, int async) {
    return icm<int>(W, H, L, (const int *)D, model, scale, d, (const int *)V, initial, iters, result, async != 0);
}
float ref_energy_f32(int W, int H, int L, const float *D, int model, float scale, float d, const float *V,
                     const int32_t *labels) {
    return energy<float>(W, H, L, D, model, scale, d, V, labels);
}
int32_t ref_energy_i32(int W, int H, int L, const int32_t *D, int model, int32_t scale, int32_t d,
                       const int32_t *V, const int32_t *labels) {
    return energy<int>(W, H, L, (const int *)D, model, scale, d, (const int *)V, labels);
}

int ref_alpha_beta_i32(int W, int H, int L, const int32_t *D, int model, int32_t scale, int32_t d,
                       const int32_t *V, const int32_t *initial, int iters, int32_t *result) {
    return alpha_beta(W, H, L, (const int *)D, model, scale, d, (const int *)V, initial, iters, result);
}

}  // extern "C"
