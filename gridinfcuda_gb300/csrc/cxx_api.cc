// cxx_api.cc -- the GridInfCuda C++ API (namespace ginf) on top of the C ABI.
//
// Matrix / Grid re-implement src/matrix.cc and src/grid.cc; the solver entry
// points that the reference defines in src/bp.cc, src/gpu/bp.cu, src/icm.cc
// and src/gpu/icm.cu forward to ginf_decode_hbp / ginf_decode_icm, the
// alpha-beta swap of src/graphcut.cc to ginf_decode_alpha_beta, and
// Grid::getLabelingCost(f) (src/grid.cc:102-125) to ginf_energy.  Explicit
// instantiations for float and int match the reference's.
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "ginf/bp.h"
#include "ginf/graphcut.h"
#include "ginf/icm.h"
#include "ginf_gb300.h"

namespace ginf {

// ---------------------------------------------------------------- Matrix

template <typename T>
Matrix<T>::Matrix(int numDims, ...) {
    if (numDims < 1 || numDims > GINF_MAT_MAX_NUM_DIMS) {
        std::fprintf(stderr, "ginf::Matrix: numDims must be 1..%d\n", GINF_MAT_MAX_NUM_DIMS);
        std::abort();
    }
    numDims_ = numDims;
    va_list args;
    va_start(args, numDims);
    int64_t stride = 1;
    for (int i = 0; i < GINF_MAT_MAX_NUM_DIMS; i++) {
        dimSize_[i] = i < numDims ? va_arg(args, int) : 1;
        stride *= dimSize_[i];
        stride_[i] = stride;
    }
    va_end(args);
    total_ = stride_[numDims - 1];
    data = static_cast<T *>(std::calloc((size_t)total_ ? (size_t)total_ : 1, sizeof(T)));
    if (!data) {
        std::fprintf(stderr, "ginf::Matrix: out of host memory\n");
        std::abort();
    }
}

template <typename T>
Matrix<T>::~Matrix() {
    std::free(data);
    data = nullptr;
}

template <typename T>
void Matrix<T>::copyFrom(Matrix<T> *m) {
    std::memcpy(data, m->data, sizeof(T) * (size_t)total_);
}

template <typename T>
void Matrix<T>::clear() {
    std::memset(data, 0, sizeof(T) * (size_t)total_);
}

template class Matrix<int>;
template class Matrix<float>;

// ------------------------------------------------------------------ Grid

template <typename T>
Grid<T>::Grid(int w, int h, int n) {
    dtCosts = new Matrix<T>(3, w, h, n);
    smCosts = new Matrix<T>(2, n, n);
    smModel = GINF_SM_POTTS;  // all-zero V: Potts with lambda 0
    width = w;
    height = h;
    numLabels = n;
}

template <typename T>
Grid<T>::~Grid() {
    delete dtCosts;
    delete smCosts;
}

template <typename T>
int Grid<T>::getWidth() {
    return width;
}
template <typename T>
int Grid<T>::getHeight() {
    return height;
}
template <typename T>
int Grid<T>::getNumLabels() {
    return numLabels;
}
template <typename T>
int Grid<T>::getNumNodes() {
    return width * height;
}
template <typename T>
SmoothnessFunctions Grid<T>::getSmModel() {
    return smModel;
}
template <typename T>
T Grid<T>::getDataCost(int x, int y, int fp) {
    return dtCosts->at(x, y, fp);
}
template <typename T>
void Grid<T>::setDataCost(int x, int y, int fp, T cost) {
    dtCosts->get(x, y, fp) = cost;
}
template <typename T>
T Grid<T>::getSmoothnessCost(int fp, int fq) {
    return smCosts->at(fp, fq);
}
template <typename T>
void Grid<T>::setSmoothnessCost(int fp, int fq, T cost) {
    smModel = GINF_SM_EXPLICIT;
    smCosts->get(fp, fq) = cost;
}

template <typename T>
void Grid<T>::useSmoothnessPotts(T lambda) {
    smModel = GINF_SM_POTTS;
    for (int fp = 0; fp < numLabels; fp++)
        for (int fq = 0; fq < numLabels; fq++) smCosts->get(fp, fq) = lambda * (T)(fp != fq);
}

template <typename T>
void Grid<T>::useSmoothnessTruncLinear(T scale, T d) {
    smModel = GINF_SM_TRUNC_LINEAR;
    for (int fp = 0; fp < numLabels; fp++)
        for (int fq = 0; fq < numLabels; fq++) {
            const T v = scale * (T)GINF_ABS(fp - fq);
            smCosts->get(fp, fq) = GINF_MIN(v, d);
        }
}

template <typename T>
void Grid<T>::useSmoothnessTruncQuad(T scale, T d) {
    smModel = GINF_SM_TRUNC_QUAD;
    for (int fp = 0; fp < numLabels; fp++)
        for (int fq = 0; fq < numLabels; fq++) {
            const T v = scale * (T)GINF_SQ(fp - fq);
            smCosts->get(fp, fq) = GINF_MIN(v, d);
        }
}

namespace {

thread_local int t_status = GINF_OK;
thread_local char t_error[512] = "";

// One reusable device workspace per host thread.
struct ThreadWorkspace {
    ginf_workspace *ws = nullptr;
    ~ThreadWorkspace() { ginf_workspace_destroy(ws); }
    ginf_workspace *get() {
        if (!ws) ginf_workspace_create(&ws);
        return ws;
    }
};
thread_local ThreadWorkspace t_ws;

template <typename T>
int cost_type();
template <>
int cost_type<float>() {
    return GINF_F32;
}
template <>
int cost_type<int>() {
    return GINF_I32;
}

template <typename T>
ginf_grid to_c(Grid<T> *g) {
    ginf_grid c;
    c.width = g->getWidth();
    c.height = g->getHeight();
    c.num_labels = g->getNumLabels();
    c.cost_type = cost_type<T>();
    c.sm_model = (int)g->getSmModel();
    c.memory = GINF_HOST;
    c.data_costs = g->getDataCosts()->data;
    c.sm_costs = g->getSmCosts()->data;
    return c;
}

bool report(ginf_status s, const char *what) {
    t_status = s;
    if (s == GINF_OK) {
        t_error[0] = '\0';
        return true;
    }
    std::snprintf(t_error, sizeof(t_error), "%s: %s", what, ginf_last_error());
    std::fprintf(stderr, "ginf: %s\n", t_error);
    return false;
}

bool check_labels(Matrix<int> *m, int64_t n, const char *what) {
    if (!m || m->getTotalSize() < n) {
        t_status = GINF_ERR_INVALID_ARGUMENT;
        std::snprintf(t_error, sizeof(t_error), "%s: label matrix missing or smaller than the grid", what);
        std::fprintf(stderr, "ginf: %s\n", t_error);
        return false;
    }
    return true;
}

}  // namespace

int lastStatus() { return t_status; }
const char *lastError() { return t_error; }

template <typename T>
T Grid<T>::getLabelingCost(Matrix<int> *f) {
    if (!check_labels(f, (int64_t)width * height, "getLabelingCost")) return T(0);
    ginf_grid c = to_c(this);
    double e = 0.0;
    report(ginf_energy(t_ws.get(), &c, f->data, &e, nullptr), "getLabelingCost");
    return (T)e;
}

template <typename T>
T Grid<T>::getLabelingCost(Matrix<int> *f, int x, int y, int label) {
    T total = getDataCost(x, y, label);
    for (int d = 0; d < GINF_NUM_DIR; d++) total += getSmoothnessCost(label, f->at(x + dirX[d], y + dirY[d]));
    return total;
}

template <typename T>
Matrix<T> *Grid<T>::getDataCosts() {
    return dtCosts;
}
template <typename T>
Matrix<T> *Grid<T>::getSmCosts() {
    return smCosts;
}

template class Grid<int>;
template class Grid<float>;

// ------------------------------------------------------------- solvers

template <typename T>
void decodeHbp(Grid<T> *grid, int numLevels, int numItersPerLevel, Matrix<int> *result) {
    if (!check_labels(result, (int64_t)grid->getWidth() * grid->getHeight(), "decodeHbp")) return;
    ginf_grid c = to_c(grid);
    report(ginf_decode_hbp(t_ws.get(), &c, numLevels, numItersPerLevel, result->data, nullptr, nullptr),
           "decodeHbp");
}

template <typename T>
void gpuDecodeHbp(Grid<T> *grid, int numLevels, int numItersPerLevel, Matrix<int> *result) {
    decodeHbp(grid, numLevels, numItersPerLevel, result);
}

template <typename T>
void decodeBp(Grid<T> *grid, int numIters, Matrix<int> *result) {
    // Loopy BP is hierarchical BP with one level (bp.cc:182-187).
    decodeHbp(grid, 1, numIters, result);
}

template <typename T>
void gpuDecodeBp(Grid<T> *grid, int numIters, Matrix<int> *result) {
    decodeHbp(grid, 1, numIters, result);
}

template <typename T>
static void icm(Grid<T> *grid, Matrix<int> *initial, int numIters, Matrix<int> *result, int async, const char *what) {
    const int64_t n = (int64_t)grid->getWidth() * grid->getHeight();
    if (!check_labels(initial, n, what) || !check_labels(result, n, what)) return;
    ginf_grid c = to_c(grid);
    report(ginf_decode_icm(t_ws.get(), &c, initial->data, numIters, async, result->data, nullptr, nullptr), what);
}

template <typename T>
void decodeIcmSync(Grid<T> *grid, Matrix<int> *initial, int numIters, Matrix<int> *result) {
    icm(grid, initial, numIters, result, 0, "decodeIcmSync");
}

template <typename T>
void gpuDecodeIcm(Grid<T> *grid, Matrix<int> *initial, int numIters, Matrix<int> *results) {
    icm(grid, initial, numIters, results, 0, "gpuDecodeIcm");
}

template <typename T>
void decodeIcmAsync(Grid<T> *grid, Matrix<int> *initial, int numIters, Matrix<int> *result) {
    icm(grid, initial, numIters, result, 1, "decodeIcmAsync");
}

template <typename T>
void decodeAlphaBeta(Grid<T> *grid, Matrix<int> *initial, int numIters, Matrix<int> *result) {
    const int64_t n = (int64_t)grid->getWidth() * grid->getHeight();
    if (!check_labels(initial, n, "decodeAlphaBeta") || !check_labels(result, n, "decodeAlphaBeta")) return;
    ginf_grid c = to_c(grid);
    report(ginf_decode_alpha_beta(t_ws.get(), &c, initial->data, numIters, result->data, nullptr, nullptr),
           "decodeAlphaBeta");
}

template <typename T>
void gpuDecodeAlphaBeta(Grid<T> *grid, Matrix<int> *initial, int numIters, Matrix<int> *result) {
    decodeAlphaBeta(grid, initial, numIters, result);
}

template void decodeAlphaBeta<int>(Grid<int> *, Matrix<int> *, int, Matrix<int> *);
template void gpuDecodeAlphaBeta<int>(Grid<int> *, Matrix<int> *, int, Matrix<int> *);

template void decodeHbp<float>(Grid<float> *, int, int, Matrix<int> *);
template void decodeHbp<int>(Grid<int> *, int, int, Matrix<int> *);
template void gpuDecodeHbp<float>(Grid<float> *, int, int, Matrix<int> *);
template void gpuDecodeHbp<int>(Grid<int> *, int, int, Matrix<int> *);
template void decodeBp<float>(Grid<float> *, int, Matrix<int> *);
template void decodeBp<int>(Grid<int> *, int, Matrix<int> *);
template void gpuDecodeBp<float>(Grid<float> *, int, Matrix<int> *);
template void gpuDecodeBp<int>(Grid<int> *, int, Matrix<int> *);
template void decodeIcmSync<float>(Grid<float> *, Matrix<int> *, int, Matrix<int> *);
template void decodeIcmSync<int>(Grid<int> *, Matrix<int> *, int, Matrix<int> *);
template void gpuDecodeIcm<float>(Grid<float> *, Matrix<int> *, int, Matrix<int> *);
template void gpuDecodeIcm<int>(Grid<int> *, Matrix<int> *, int, Matrix<int> *);
template void decodeIcmAsync<float>(Grid<float> *, Matrix<int> *, int, Matrix<int> *);
template void decodeIcmAsync<int>(Grid<int> *, Matrix<int> *, int, Matrix<int> *);

}  // namespace ginf
