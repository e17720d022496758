// ginf/matrix.h -- N-dimensional (N <= 4) dense array, first index fastest,
// zero-initialised: the container of GridInfCuda's API (src/include/matrix.h).
// Element (x, y, z, w) lives at x + d0*y + d0*d1*z + d0*d1*d2*w.  Offsets are
// 64-bit here, so grids beyond 2^31 elements index correctly.
#ifndef GINF_GB300_MATRIX_H
#define GINF_GB300_MATRIX_H

#include <cstdint>

#include "utils.h"

#define GINF_MAT_MAX_NUM_DIMS 4

namespace ginf {

template <typename T>
class Matrix {
public:
    // Flat element array (public, as in the reference, for bulk copies).
    T *data;

    // Matrix(numDims, size0, size1, ...): every size an int.
    Matrix(int numDims, ...);
    ~Matrix();
    Matrix(const Matrix &) = delete;
    Matrix &operator=(const Matrix &) = delete;

    int getNumDims() const { return numDims_; }
    int getSize(int dim) const { return dimSize_[dim]; }
    int64_t getTotalSize() const { return total_; }

    T at(int x, int y, int z = 0, int w = 0) const { return data[offset(x, y, z, w)]; }
    T &get(int x, int y, int z = 0, int w = 0) { return data[offset(x, y, z, w)]; }

    // Copies every element of a matrix of the same total size.
    void copyFrom(Matrix<T> *m);
    // Sets every element to zero.
    void clear();

private:
    int64_t offset(int x, int y, int z, int w) const {
        return x + stride_[0] * y + stride_[1] * z + stride_[2] * w;
    }
    int numDims_;
    int dimSize_[GINF_MAT_MAX_NUM_DIMS];
    int64_t stride_[GINF_MAT_MAX_NUM_DIMS];
    int64_t total_;
};

}  // namespace ginf

#endif
