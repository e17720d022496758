// ginf/icm.h -- iterated conditional modes (src/include/icm.h), on the GPU.
// result receives a copy of initial, then each sweep moves every interior
// node to the label minimising D + sum of V to its four neighbours (lowest
// label on ties).
#ifndef GINF_GB300_ICM_H
#define GINF_GB300_ICM_H

#include "core.h"

// Thread-block side of the reference's GPU ICM kernel (16 x 16).  Kept so
// code written against the reference keeps compiling; this library's ICM
// kernels use lanes per node and do not read it.
#define GINF_ICM_BLOCK_SIZE 16

namespace ginf {

// Synchronous (Jacobi) sweeps: every node reads the previous sweep's labels.
template <typename T>
void decodeIcmSync(Grid<T> *grid, Matrix<int> *initial, int numIters, Matrix<int> *result);

template <typename T>
void gpuDecodeIcm(Grid<T> *grid, Matrix<int> *initial, int numIters, Matrix<int> *results);

// Asynchronous sweeps in raster order (each node sees its west and north
// neighbours' new labels), computed exactly as an anti-diagonal wavefront.
template <typename T>
void decodeIcmAsync(Grid<T> *grid, Matrix<int> *initial, int numIters, Matrix<int> *result);

}  // namespace ginf

#endif
