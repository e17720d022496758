// ginf/bp.h -- loopy and hierarchical min-sum belief propagation
// (src/include/bp.h).  All four entry points run on the GPU (sm_103a) with the
// reference CPU code's semantics (src/bp.cc): checkerboard half-sweeps over
// interior nodes, O(L) updates for Potts / truncated-linear smoothness, and
// the label of each interior node taken as the argmin of its belief at its
// last update.  Interior entries of result are written, border entries keep
// their values.  numIters counts half-sweeps (one colour each).
#ifndef GINF_GB300_BP_H
#define GINF_GB300_BP_H

#include "core.h"

// Thread-block shape of the reference's GPU BP kernels (32 x 4).  Kept so
// code written against the reference keeps compiling; this library's sweep
// kernels choose their own tiles (8, 16 or 32 same-colour nodes of a row) and
// do not read these values.
#define GINF_BP_BLOCK_WIDTH 32
#define GINF_BP_BLOCK_HEIGHT 4

namespace ginf {

template <typename T>
void decodeBp(Grid<T> *grid, int numIters, Matrix<int> *result);

template <typename T>
void gpuDecodeBp(Grid<T> *grid, int numIters, Matrix<int> *result);

template <typename T>
void decodeHbp(Grid<T> *grid, int numLevels, int numItersPerLevel, Matrix<int> *result);

template <typename T>
void gpuDecodeHbp(Grid<T> *grid, int numLevels, int numItersPerLevel, Matrix<int> *result);

}  // namespace ginf

#endif
