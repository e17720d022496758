// ginf/graphcut.h -- alpha-beta-swap graph cuts (src/include/graphcut.h), on
// the GPU.  For each pass, every label pair alpha < beta: the nodes labelled
// alpha or beta are split between the two labels by the minimum cut of the
// pair's graph (push-relabel max-flow), and the swap is kept when it lowers
// the energy; the passes stop early after one without a change.  Results are
// the reference CPU code's (src/graphcut.cc) bit for bit; int grids only, as
// the reference instantiates it.
#ifndef GINF_GB300_GRAPHCUT_H
#define GINF_GB300_GRAPHCUT_H

#include "core.h"

// The reference's push-relabel constants (graphcut.h:8-11): push and relabel
// sweeps between global relabels (this library uses the same count, which
// its results depend on), and the reference GPU code's block shape (kept for
// source compatibility, not read).
#define GINF_GRAPHCUT_NUM_ITERS_PER_GLOBAL_RELABEL 10
#define GINF_GRAPHCUT_BLOCK_WIDTH 32
#define GINF_GRAPHCUT_BLOCK_HEIGHT 8
#define GINF_GRAPHCUT_NUM_THREADS_PER_BLOCK (GINF_GRAPHCUT_BLOCK_WIDTH * GINF_GRAPHCUT_BLOCK_HEIGHT)

namespace ginf {

// Residue slots beyond the four directions.
enum TerminalDirections { GINF_DIR_SOURCE = GINF_NUM_DIR, GINF_DIR_SINK };

// result receives a copy of initial, then the swaps; numIters passes at most.
template <typename T>
void decodeAlphaBeta(Grid<T> *grid, Matrix<int> *initial, int numIters, Matrix<int> *result);

template <typename T>
void gpuDecodeAlphaBeta(Grid<T> *grid, Matrix<int> *initial, int numIters, Matrix<int> *result);

}  // namespace ginf

#endif
