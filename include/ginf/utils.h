// ginf/utils.h -- conventions of the GridInfCuda API (src/include/utils.h):
// direction numbering, neighbour offsets and the small arithmetic macros that
// user code written against the reference may use.
#ifndef GINF_GB300_UTILS_H
#define GINF_GB300_UTILS_H

#define GINF_UNDEFINED -1

// Number of neighbours of a grid node.
#define GINF_NUM_DIR 4

// The direction opposite to d (S <-> N, E <-> W).
#define GINF_OPP_DIR(x) ((x) >= 2 ? (x) - 2 : (x) + 2)

// True if (x, y) lies inside a w x h grid.
#define GINF_IS_VALID_NODE(x, y, w, h) ((x) >= 0 && (y) >= 0 && (x) < (w) && (y) < (h))

#define GINF_MIN(a, b) (((a) < (b)) ? (a) : (b))
#define GINF_MAX(a, b) (((a) > (b)) ? (a) : (b))
#define GINF_ABS(x) ((x) < 0 ? (-(x)) : (x))
#define GINF_SQ(x) ((x) * (x))

// Largest label count the GPU solvers accept (the reference GPU code stops at 16).
#define GINF_MAX_NUM_LABELS 128

namespace ginf {
// Direction numbering: S is +y, E is +x, N is -y, W is -x.
enum Directions { GINF_DIR_S, GINF_DIR_E, GINF_DIR_N, GINF_DIR_W };

const int dirX[] = {0, 1, 0, -1};
const int dirY[] = {1, 0, -1, 0};
}  // namespace ginf

#endif
