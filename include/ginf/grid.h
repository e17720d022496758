// ginf/grid.h -- a 4-connected grid MRF with L labels: data costs D(x, y, f)
// and a pairwise smoothness table V(fp, fq) (src/include/grid.h).
#ifndef GINF_GB300_GRID_H
#define GINF_GB300_GRID_H

#include "matrix.h"
#include "utils.h"

namespace ginf {

// Smoothness model of a grid; the O(L) message updates apply to POTTS and
// TRUNC_LINEAR (and, under the standard message rule, TRUNC_QUAD).
enum SmoothnessFunctions { GINF_SM_EXPLICIT, GINF_SM_POTTS, GINF_SM_TRUNC_LINEAR, GINF_SM_TRUNC_QUAD };

template <typename T>
class Grid {
public:
    // A w x h grid with n labels; all costs start at zero (Potts, lambda 0).
    Grid(int w, int h, int n);
    ~Grid();
    Grid(const Grid &) = delete;
    Grid &operator=(const Grid &) = delete;

    int getWidth();
    int getHeight();
    int getNumLabels();
    int getNumNodes();
    SmoothnessFunctions getSmModel();

    T getDataCost(int x, int y, int fp);
    void setDataCost(int x, int y, int fp, T cost);

    T getSmoothnessCost(int fp, int fq);
    // Sets one entry of V and switches the model to GINF_SM_EXPLICIT.
    void setSmoothnessCost(int fp, int fq, T cost);

    // V(fp, fq) = lambda * (fp != fq)
    void useSmoothnessPotts(T lambda);
    // V(fp, fq) = min(scale * |fp - fq|, d)
    void useSmoothnessTruncLinear(T scale, T d);
    // V(fp, fq) = min(scale * (fp - fq)^2, d)
    void useSmoothnessTruncQuad(T scale, T d);

    // Energy of a labelling: interior nodes' data costs plus their north and
    // east smoothness terms, summed in FP64 on the GPU and returned as T.
    T getLabelingCost(Matrix<int> *f);
    // D(x, y, label) + sum over the four neighbours of V(label, f(neighbour)).
    T getLabelingCost(Matrix<int> *f, int x, int y, int label);

    Matrix<T> *getDataCosts();
    Matrix<T> *getSmCosts();

private:
    Matrix<T> *dtCosts;  // (w, h, n), label-planar
    Matrix<T> *smCosts;  // (n, n)
    SmoothnessFunctions smModel;
    int width, height, numLabels;
};

}  // namespace ginf

#endif
