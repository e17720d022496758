// A program written against the GridInfCuda C++ API (the shape of
// examples/stereo/stereo.cc: Grid<int>, truncated-linear smoothness, loopy BP),
// here on a seeded synthetic stereo pair read from a raw file instead of
// OpenCV images.  It exercises the drop-in headers include/ginf/*.h.
//
//   dropin_stereo <in.raw> <out.raw>
//   in.raw : int32 W, H, L, then W*H*L int32 costs (label-planar)
//   out.raw: int32 W*H labels of gpuDecodeBp (30 iterations), then
//            W*H labels of decodeHbp (3 levels x 6), then W*H labels of
//            decodeIcmSync (2 sweeps from the BP labels), then the
//            energy of the BP labelling as int32; then, for the same costs
//            as a Grid<float> with TruncLinear(1.5, 3): decodeBp (12),
//            gpuDecodeHbp (2 levels x 5), decodeIcmAsync (2 sweeps) and
//            gpuDecodeIcm (3 sweeps) from the decodeBp labels, W*H labels
//            each, and the float energy of the decodeBp labelling; then the
//            int grid's gpuDecodeAlphaBeta (1 pass from the BP labels), W*H.
#include <cstdio>
#include <vector>

#include "ginf/bp.h"
#include "ginf/core.h"
#include "ginf/graphcut.h"
#include "ginf/icm.h"

// Reference code may size its own buffers or launches with the library's
// block-shape macros (src/include/bp.h:8-9, icm.h:8); they stay defined.
static_assert(GINF_BP_BLOCK_WIDTH * GINF_BP_BLOCK_HEIGHT == 128 && GINF_ICM_BLOCK_SIZE == 16,
              "reference block-shape macros");

int main(int argc, char **argv) {
    if (argc != 3) {
        std::fprintf(stderr, "usage: %s in.raw out.raw\n", argv[0]);
        return 2;
    }
    FILE *f = std::fopen(argv[1], "rb");
    if (!f) return 2;
    int hdr[3];
    if (std::fread(hdr, sizeof(int), 3, f) != 3) return 2;
    const int W = hdr[0], H = hdr[1], L = hdr[2];
    ginf::Grid<int> grid(W, H, L);
    std::vector<int> costs((size_t)W * H * L);
    if (std::fread(costs.data(), sizeof(int), costs.size(), f) != costs.size()) return 2;
    std::fclose(f);
    for (int k = 0; k < L; k++)
        for (int y = 0; y < H; y++)
            for (int x = 0; x < W; x++) grid.setDataCost(x, y, k, costs[(size_t)x + (size_t)W * y + (size_t)W * H * k]);
    grid.useSmoothnessTruncLinear(10, 20);

    ginf::Matrix<int> bp(2, W, H), hbp(2, W, H), icm(2, W, H);
    ginf::gpuDecodeBp(&grid, 30, &bp);
    if (ginf::lastStatus() != 0) return 1;
    ginf::decodeHbp(&grid, 3, 6, &hbp);
    if (ginf::lastStatus() != 0) return 1;
    ginf::decodeIcmSync(&grid, &bp, 2, &icm);
    if (ginf::lastStatus() != 0) return 1;
    const int energy = grid.getLabelingCost(&bp);
    if (ginf::lastStatus() != 0) return 1;

    ginf::Grid<float> fgrid(W, H, L);
    for (int k = 0; k < L; k++)
        for (int y = 0; y < H; y++)
            for (int x = 0; x < W; x++)
                fgrid.setDataCost(x, y, k, 0.25f * (float)costs[(size_t)x + (size_t)W * y + (size_t)W * H * k]);
    fgrid.useSmoothnessTruncLinear(1.5f, 3.0f);
    ginf::Matrix<int> fbp(2, W, H), fhbp(2, W, H), ficma(2, W, H), ficmg(2, W, H);
    ginf::decodeBp(&fgrid, 12, &fbp);
    if (ginf::lastStatus() != 0) return 1;
    ginf::gpuDecodeHbp(&fgrid, 2, 5, &fhbp);
    if (ginf::lastStatus() != 0) return 1;
    ginf::decodeIcmAsync(&fgrid, &fbp, 2, &ficma);
    if (ginf::lastStatus() != 0) return 1;
    ginf::gpuDecodeIcm(&fgrid, &fbp, 3, &ficmg);
    if (ginf::lastStatus() != 0) return 1;
    const float fenergy = fgrid.getLabelingCost(&fbp);
    if (ginf::lastStatus() != 0) return 1;
    ginf::Matrix<int> ab(2, W, H);
    ginf::gpuDecodeAlphaBeta(&grid, &bp, 1, &ab);
    if (ginf::lastStatus() != 0) return 1;

    FILE *o = std::fopen(argv[2], "wb");
    if (!o) return 2;
    std::fwrite(bp.data, sizeof(int), (size_t)W * H, o);
    std::fwrite(hbp.data, sizeof(int), (size_t)W * H, o);
    std::fwrite(icm.data, sizeof(int), (size_t)W * H, o);
    std::fwrite(&energy, sizeof(int), 1, o);
    std::fwrite(fbp.data, sizeof(int), (size_t)W * H, o);
    std::fwrite(fhbp.data, sizeof(int), (size_t)W * H, o);
    std::fwrite(ficma.data, sizeof(int), (size_t)W * H, o);
    std::fwrite(ficmg.data, sizeof(int), (size_t)W * H, o);
    std::fwrite(&fenergy, sizeof(float), 1, o);
    std::fwrite(ab.data, sizeof(int), (size_t)W * H, o);
    std::fclose(o);
    return 0;
}
