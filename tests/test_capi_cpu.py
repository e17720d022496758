"""The C-ABI library without a GPU: it loads, exports every symbol the public
headers declare, and rejects bad arguments before touching a device."""
import ctypes
import os
import re
import subprocess

import pytest

from conftest import ROOT


def _declared_c_functions():
    hdr = open(os.path.join(ROOT, "include", "ginf_gb300.h")).read()
    hdr = re.sub(r"/\*.*?\*/", "", hdr, flags=re.S)
    return sorted(set(re.findall(r"\b(ginf_[a-z0-9_]+)\s*\(", hdr)))


def test_every_c_abi_symbol_is_exported(built_lib):
    names = _declared_c_functions()
    assert len(names) >= 10
    lib = ctypes.CDLL(built_lib)
    out = subprocess.run(["nm", "-D", "--defined-only", built_lib], capture_output=True, text=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    for n in names:
        assert hasattr(lib, n), n
        assert n in exported, n


CXX_SIGNATURES = [
    "ginf::decodeBp<float>(ginf::Grid<float>*, int, ginf::Matrix<int>*)",
    "ginf::decodeBp<int>(ginf::Grid<int>*, int, ginf::Matrix<int>*)",
    "ginf::gpuDecodeBp<float>(ginf::Grid<float>*, int, ginf::Matrix<int>*)",
    "ginf::decodeHbp<float>(ginf::Grid<float>*, int, int, ginf::Matrix<int>*)",
    "ginf::decodeHbp<int>(ginf::Grid<int>*, int, int, ginf::Matrix<int>*)",
    "ginf::gpuDecodeHbp<int>(ginf::Grid<int>*, int, int, ginf::Matrix<int>*)",
    "ginf::decodeIcmSync<float>(ginf::Grid<float>*, ginf::Matrix<int>*, int, ginf::Matrix<int>*)",
    "ginf::decodeIcmAsync<int>(ginf::Grid<int>*, ginf::Matrix<int>*, int, ginf::Matrix<int>*)",
    "ginf::gpuDecodeIcm<float>(ginf::Grid<float>*, ginf::Matrix<int>*, int, ginf::Matrix<int>*)",
    "ginf::Grid<float>::getLabelingCost(ginf::Matrix<int>*)",
    "ginf::Grid<int>::useSmoothnessTruncLinear(int, int)",
    "ginf::Grid<float>::useSmoothnessTruncQuad(float, float)",
    "ginf::Grid<float>::setSmoothnessCost(int, int, float)",
    "ginf::Matrix<int>::Matrix(int, ...)",
    "ginf::Matrix<float>::copyFrom(ginf::Matrix<float>*)",
    "ginf::lastStatus()",
    "ginf::decodeAlphaBeta<int>(ginf::Grid<int>*, ginf::Matrix<int>*, int, ginf::Matrix<int>*)",
    "ginf::gpuDecodeAlphaBeta<int>(ginf::Grid<int>*, ginf::Matrix<int>*, int, ginf::Matrix<int>*)",
]


def test_cpp_api_symbols_are_exported(built_lib):
    out = subprocess.run(["nm", "-DC", "--defined-only", built_lib], capture_output=True, text=True).stdout
    for sig in CXX_SIGNATURES:
        assert sig in out, sig


def test_cpp_dropin_program_compiles_against_headers(built_lib, tmp_path):
    """The drop-in example builds against include/ginf and links the library."""
    exe = tmp_path / "dropin"
    r = subprocess.run(["g++", "-O2", "-std=c++17", "-I" + os.path.join(ROOT, "include"),
                        os.path.join(ROOT, "tests", "cpp", "dropin_stereo.cc"), "-o", str(exe),
                        built_lib, "-Wl,-rpath," + os.path.dirname(built_lib)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_argument_validation_without_device(built_lib):
    from gridinfcuda_gb300 import capi
    L = capi.lib()
    assert L.ginf_decode_hbp(None, None, 1, 1, None, None, None) == capi.ERR_INVALID_ARGUMENT
    assert b"NULL" in L.ginf_last_error()
    import numpy as np
    D = np.zeros((1, 4, 4), np.float32)
    V = np.zeros(1, np.float32)
    g = capi.Grid(4, 4, 1, capi.F32, capi.TRUNC_LINEAR, capi.HOST, D.ctypes.data, V.ctypes.data)
    lab = np.zeros((4, 4), np.int32)
    assert L.ginf_decode_hbp(None, ctypes.byref(g), 1, 1, lab.ctypes.data, None, None) == capi.ERR_INVALID_ARGUMENT
    g.num_labels, g.sm_model = 4, 9
    assert L.ginf_decode_hbp(None, ctypes.byref(g), 1, 1, lab.ctypes.data, None, None) == capi.ERR_INVALID_ARGUMENT
    assert b"model" in L.ginf_last_error()


def test_default_options_layout(built_lib):
    from gridinfcuda_gb300 import capi
    o = capi.options()
    assert (o.msg_rule, o.msg_store, o.decode, o.normalize, o.compute_type) == (0, 0, 0, 0, -1)
    assert ctypes.sizeof(capi.Options) == 8 * 4 + 2 * 8 + 6 * 8
    assert ctypes.sizeof(capi.Grid) == 6 * 4 + 2 * 8
    assert ctypes.sizeof(capi.Stats) == 8 * 8 + 7 * 8
    assert capi.version().startswith("gridinfcuda-gb300")


def test_option_and_entry_point_validation_without_device(built_lib):
    """Bad options and arguments of the newer entry points are rejected with
    GINF_ERR_INVALID_ARGUMENT / GINF_ERR_UNSUPPORTED before any device work."""
    import numpy as np
    from gridinfcuda_gb300 import capi
    L = capi.lib()
    D = np.zeros((8, 6, 5), np.float32)
    V = np.zeros(64, np.float32)
    lab = np.zeros((6, 5), np.int32)
    g = capi.Grid(5, 6, 8, capi.F32, capi.TRUNC_LINEAR, capi.HOST, D.ctypes.data, V.ctypes.data)

    def hbp(**opt):
        o = capi.options(**opt)
        return L.ginf_decode_hbp(None, ctypes.byref(g), 2, 3, lab.ctypes.data, ctypes.byref(o), None)

    assert hbp(tile_nodes=12) == capi.ERR_INVALID_ARGUMENT
    assert hbp(host_access=5) == capi.ERR_INVALID_ARGUMENT and b"host_access" in L.ginf_last_error()
    assert hbp(stream_ordered=1) == capi.ERR_INVALID_ARGUMENT and b"workspace" in L.ginf_last_error()
    assert hbp(store=capi.STORE_F16, compute_type=capi.F64) == capi.ERR_UNSUPPORTED
    # seeded hierarchical BP: the prediction buffer and the level range
    o = capi.options()
    assert L.ginf_decode_hbp_warm(None, ctypes.byref(g), 3, 2, 1, 0, 0, None, 1, lab.ctypes.data,
                                  ctypes.byref(o), None) == capi.ERR_INVALID_ARGUMENT
    assert L.ginf_decode_hbp_learned(None, ctypes.byref(g), 3, 2, 1, 0, -1, None, lab.ctypes.data,
                                     ctypes.byref(o), None) == capi.ERR_INVALID_ARGUMENT
    # batches: only device buffers, 2 <= L <= 64
    grids = (capi.Grid * 1)(g)
    labs = (ctypes.c_void_p * 1)(lab.ctypes.data)
    h = ctypes.c_void_p()
    assert L.ginf_batch_create(ctypes.byref(h), grids, labs, 1, 5, None) == capi.ERR_INVALID_ARGUMENT
    assert L.ginf_batch_sync(None) == capi.ERR_INVALID_ARGUMENT
    assert L.ginf_workspace_sync(None) == capi.ERR_INVALID_ARGUMENT
    # the bounded-wait self-test needs its output pointers
    assert L.ginf_selftest_bounded_waits(None, None) == capi.ERR_INVALID_ARGUMENT


MACRO_PROGRAM = r'''
#include "ginf/core.h"
#include "ginf/bp.h"
#include "ginf/icm.h"
#include "ginf/graphcut.h"
// Every macro, enum and constant the reference's public headers define
// (src/include/{utils,matrix,bp,icm,graphcut}.h), with the reference's values.
static_assert(GINF_BP_BLOCK_WIDTH == 32 && GINF_BP_BLOCK_HEIGHT == 4, "bp.h:8-9");
static_assert(GINF_ICM_BLOCK_SIZE == 16, "icm.h:8");
static_assert(GINF_MAT_MAX_NUM_DIMS == 4, "matrix.h:6");
static_assert(GINF_UNDEFINED == -1 && GINF_NUM_DIR == 4, "utils.h:4-7");
static_assert(GINF_OPP_DIR(ginf::GINF_DIR_S) == ginf::GINF_DIR_N && GINF_OPP_DIR(ginf::GINF_DIR_W) == ginf::GINF_DIR_E,
              "utils.h:10");
static_assert(GINF_IS_VALID_NODE(0, 0, 1, 1) && !GINF_IS_VALID_NODE(1, 0, 1, 1), "utils.h:13");
static_assert(GINF_MIN(3, 4) == 3 && GINF_MAX(3, 4) == 4 && GINF_ABS(-5) == 5 && GINF_SQ(-3) == 9, "utils.h:16-19");
static_assert(GINF_MAX_NUM_LABELS >= 16, "utils.h:22 (raised to 128 here)");
static_assert(ginf::GINF_SM_EXPLICIT == 0 && ginf::GINF_SM_TRUNC_QUAD == 3, "grid.h:9-14");
static_assert(GINF_GRAPHCUT_NUM_ITERS_PER_GLOBAL_RELABEL == 10 && GINF_GRAPHCUT_BLOCK_WIDTH == 32 &&
              GINF_GRAPHCUT_BLOCK_HEIGHT == 8 && GINF_GRAPHCUT_NUM_THREADS_PER_BLOCK == 256, "graphcut.h:8-11");
static_assert(ginf::GINF_DIR_SOURCE == 4 && ginf::GINF_DIR_SINK == 5, "graphcut.h:14-17");
int main() {
    int block[2] = {GINF_BP_BLOCK_WIDTH, GINF_BP_BLOCK_HEIGHT};
    int s = 0;
    for (int d = 0; d < GINF_NUM_DIR; ++d) s += ginf::dirX[d] * 10 + ginf::dirY[d];
    return (s == 0 && block[0] * block[1] == 128 && GINF_ICM_BLOCK_SIZE * GINF_ICM_BLOCK_SIZE == 256) ? 0 : 1;
}
'''


def test_reference_macros_compile_against_headers(tmp_path):
    """User code that uses the reference headers' macros (the BP / ICM block
    sizes included) compiles against include/ginf and sees the same values."""
    src = tmp_path / "macros.cc"
    src.write_text(MACRO_PROGRAM)
    exe = tmp_path / "macros"
    r = subprocess.run(["g++", "-std=c++17", "-I" + os.path.join(ROOT, "include"), str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert subprocess.run([str(exe)]).returncode == 0


def test_new_entry_points_validate_without_device(built_lib):
    """Argument errors of the alpha-beta swap, the integer stereo costs and
    the half-sweeps-per-launch option are reported before any device work."""
    import numpy as np
    from gridinfcuda_gb300 import capi
    L = capi.lib()
    D = np.zeros((4, 6, 5), np.float32)
    V = np.zeros(16, np.float32)
    lab = np.zeros((6, 5), np.int32)
    g = capi.Grid(5, 6, 4, capi.F32, capi.TRUNC_LINEAR, capi.HOST, D.ctypes.data, V.ctypes.data)
    # the swap takes int32 grids only, as the reference instantiates it
    assert L.ginf_decode_alpha_beta(None, ctypes.byref(g), lab.ctypes.data, 1, lab.ctypes.data, None,
                                    None) == capi.ERR_UNSUPPORTED
    assert b"int" in L.ginf_last_error()
    Di, Vi = D.astype(np.int32), V.astype(np.int32)
    gi = capi.Grid(5, 6, 4, capi.I32, capi.TRUNC_LINEAR, capi.HOST, Di.ctypes.data, Vi.ctypes.data)
    assert L.ginf_decode_alpha_beta(None, ctypes.byref(gi), None, 1, lab.ctypes.data, None,
                                    None) == capi.ERR_INVALID_ARGUMENT
    assert L.ginf_decode_alpha_beta(None, ctypes.byref(gi), lab.ctypes.data, -1, lab.ctypes.data, None,
                                    None) == capi.ERR_INVALID_ARGUMENT
    img = np.zeros((6, 5), np.uint8)
    assert L.ginf_stereo_costs_u8(5, 6, 4, capi.HOST, img.ctypes.data, None, 20, Di.ctypes.data,
                                  None) == capi.ERR_INVALID_ARGUMENT
    assert L.ginf_stereo_costs_u8(0, 6, 4, capi.HOST, img.ctypes.data, img.ctypes.data, 20, Di.ctypes.data,
                                  None) == capi.ERR_INVALID_ARGUMENT
    o = capi.options(sweeps_per_launch=-2)
    assert L.ginf_decode_hbp(None, ctypes.byref(g), 1, 2, lab.ctypes.data, ctypes.byref(o),
                             None) == capi.ERR_INVALID_ARGUMENT
    assert b"sweeps_per_launch" in L.ginf_last_error()
