"""gridinfcuda_gb300 -- GB300 (sm_103a) grid-MRF inference: loopy and
hierarchical min-sum BP, ICM and energies, behind the C ABI of
include/ginf_gb300.h and the C++ API of include/ginf/.

Python is the test / benchmark harness: :mod:`gridinfcuda_gb300.capi` binds
the C ABI with ctypes, :mod:`gridinfcuda_gb300.synth` generates the seeded
synthetic stereo problems, :func:`build` compiles the shared library in tree.
"""
from . import synth  # noqa: F401


def build(verbose: bool = False) -> str:
    """Compile libginf_gb300.so (sm_103a) in the package directory."""
    from . import _build
    return _build.build(verbose=verbose)


def lib_path() -> str:
    from . import _build
    return _build.LIB
