"""GB300-native (sm_103a) implementation of TUCuda's 2D-filter path.

Hand-written CUDA kernels behind a C ABI (include/tucu_gb300.h), with the
reference's TU::cu filter classes mirrored in ``tucuda_gb300.filters`` for
torch CUDA tensors.  Build the library with ``__graft_entry__.build()``.
"""
from . import _lib  # noqa: F401
from ._lib import TucuError, check, load  # noqa: F401

__all__ = ["load", "check", "TucuError", "filters"]


def __getattr__(name):
    # The filter classes need torch; import them lazily so that the C-ABI
    # binding can be loaded without it.
    if name in ("filters", "FIRFilter2", "FIRGaussianConvolver2", "BoxFilter2", "GuidedFilter2"):
        import importlib
        mod = importlib.import_module(__name__ + ".filters")
        return mod if name == "filters" else getattr(mod, name)
    raise AttributeError(name)
