"""GB300-native 2D-DIC engine: FFTCC seed + first-order IC-GN on sm_103a.

The compute path is libdic.so (hand-written CUDA behind the C ABI of include/dic.h);
this package is its Python face.  There is no CPU fallback.
"""
from ._lib import POI_DTYPE, DicError
from .engine import Engine, FFTCC2D, ICGN2D1, grid_queue, make_queue, process_pair_multi, split_rows

__all__ = ["POI_DTYPE", "DicError", "Engine", "FFTCC2D", "ICGN2D1", "grid_queue", "make_queue",
           "process_pair_multi", "split_rows"]
__version__ = "0.1.0"
