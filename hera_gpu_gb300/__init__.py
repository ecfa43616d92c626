"""GB300-native drop-in for hera_gpu's visibility simulator (``vis_gpu``), its
2-D median filter (``MedianFilter``) and its Omnical solver (``omnical``).

The compute path is libheravis.so (hand-written sm_103a CUDA behind the C ABI
of include/heravis.h), loaded through ctypes; there is no CPU fallback.
"""
name = "hera_gpu_gb300"

from .vis import vis_gpu, vis_gpu_multifreq  # noqa: E402,F401
from .median import MedianFilter  # noqa: E402,F401
from .redcal import omnical  # noqa: E402,F401
from ._native import Context, HeraVisError, default_context  # noqa: E402,F401
