"""pyraft_gb300: pyraft's reconstruction hot path on NVIDIA GB300 (sm_103a).

Mirrors pyraft's public API for the slant-stack and DDA projectors, the FBP
filter step and EM/OSEM (pyraft/__init__.py:9-19), with every operator a
hand-written CUDA kernel in libraftgb.so reached through ctypes.
"""
from .raftypes import image, gpu_image
from ._native import RaftError
from .sinogram import (radon, radon_3d_stack, radon_gpu, radon_method, radon_view,
                       radon_withmesh, snapshot)
from .backprojection import backprojection, backprojection_gpu, backprojection_plan, radon_transpose
from .filters import lowpassino_fbp, ramlak
from .inversion import fbp, fbp_gpu
from .iterative import (em, em_checkpointed, em_gpu, em_plain, em_transmission_gpu, make_em,
                        osem, osem_batch)
from .phantom import random_ellipses, shepplogan, phantom_fromdesc

__version__ = "0.1.0"
