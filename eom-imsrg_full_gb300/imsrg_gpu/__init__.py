"""imsrg_gpu: GB300 (sm_103a) engine for the IMSRG(2) scalar commutator.

Host-side mirror of the reference operator interface over the C-ABI library
``libimsrg_gpu.so`` (declared in include/imsrg_gpu.h).  ``layout`` and
``synth`` are pure numpy and need no GPU; ``api`` loads the CUDA library on
first use and raises if it is missing.
"""
from .layout import Layout, ho_basis  # noqa: F401
