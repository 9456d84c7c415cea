"""stonewall -- GB300-native (sm_103a) D3Q19 wall-wind solver.

A drop-in for the Warp kernels of Cat-yejun/jeju-stonewall-lbm
(stonewall3d/lbm3d.py): geometry mask in, checkpoints and drag /
overturning-moment series out.  The compute runs in libstonewall.so
(hand-written CUDA, C ABI in include/stonewall.h); this package is the host
side.  There is no CPU fallback.
"""
__version__ = "0.1.0"
