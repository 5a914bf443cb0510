"""merge_fusion_gb300 -- GB300 (sm_103a) depth-fusion hot path of kifi
(denniskb/merge_fusion): splat, sort, merge + TSDF update, marching cubes and
ICP as hand-written CUDA kernels behind the C ABI of include/kifi_gpu.h.

The Python modules are a thin mirror of the reference's classes over that
ABI (``kifi``), the build recipe (``build``) and a synthetic-scene
generator (``scenes``).
"""
from ._lib import KifiError, device_count  # noqa: F401
