"""polysplat_gb300 -- GB300-native 3D Gaussian Splatting forward rasterizer.

Drop-in for the reference's forward path:

    import polysplat_gb300 as polysplat          # polysplat.ops.<43 ops>
    from polysplat_gb300 import Scene, Camera, Rasterizer, savePpm

The compute path is the hand-written sm_103a CUDA library ``libgsr.so``
(``csrc/``, C ABI in ``include/gsr.h``), built in-tree by
``polysplat_gb300.build``.
"""
from . import ops  # noqa: F401
from ._lib import GsrError  # noqa: F401
from .rasterizer import Camera, Rasterizer, Scene, savePpm  # noqa: F401

__version__ = "0.1.0"
