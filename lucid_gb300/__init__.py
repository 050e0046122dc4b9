"""lucid_gb300: GB300-native (sm_103a) compute rasterization pipeline of LucidRaster.

The hot path (quad setup, bin count / categorize / dispatch, exact-order raster and blend)
runs in the hand-written CUDA kernels of ``liblucid_gb300.so`` behind a C ABI
(``include/lucid_gb300.h``). This package holds the Python mirror of the reference's
``LucidRenderer`` interface, the synthetic workload generators and the build script.
"""
from . import scenes  # noqa: F401  (numpy only; importable without a GPU)

__all__ = ["scenes", "LucidRenderer", "FrameInputs", "build"]


def __getattr__(name):
    if name in ("LucidRenderer", "FrameInputs", "default_options"):
        from . import renderer
        return getattr(renderer, name)
    if name == "build":
        from .build import build
        return build
    raise AttributeError(name)
