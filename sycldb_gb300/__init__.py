"""sycldb_gb300: GB300 (sm_103a) operator kernels and host executor for the
SYCLDB star-schema operator path.

The compute path is the native library ``_build/libsycldb_gb300.so`` (CUDA
kernels + C++ executor behind the C ABI in ``include/sycldb_gpu.h``); this
package only binds it.  Build it with ``python -m sycldb_gb300.build``.
"""
from . import capi  # noqa: F401

__all__ = ["capi", "engine", "plans", "ssb", "build"]
