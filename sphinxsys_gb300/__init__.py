"""GB300 (sm_103a) execution policy for SPHinXsys' weakly-compressible fluid step.

The compute path is libsphx_cuda.so (C ABI in include/sphx/sphx.h), built in-tree by
``sphinxsys_gb300.build``.  ``sphinxsys_gb300.sph`` mirrors the reference call-site API
on top of that ABI; ``sphinxsys_gb300.dambreak`` is the dam-break driver.
"""
from . import cases, native  # noqa: F401

__all__ = ["cases", "native"]
