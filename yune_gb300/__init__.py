"""yune_gb300 -- GB300 (sm_103a) path-tracing core with Yune's render-pass contract.

The product is libyune_gb300.so (C-ABI in include/yune_cuda.h and include/yune_host.h);
this package is the Python side of it: ctypes bindings (_native), numpy views of the
buffer layouts (layouts), procedural scenes and configurations (scenes) and a
RendererCore-style pass driver (core).
"""
from ._native import YuneError, lib  # noqa: F401
