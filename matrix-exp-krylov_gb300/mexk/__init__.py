"""mexk: GB300 (sm_103a) restarted-Arnoldi exp(t*A)*v.

The compute path is the CUDA library ``_build/libmexk.so`` reached through
its C ABI (``include/mexk.h``); this package holds the Python binding, the
build recipe, the seeded synthetic workloads and the Binary CSR writer.
"""
from ._lib import MexkError, lib  # noqa: F401
