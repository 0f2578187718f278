"""GB300 (sm_103a) bitmap SpMM: C = A·B with A an M×K 0/1 matrix stored as
packed 32-bit row bitmasks and B dense.  The compute runs in hand-written
CUDA kernels in ``libbsp.so`` behind the C ABI of ``include/bsp.h``; this
package is the host-side front end (ctypes binding + torch tensors)."""
from . import capi  # noqa: F401

__version__ = "0.1.0"


def __getattr__(name):
    # torch-dependent helpers are imported lazily so ``import bitwise_spgemm_gb300``
    # stays light for tools that only need the C ABI binding.
    if name in ("ops", "workloads", "autograd"):
        import importlib
        return importlib.import_module("." + name, __name__)
    raise AttributeError(name)
