"""CPU oracle for the bitmap-SpMM path — test infrastructure only.

This package restates, in plain C (``bsp_oracle.c``) with a ctypes wrapper
(``core.py``), what the reference ZSL98/bitwise_spgemm computes on this path.
It is the checker: only ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` may import it.  The library
(``bitwise_spgemm_gb300``) never imports it and has no CPU fallback.
"""
from .core import *  # noqa: F401,F403
