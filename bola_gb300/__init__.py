"""bola_gb300 — BOLA's dense BLAS-3/LAPACK path on GB300 (sm_103a) CUDA.

The routines live in the C-ABI library ``lib/libbola_gb300.so`` (declared in
``include/bola_gb300.h``); ``bola_gb300.api`` mirrors BOLA's Rust signatures
over device buffers.  Nothing here falls back to the CPU: if the library is
missing, every call raises.
"""
from . import workloads  # noqa: F401

__all__ = ["workloads"]
