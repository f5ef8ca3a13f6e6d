"""diaq_gb300 -- DiaQ's diagonal-sparse hot path on GB300 (sm_103a).

Two ways in, both over the native library libdiaq_gb300.so (CUDA kernels + C ABI):
  ``from diaq_gb300 import diaq_gpu``  the drop-in for the reference's ``diaq_gpu`` pybind11 module
  ``diaq_gb300.capi``                  ctypes bindings of the C ABI in include/diaq_gb300.h

``diaq_gb300.hamiltonians`` builds test Hamiltonians (TFIM, XXZ, Pauli sums) in the DiaQ format.
Build the native parts with ``python -m diaq_gb300.build``; importing ``diaq_gpu`` without them
raises ImportError -- there is no CPU fallback.
"""
__all__ = ["hamiltonians", "capi", "build"]
