"""thcpp_gb300 -- GB300-native ISDF factorisation (k-means interpolating points,
least-squares interpolating vectors, FFT Coulomb matrix) behind thcpp's interfaces.

The compute path is libthc_gb300.so (hand-written CUDA for sm_103a) reached through its
C ABI (include/thc_gb300.h); :mod:`thcpp_gb300.capi` binds it for Python.
"""

__all__ = ["capi", "synth", "build"]
