"""GB300-native Glynn / BBFG permanent calculators (drop-in for piquassoboost's
permanent calculator API).  Compute runs in hand-written sm_103a CUDA kernels
(libgbperm.so) called through a C ABI; there is no CPU fallback."""

__version__ = "0.1.0"
