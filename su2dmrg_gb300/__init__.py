"""GB300-native SU(2) block-sparse DMRG hot path (H_eff*psi, Lanczos) behind
the C ABI of libsu2g.so (include/su2g.h)."""
__version__ = "0.1.0"
