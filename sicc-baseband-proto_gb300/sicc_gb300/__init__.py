"""GB300-native receive path of the SICC baseband prototype.

LDPC decoding (layered / flooding normalized min-sum BP with an OSD fallback)
and the OFDM demodulator, as hand-written sm_103a CUDA kernels behind the
reference's C ABI (include/sicc_fec.h, include/sicc_pipe.h).  This package is
the host side: code construction, synthetic channel inputs and ctypes
wrappers of libsicc_gb300.so.
"""
from . import codes, channel  # noqa: F401

__all__ = ["codes", "channel"]
