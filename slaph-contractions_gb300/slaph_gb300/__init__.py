"""GB300 engine for the sLapH contraction hot path (VdaggerV, diluted factors,
diluted traces, correlator assembly) behind the reference's interfaces.

The compute path is libslaph_gb300.so (hand-written sm_103a CUDA kernels plus a
C++ host layer) driven through the C ABI of include/slaph_gb300.h; this Python
package is a thin ctypes mirror of the reference classes for tests and tools.
"""
from ._lib import SlaphError, LIB_PATH  # noqa: F401
from .frontend import GlobalData  # noqa: F401
