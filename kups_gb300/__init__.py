"""kups_gb300: GB300-native (sm_103a) kernels for kUPS's batched particle-interaction path.

Host-side mirrors of kUPS's ``NearestNeighborList``, ``Potential`` and
``Propagator`` interfaces over a C-ABI CUDA library (``libkups_gb300.so``,
declared in ``include/kups_gb300.h``).  There is no CPU fallback: every
compute call goes through the CUDA library and raises if it is unavailable.
"""

__version__ = "0.1.0"
