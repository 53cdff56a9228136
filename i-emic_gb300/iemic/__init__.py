"""GB300 engine for the THCM Newton step of I-EMIC.

``iemic.Ocean`` mirrors the reference's ``Ocean`` model (src/ocean/Ocean.H)
over the C ABI in ``include/iemic_gb300.h``; the compute runs in the CUDA
library ``libiemic_gb300.so`` built in-tree for sm_103a. There is no CPU
fallback: without a GPU or without the library every compute call raises.
"""
from .ocean import Ocean, IemicError, PARAMETER_NAMES, load_library  # noqa: F401
from . import workloads  # noqa: F401
