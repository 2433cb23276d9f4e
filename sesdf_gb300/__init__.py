"""GB300-native Solvent-Excluded Surface build (drop-in for PlathC/SESDF's SES build).

The product is the CUDA library behind include/sesgb.h (sesdf_gb300/lib/libsesgb.so)
and the C++ classes in include/bcs/; this package holds its build helpers, a Python
binding of the C ABI and the synthetic workloads.
"""
from .api import SesBatch, SesBuild, SesgbError, aabb, load_library  # noqa: F401

__all__ = ["SesBatch", "SesBuild", "SesgbError", "aabb", "load_library"]
