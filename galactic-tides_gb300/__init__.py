"""GB300 gravity backend for galactic-tides: `device = cuda` for the grouped
(`gravity = group`) and direct (`gravity = direct`) solvers.

The product is libgtc.so (CUDA kernels for sm_103a behind the C ABI in
include/gtc.h); this package holds its sources (csrc/), the C++ host wrapper
(host/gtc.hpp) and the Python binding of the C ABI (gtc.py).
"""

from . import gtc  # noqa: F401  (fails loudly when libgtc.so is not built)
