"""litert_gb300 — GB300-native ray-query engine for LiteRT's SDF/mesh hot path.

The compute path is CUDA for sm_103a behind a C ABI (include/lrt_gpu.h); this
package holds the build recipe, the Python host mirror of the reference's
scene/renderer interface (``lrt``) and the synthetic scene generators of the
benchmark configurations (``scenes``).
"""
from . import lrt  # noqa: F401
