"""GB300-native proton transport for moqui's dose engine: a C ABI (libmqigpu.so) over
hand-written sm_103a kernels, with a thin Python binding for tests, benchmarks and the
differentiable Dij operator."""
from . import build  # noqa: F401

__all__ = ["build", "capi"]
