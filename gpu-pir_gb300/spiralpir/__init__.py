"""GB300-native Spiral PIR server answer path.

The compute path is the CUDA library ``libspiralpir.so`` (sources in
``gpu-pir_gb300/csrc``) behind the C ABI declared in ``include/spiralpir.h``;
this package holds its ctypes binding (``lib``), the host-side Spiral client
(``client``, ``ring``), parameters and the serving loop.
"""
from .params import PARAMS, DbShape, SpiralParams  # noqa: F401
