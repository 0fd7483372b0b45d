"""GB300-native Dual Threshold Optimization.

The permutation null of the threshold-pair search (the reference crate's
``src/dto``, ``src/stat_operations`` and ``src/run`` hot path) runs in
hand-written CUDA for sm_103a behind the C ABI of ``include/dto.h``
(``libdto.so``).  The Python modules mirror the reference's library surface.
"""
from .engine import DevicePair, Engine, Job, Server  # noqa: F401

__version__ = "0.1.0"
