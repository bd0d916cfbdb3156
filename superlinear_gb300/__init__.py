"""GB300-native SUS2-SH descriptor -> energy -> force / virial / parameter-gradient engine.

The compute path is hand-written CUDA for sm_103a behind the C ABI of ``include/sus2g.h``
(``superlinear_gb300/_build/libsus2g.so``, built by ``superlinear_gb300.build.build()``).
"""
from .engine import FP32, FP64, Engine, Model, Sus2Error  # noqa: F401
from .trainer import Trainer  # noqa: F401

__version__ = "0.1.0"
