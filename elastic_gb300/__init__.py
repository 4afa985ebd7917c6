"""GB300-native (sm_103a) engine for the elastic RTM hot path of lgan/elastic.

The compute lives in libelastic_rtm.so (hand-written CUDA behind the C-ABI
of include/elastic_rtm.h); this package is its Python mirror.
"""
from ._lib import RtmError, load  # noqa: F401
from . import rtm  # noqa: F401

__all__ = ["RtmError", "load", "rtm"]
