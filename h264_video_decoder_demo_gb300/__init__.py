"""GB300-native H.264 macroblock-reconstruction engine.

The product is libh264r.so (CUDA for sm_103a behind the C ABI in
include/h264r.h); this package builds it in-tree and binds it for Python
callers (tests, benchmarks, serving loop).
"""
from . import records  # noqa: F401
from .engine import Context, EngineError, Order, Server, Stream, Synth, lib, synth, validate  # noqa: F401

__all__ = ["records", "Context", "Stream", "Synth", "EngineError", "lib", "synth", "validate"]
