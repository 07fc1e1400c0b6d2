"""GB300-native H.264 macroblock-reconstruction engine.

The product is libh264r.so (CUDA for sm_103a behind the C ABI in
include/h264r.h, with the host front end of include/h264r_parser.h and the
whole-stream decoder of include/h264r_decoder.h); this package builds it
in-tree and binds it for Python callers (tests, benchmarks, serving loop).
"""
from . import records  # noqa: F401
from .engine import (Context, Decoder, EngineError, Order, Parser, Server, Stream, Synth, lib, synth,  # noqa: F401
                     validate, write_stream)

__all__ = ["records", "Context", "Decoder", "Parser", "Order", "Server", "Stream", "Synth", "EngineError", "lib",
           "synth", "validate", "write_stream"]
