"""GB300-native batch controller-tuning engine (drop-in for ControllerEngine's tuning path).

The product is libControllerEngine.so (C ABI in include/controller_engine.h,
CUDA kernels for sm_103a under csrc/).  This package builds it in-tree and
wraps it for Python callers; see engine.py.
"""
from .engine import (ControllerEngineError, EngineConfig, PlantFiles, Ragged, Request, Server, Session,
                     decode_instructions, run_controller_engine)
from ._ffi import load_library, LIB_PATH

__all__ = ["ControllerEngineError", "EngineConfig", "PlantFiles", "Ragged", "Request", "Server", "Session",
           "decode_instructions",
           "run_controller_engine", "load_library", "LIB_PATH"]
