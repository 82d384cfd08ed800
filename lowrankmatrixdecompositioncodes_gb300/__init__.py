"""GB300-native RSVDPACK engine.

The product is the C-ABI shared library ``librsvdpack.so`` built from ``csrc/`` for
sm_103a (see ``include/rsvdpack.h``).  This package only locates, builds and binds it:
``load_engine()`` returns a :class:`capi.RsvdLibrary` over the engine with the
reference's API names.  There is no CPU fallback: if the library is missing,
``load_engine()`` raises; if no GB300 is visible, every decomposition call reports
``RSVD_ERR_NO_DEVICE`` through ``rsvdpack_last_error()``.  ``load_engine64()`` binds
``librsvdpack64.so``, the same engine behind the reference API with int64_t dimensions;
``load_engine_f32()`` binds ``librsvdpack_f32.so``, the oneAPI variant's float-data API.
"""
from __future__ import annotations

import ctypes as C
import os

from .capi import RsvdLibrary

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG_DIR, "librsvdpack.so")
LIB64_PATH = os.path.join(PKG_DIR, "librsvdpack64.so")
LIBF32_PATH = os.path.join(PKG_DIR, "librsvdpack_f32.so")

PREC = {"fp64": 0, "fp32": 1, "tf32": 2, "bf16": 3, "fp64x": 4}


class RsvdOpts(C.Structure):
    _fields_ = [("precision", C.c_int), ("use_provider", C.c_int), ("seed", C.c_ulonglong),
                ("verbose", C.c_int), ("learned", C.c_int), ("reserved", C.c_int * 7)]


class RsvdTiming(C.Structure):
    _fields_ = [("upload_ms", C.c_double), ("sketch_ms", C.c_double), ("orth_ms", C.c_double),
                ("small_ms", C.c_double), ("download_ms", C.c_double), ("total_ms", C.c_double),
                ("gemm_launches", C.c_longlong), ("kernel_launches", C.c_longlong),
                ("learned_path", C.c_int), ("pad_", C.c_int)]


class EngineLibrary(RsvdLibrary):
    """RsvdLibrary plus the engine's extension entry points (include/rsvdpack.h Part 2)."""

    def __init__(self, path: str = LIB_PATH, index64: bool = False, real32: bool = False):
        super().__init__(path, index64=index64, real32=real32)
        L = self.lib
        L.rsvdpack_last_error.restype = C.c_int
        L.rsvdpack_last_error_string.restype = C.c_char_p
        L.rsvdpack_get_opts.argtypes = [C.POINTER(RsvdOpts)]
        L.rsvdpack_set_opts.argtypes = [C.POINTER(RsvdOpts)]
        L.rsvdpack_device_info.argtypes = [C.c_char_p, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int)]
        L.rsvdpack_device_info.restype = C.c_int
        L.rsvdpack_last_timing.argtypes = [C.POINTER(RsvdTiming)]

    def last_error(self):
        return int(self.lib.rsvdpack_last_error()), self.lib.rsvdpack_last_error_string().decode()

    def check(self):
        code, msg = self.last_error()
        if code:
            raise RuntimeError(f"rsvdpack error {code}: {msg}")

    def get_opts(self) -> RsvdOpts:
        o = RsvdOpts()
        self.lib.rsvdpack_get_opts(C.byref(o))
        return o

    def set_precision(self, prec: str):
        o = self.get_opts()
        o.precision = PREC[prec]
        self.lib.rsvdpack_set_opts(C.byref(o))

    def set_use_provider(self, flag: bool):
        o = self.get_opts()
        o.use_provider = 1 if flag else 0
        self.lib.rsvdpack_set_opts(C.byref(o))

    def set_learned(self, flag: bool):
        """Fixed-precision QB (randQB_pb_new, TOL mode, FP32 data) through the learned proposal."""
        o = self.get_opts()
        o.learned = 1 if flag else 0
        self.lib.rsvdpack_set_opts(C.byref(o))

    def load_proposal_model(self, path: str):
        self.lib.rsvdpack_load_proposal_model.argtypes = [C.c_char_p]
        if self.lib.rsvdpack_load_proposal_model(path.encode()) != 0:
            raise RuntimeError(self.last_error())

    def device_info(self):
        name = C.create_string_buffer(128)
        maj, mnr = C.c_int(0), C.c_int(0)
        sms = self.lib.rsvdpack_device_info(name, 128, C.byref(maj), C.byref(mnr))
        return sms, name.value.decode(), (maj.value, mnr.value)

    def last_timing(self) -> RsvdTiming:
        t = RsvdTiming()
        self.lib.rsvdpack_last_timing(C.byref(t))
        return t


_ENGINE = None
_ENGINE64 = None
_ENGINE_F32 = None


def build(verbose: bool = False) -> str:
    from .build import build as _build
    return _build(verbose=verbose)


def load_engine() -> EngineLibrary:
    """Load librsvdpack.so (building it first if it is absent).  Raises if it cannot."""
    global _ENGINE
    if _ENGINE is None:
        if not os.path.exists(LIB_PATH):
            build()
        _ENGINE = EngineLibrary(LIB_PATH)
    return _ENGINE


def load_engine64() -> EngineLibrary:
    """Load librsvdpack64.so, the int64_t-dimension form of the reference API."""
    global _ENGINE64
    if _ENGINE64 is None:
        if not os.path.exists(LIB64_PATH):
            build()
        _ENGINE64 = EngineLibrary(LIB64_PATH, index64=True)
    return _ENGINE64


def load_engine_f32() -> EngineLibrary:
    """Load librsvdpack_f32.so, the float-data (oneAPI variant) form of the reference API."""
    global _ENGINE_F32
    if _ENGINE_F32 is None:
        if not os.path.exists(LIBF32_PATH):
            build()
        _ENGINE_F32 = EngineLibrary(LIBF32_PATH, real32=True)
    return _ENGINE_F32


def engine_available() -> bool:
    """True when the engine loads and a GB300 (sm_103) is visible."""
    try:
        sms, _, cc = load_engine().device_info()
        return sms > 0 and cc == (10, 3)
    except Exception:
        return False
