"""ctypes binding of the sm_103a C-ABI library (include/temgym_gb300.h).

The library is built in-tree (``temgymcore_gb300/_lib/libtemgym_gb300.so``)
by ``temgymcore_gb300.build``.  There is no CPU fallback: if the library is
missing or a CUDA device is absent, calls raise ``RuntimeError``.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

import torch

from . import build as _build

TG_OK = 0
STATUS = {
    0: "ok", -1: "invalid argument", -2: "unsupported component or option",
    -3: "pointer alignment requirement violated", -4: "CUDA runtime error",
    -5: "size beyond the stated maximum", -6: "workspace too small",
}

# enum tg_kind
PLANE, LENS, SCANNER, DESCANNER, DEFLECTOR, BIPRISM, ROTATOR, THICKLENS, APERTURE, ABERLENS = range(10)
FLAG_PER_PROBE = 0x1
PROP_PARAXIAL, PROP_DIRCOS = 0, 1
MAX_COMPONENTS = 60

EW_NONFINITE, EW_TABLE, EW_TIMEOUT, EW_MMA = 0x1, 0x2, 0x4, 0x8


class TgComponent(C.Structure):
    _fields_ = [("kind", C.c_int32), ("flags", C.c_int32), ("z", C.c_double),
                ("p", C.c_double * 32)]


class TgModel(C.Structure):
    _fields_ = [("n_components", C.c_int32), ("propagator", C.c_int32),
                ("components", C.POINTER(TgComponent))]


class TgRays(C.Structure):
    _fields_ = [("n", C.c_int64), ("x", C.c_void_p), ("y", C.c_void_p), ("dx", C.c_void_p),
                ("dy", C.c_void_p), ("z", C.c_void_p), ("z_scalar", C.c_double),
                ("pathlength", C.c_void_p), ("pl_scalar", C.c_double),
                ("amplitude", C.c_void_p)]


class TgGrid(C.Structure):
    _fields_ = [("h", C.c_int32), ("w", C.c_int32), ("m", C.c_double * 6)]


_lib = None
_lock = threading.Lock()

_SIGS = {
    "tg_version": (C.c_char_p, []),
    "tg_status_string": (C.c_char_p, [C.c_int]),
    "tg_get_error_word": (C.c_int, [C.POINTER(C.c_uint32), C.c_int]),
    "tg_trace_fwd": (C.c_int, [C.POINTER(TgModel), C.POINTER(TgRays), C.POINTER(TgRays),
                               C.POINTER(C.c_double), C.POINTER(TgGrid), C.c_void_p,
                               C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p]),
    "tg_trace_image_workspace": (C.c_size_t, [C.c_int64, C.POINTER(TgGrid)]),
    "tg_trace_image": (C.c_int, [C.POINTER(TgModel), C.POINTER(TgRays), C.POINTER(TgRays),
                                 C.POINTER(C.c_double), C.POINTER(TgGrid), C.c_void_p,
                                 C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p, C.c_size_t,
                                 C.c_void_p]),
    "tg_hist_workspace": (C.c_size_t, [C.c_int64, C.c_int32, C.c_int32]),
    "tg_bin_image": (C.c_int, [C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(TgGrid),
                               C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p, C.c_size_t,
                               C.c_void_p]),
    "tg_hist_pixels": (C.c_int, [C.c_int64, C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_int32,
                                 C.c_void_p, C.c_int32, C.c_void_p, C.c_size_t, C.c_void_p]),
    "tg_bin": (C.c_int, [C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(TgGrid),
                         C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p]),
    "tg_aber_monomials": (C.c_int, [C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_double),
                                     C.POINTER(C.c_double)]),
    "tg_abcd_compose": (C.c_int, [C.POINTER(TgModel), C.POINTER(C.c_double),
                                  C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "tg_trace_vjp_workspace": (C.c_size_t, [C.c_int64, C.POINTER(TgModel)]),
    "tg_trace_vjp": (C.c_int, [C.POINTER(TgModel), C.POINTER(TgRays), C.POINTER(TgRays),
                               C.POINTER(TgRays), C.c_void_p, C.c_void_p, C.c_size_t,
                               C.c_void_p]),
}


def register(name, restype, argtypes):
    """Declare the signature of another exported entry point."""
    _SIGS[name] = (restype, argtypes)
    if _lib is not None:
        f = getattr(_lib, name)
        f.restype, f.argtypes = restype, argtypes


def lib():
    """Load (building first if needed) the native library."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.lib_path()
        if not os.path.exists(path) or os.environ.get("TEMGYM_GB300_REBUILD"):
            path = _build.build()
        lib_ = C.CDLL(path)
        for name, (res, args) in _SIGS.items():
            f = getattr(lib_, name)
            f.restype, f.argtypes = res, args
        _lib = lib_
    return _lib


def check(status: int, what: str = "") -> None:
    if status != TG_OK:
        raise RuntimeError(f"temgym_gb300 {what}: {STATUS.get(status, status)} (status {status})")


_cuda_ok = False


def require_cuda(t: torch.Tensor | None = None) -> None:
    global _cuda_ok
    if not _cuda_ok:  # checked until it first succeeds (a per-call check costs microseconds)
        if not torch.cuda.is_available():
            raise RuntimeError("temgymcore_gb300 needs a CUDA device (sm_103a); there is no CPU path")
        _cuda_ok = True
    if t is not None and not t.is_cuda:
        raise RuntimeError("temgymcore_gb300: tensors must live on the CUDA device")


# the current stream's raw handle without building a Stream object (the
# public call is the fallback where torch does not offer the raw one)
_raw_stream = getattr(torch._C, "_cuda_getCurrentRawStream", None)


def stream_ptr() -> int:
    if _raw_stream is not None:
        return _raw_stream(torch.cuda.current_device())
    return torch.cuda.current_stream().cuda_stream


def ptr(t: torch.Tensor | None):
    return None if t is None else t.data_ptr()


def error_word(clear: bool = True) -> int:
    v = C.c_uint32(0)
    check(lib().tg_get_error_word(C.byref(v), 1 if clear else 0), "tg_get_error_word")
    return int(v.value)
