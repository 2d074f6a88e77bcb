"""ctypes bindings of the engine's native libraries.

The GPU library is mandatory for every query path: if it is missing the
import of the query functions fails loudly instead of falling back to any CPU
code.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

LIB_DIR = Path(__file__).resolve().parent / "lib"

u8p = C.POINTER(C.c_uint8)
u32p = C.POINTER(C.c_uint32)
u64p = C.POINTER(C.c_uint64)
f32p = C.POINTER(C.c_float)
f64p = C.POINTER(C.c_double)


class FarmError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"farm error {code}: {msg}")
        self.code = code


class GenParams(C.Structure):
    _fields_ = [("dom_lo", C.c_double), ("dom_hi", C.c_double), ("r_lo", C.c_double), ("r_hi", C.c_double),
                ("n_lo", C.c_int32), ("n_hi", C.c_int32), ("sigma", C.c_double)]


_host = None
_gpu = None


def host() -> C.CDLL:
    global _host
    if _host is None:
        path = LIB_DIR / "libfarm_host.so"
        if not path.exists():
            raise ImportError(f"{path} is not built; run farm_gb300.build.build_all()")
        lib = C.CDLL(str(path))
        lib.farm_host_last_error.restype = C.c_char_p
        lib.farm_gen_counts.argtypes = [C.POINTER(GenParams), C.c_uint64, C.c_uint64, C.c_uint64, u32p]
        lib.farm_gen_fill.argtypes = [C.POINTER(GenParams), C.c_uint64, C.c_uint64, C.c_uint64, u64p, f32p, C.c_int]
        lib.farm_gen_centres.argtypes = [C.POINTER(GenParams), C.c_uint64, C.c_uint64, C.c_uint64, f64p]
        lib.farm_gen_radii.argtypes = [C.POINTER(GenParams), C.c_uint64, C.c_uint64, C.c_uint64, f64p, C.c_int]
        lib.farm_gen_counts_idx.argtypes = [C.POINTER(GenParams), C.c_uint64, u64p, C.c_uint64, u32p]
        lib.farm_gen_fill_idx.argtypes = [C.POINTER(GenParams), C.c_uint64, u64p, C.c_uint64, u64p, f32p, C.c_int]
        lib.farm_dt_write.argtypes = [C.c_char_p, C.c_uint64, u64p, f32p]
        lib.farm_dt_read.argtypes = [C.c_char_p, u64p, u64p, u64p, f32p]
        lib.farm_wkt_read.argtypes = [C.c_char_p, u64p, u64p, u64p, f32p]
        lib.farm_wkt_to_dt.argtypes = [C.c_char_p, C.c_char_p, u64p]
        lib.farm_mbr.argtypes = [C.c_uint64, u64p, f32p, f64p, C.c_int]
        lib.farm_mbr_join.argtypes = [C.c_uint64, f64p, C.c_uint64, f64p, C.c_double, C.c_int, C.c_int, u64p, u32p,
                                      C.c_int]
        lib.farm_degree_table.argtypes = [f64p]
        lib.farm_degree_table.restype = None
        _host = lib
    return _host


def check_host(rc: int) -> None:
    if rc != 0:
        raise FarmError(rc, host().farm_host_last_error().decode())


def gpu() -> C.CDLL:
    """The CUDA library; raises if it is not built (no CPU fallback exists)."""
    global _gpu
    if _gpu is None:
        path = LIB_DIR / "libfarm_gpu.so"
        if not path.exists():
            raise ImportError(f"{path} is not built: the GPU engine is required (build with farm_gb300.build)")
        lib = C.CDLL(str(path))
        from . import _gpu_sig
        _gpu_sig.declare(lib)
        _gpu = lib
    return _gpu


def check_gpu(rc: int) -> None:
    if rc != 0:
        raise FarmError(rc, gpu().farm_last_error().decode())


def ptr(a, t):
    return a.ctypes.data_as(t)
