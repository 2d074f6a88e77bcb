"""The C ABI libraries load here (no GPU needed) and export every declared symbol."""
import ctypes as C
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def declared(header: str) -> list:
    txt = (ROOT / "include" / header).read_text()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(farm_[a-z0-9_]+)\s*\(", txt)))


def test_host_library_exports(host_built):
    lib = C.CDLL(str(ROOT / "farm_gb300" / "lib" / "libfarm_host.so"))
    names = declared("farm_host.h")
    assert len(names) >= 8
    for n in names:
        assert hasattr(lib, n), n


def test_gpu_library_loads_and_exports(host_built):
    from farm_gb300 import build
    build.build_cuda()
    lib = C.CDLL(str(ROOT / "farm_gb300" / "lib" / "libfarm_gpu.so"))
    names = declared("farm_gpu.h")
    assert "farm_intersect" in names and "farm_rasterize" in names
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
