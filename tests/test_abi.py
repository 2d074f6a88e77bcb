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


def test_query_program_flags_without_gpu(host_built):
    """The drop-in programs parse the reference's flags: --help lists them and
    an unknown flag prints the reference's message (no GPU needed)."""
    import subprocess
    from pathlib import Path
    lib = Path(__file__).resolve().parents[1] / "farm_gb300" / "lib"
    exe = lib / "intersect"
    if not exe.exists():
        pytest.skip("query program not built")
    h = subprocess.run([str(exe), "--help"], capture_output=True, text=True, timeout=60)
    assert h.returncode == 0
    for flag in ("--rasterize", "--gpu", "--approximation", "--hierachy", "--source", "--target", "--threads",
                 "--vpr", "--batch_size", "--merge_threshold", "--within_distance", "--category_count"):
        assert flag in h.stderr, flag
    u = subprocess.run([str(exe), "--bogus"], capture_output=True, text=True, timeout=60)
    assert "Undefined Option!" in u.stdout


def test_gpu_library_reports_errors_without_a_gpu(host_built):
    """With no usable GPU the ABI returns an error code and a message; it never
    exits, aborts or dereferences a null store."""
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    from farm_gb300 import build
    build.build_cuda()
    lib = C.CDLL(str(ROOT / "farm_gb300" / "lib" / "libfarm_gpu.so"))
    lib.farm_last_error.restype = C.c_char_p
    st = C.c_void_p(None)
    rc = lib.farm_store_create(C.byref(st))
    assert rc < 0 and not st.value
    assert lib.farm_last_error()
    # null stores are rejected before any device work
    found = C.c_uint64(0)
    for call in (lambda: lib.farm_intersect(None, None, C.c_uint64(0), 0, 0, None, C.byref(found), None),
                 lambda: lib.farm_within_mode(None, None, C.c_uint64(0), C.c_double(10.0), 1, 1, 0, 0, None,
                                              C.byref(found), None),
                 lambda: lib.farm_intersection_area(None, None, C.c_uint64(0), 0, None, None)):
        assert call() < 0
        assert lib.farm_last_error()
