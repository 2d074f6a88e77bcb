"""In-tree build of the engine's native libraries.

* ``farm_gb300/lib/libfarm_gpu.so``  — CUDA kernels + the C ABI (include/farm_gpu.h),
  compiled for sm_103a only.
* ``farm_gb300/lib/libfarm_host.so`` — host services (include/farm_host.h).
* ``farm_gb300/lib/farm_query``      — the drop-in query executable.
* ``oracle/liboracle.so``            — the CPU restatement the tests verify results against.
* ``oracle/_ref/*``                  — the reference's own CPU code, only where its
  source tree is present (never on a machine without it).

Everything is compiled straight with nvcc/g++ (no cmake), translation units in
parallel, so a fresh machine builds in about a minute.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
LIB = PKG / "lib"
CSRC = PKG / "csrc"
HOST = PKG / "host"
ORACLE = ROOT / "oracle"


def ref_src() -> Path | None:
    """The reference's source tree: FARM_REF_SRC, else the default that the
    recipe in oracle/ref/Makefile names. None when that tree is absent."""
    env = os.environ.get("FARM_REF_SRC")
    if env:
        p = Path(env)
    else:
        r = subprocess.run(["make", "-s", "-C", str(ORACLE / "ref"), "print-ref"], stdout=subprocess.PIPE,
                           stderr=subprocess.DEVNULL, text=True)
        if r.returncode != 0 or not r.stdout.strip():
            return None
        p = Path(r.stdout.strip())
    return p if (p / "geometry" / "Ideal.cpp").exists() else None

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
HOST_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-pthread"]


def _run(cmd: list[str], cwd: Path | None = None) -> None:
    r = subprocess.run(cmd, cwd=cwd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed ({r.returncode}): {' '.join(cmd)}\n{r.stdout}")


def _newer(out: Path, deps: list[Path]) -> bool:
    if not out.exists():
        return False
    t = out.stat().st_mtime
    return all(d.stat().st_mtime <= t for d in deps if d.exists())


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and Path(c).exists():
            return c
    raise RuntimeError("nvcc not found")


def build_host() -> Path:
    LIB.mkdir(exist_ok=True)
    out = LIB / "libfarm_host.so"
    srcs = sorted(HOST.glob("farm_host*.cpp"))
    deps = srcs + [ROOT / "include" / "farm_host.h"]
    if not _newer(out, deps):
        _run(["g++", *HOST_FLAGS, "-shared", "-o", str(out), *map(str, srcs)])
    return out


def build_oracle() -> Path:
    out = ORACLE / "liboracle.so"
    deps = [ORACLE / "farm_oracle.c", ORACLE / "farm_oracle.h"]
    if not _newer(out, deps):
        _run(["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-ffp-contract=off", "-o", str(out),
              str(ORACLE / "farm_oracle.c"), "-lm"])
    return out


def build_ref() -> Path | None:
    """Compile the reference's CPU code into oracle/_ref when its sources exist."""
    src = ref_src()
    if src is None:
        return None
    _run(["make", "-s", "-C", str(ORACLE / "ref"), f"REF={src}", f"-j{os.cpu_count() or 4}"])
    return ORACLE / "_ref" / "ref_harness"


def _cu_objs() -> list[tuple[Path, Path]]:
    objdir = LIB / "obj"
    objdir.mkdir(parents=True, exist_ok=True)
    return [(s, objdir / (s.stem + ".o")) for s in sorted(CSRC.glob("*.cu"))]


def build_cuda() -> Path:
    LIB.mkdir(exist_ok=True)
    out = LIB / "libfarm_gpu.so"
    headers = list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + [ROOT / "include" / "farm_gpu.h"]
    pairs = _cu_objs()
    if not pairs:
        raise RuntimeError("no CUDA sources")
    nv = nvcc()
    flags = ["-O3", "-std=c++17", *ARCH, "-lineinfo", "-Xcompiler", "-fPIC", "-fmad=false",
             "--expt-relaxed-constexpr", "-I", str(ROOT / "include"), "-I", str(CSRC)]

    def one(p: tuple[Path, Path]) -> None:
        src, obj = p
        if _newer(obj, [src, *headers]):
            return
        _run([nv, *flags, "-c", str(src), "-o", str(obj)])

    with cf.ThreadPoolExecutor(max_workers=min(len(pairs), os.cpu_count() or 4)) as ex:
        list(ex.map(one, pairs))
    objs = [o for _, o in pairs]
    if not _newer(out, objs):
        _run([nv, *ARCH, "-shared", "-o", str(out), *map(str, objs), "-lcudart"])
    return out


def build_query_exe() -> Path:
    out = LIB / "farm_query"
    src = HOST / "query_main.cpp"
    if not src.exists():
        return out
    deps = [src, ROOT / "include" / "farm_gpu.h", ROOT / "include" / "farm_host.h"]
    if not _newer(out, deps + [LIB / "libfarm_gpu.so", LIB / "libfarm_host.so"]):
        _run(["g++", *HOST_FLAGS, "-o", str(out), str(src), f"-L{LIB}", "-lfarm_gpu", "-lfarm_host",
              f"-Wl,-rpath,$ORIGIN", "-I", str(ROOT / "include")])
    # the reference's program names, dispatched on by the binary
    for name in ("intersect", "within_polygon", "intersection"):
        link = LIB / name
        if link.is_symlink() or link.exists():
            link.unlink()
        link.symlink_to(out.name)
    return out


def build_tools_exe() -> Path:
    """dump_polygons and generate_polygons: one host-only binary, two names."""
    out = LIB / "farm_tools"
    src = HOST / "tools_main.cpp"
    deps = [src, ROOT / "include" / "farm_host.h", LIB / "libfarm_host.so"]
    if not _newer(out, deps):
        _run(["g++", *HOST_FLAGS, "-o", str(out), str(src), f"-L{LIB}", "-lfarm_host", f"-Wl,-rpath,$ORIGIN",
              "-I", str(ROOT / "include")])
    for name in ("dump_polygons", "generate_polygons"):
        link = LIB / name
        if link.is_symlink() or link.exists():
            link.unlink()
        link.symlink_to(out.name)
    return out


def build_all(with_ref: bool = True) -> None:
    with cf.ThreadPoolExecutor(max_workers=3) as ex:
        futs = [ex.submit(build_host), ex.submit(build_oracle), ex.submit(build_cuda)]
        if with_ref:
            futs.append(ex.submit(build_ref))
        for f in futs:
            f.result()
    build_query_exe()
    build_tools_exe()


if __name__ == "__main__":
    build_all(with_ref="--no-ref" not in sys.argv)
    print("built")
