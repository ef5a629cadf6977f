"""Build ``libtrvg.so`` (the CUDA kernels and the C ABI) for sm_103a.

Each ``csrc/*.cu`` file is compiled by nvcc in parallel and linked into
``triumvirate_gb300/libtrvg.so`` in the source tree.  Host code is compiled
with ``-ffp-contract=off`` so that wavevector magnitudes and bin edges round
exactly as in the reference on every host architecture.

Then the C++ drop-in layer (``csrc/dropin/trv_dropin.cpp``, the reference's
``trv::`` estimator interface over the C ABI) is compiled by the host C++
compiler into ``triumvirate_gb300/libtrv_dropin.so``, and the C++ test
program ``tests/cpp/dropin_bispec_gpp.cpp`` into ``_build/``.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libtrvg.so"
ARCH = "-gencode=arch=compute_103a,code=sm_103a"
DROPIN_SRC = CSRC / "dropin" / "trv_dropin.cpp"
DROPIN_LIB = PKG / "libtrv_dropin.so"
DROPIN_TEST_SRC = ROOT / "tests" / "cpp" / "dropin_bispec_gpp.cpp"
DROPIN_TEST = BUILD / "dropin_bispec_gpp"


def _nvcc():
    cuda_home = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    cand = Path(cuda_home) / "bin" / "nvcc"
    if cand.exists():
        return str(cand)
    found = shutil.which("nvcc")
    if not found:
        raise RuntimeError("nvcc not found; set CUDA_HOME")
    return found


def _flags():
    return [
        "-std=c++17", "-O3", ARCH, "-lineinfo",
        "-Xcompiler", "-fPIC,-ffp-contract=off,-O2",
        "-Xptxas", "-O3",
        f"-I{ROOT / 'include'}", f"-I{CSRC}",
    ]


def _sources():
    return sorted(CSRC.glob("*.cu"))


def _needs_rebuild(obj: Path, src: Path) -> bool:
    if not obj.exists():
        return True
    deps = [src] + list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + [
        ROOT / "include" / "trvg.h"]
    t = obj.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> Path:
    """Compile and link the library; returns its path."""
    nvcc = _nvcc()
    BUILD.mkdir(exist_ok=True)
    srcs = _sources()
    objs = [BUILD / (s.stem + ".o") for s in srcs]

    def compile_one(pair):
        src, obj = pair
        if not force and not _needs_rebuild(obj, src):
            return None
        cmd = [nvcc, *_flags(), "-c", str(src), "-o", str(obj)]
        if verbose:
            cmd.insert(1, "-Xptxas=-v")
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src.name}:\n{r.stderr}")
        return r.stderr if verbose else None

    workers = min(len(srcs), os.cpu_count() or 4)
    with ThreadPoolExecutor(max_workers=workers) as ex:
        for out in ex.map(compile_one, zip(srcs, objs)):
            if out:
                sys.stderr.write(out)
    newest = max(o.stat().st_mtime for o in objs)
    if force or not LIB.exists() or LIB.stat().st_mtime < newest:
        tmp = LIB.with_suffix(".so.tmp")
        cmd = [nvcc, ARCH, "-shared", "-o", str(tmp),
               *[str(o) for o in objs], "-lcufft"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stderr}")
        os.replace(tmp, LIB)
    build_dropin(force=force)
    return LIB


def _cxx():
    return os.environ.get("CXX") or shutil.which("g++") or "c++"


def _run(cmd, what):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"{what} failed:\n{r.stderr}")


def build_dropin(force: bool = False) -> Path:
    """The C++ drop-in library and its test program (host C++ only)."""
    cxx = _cxx()
    inc = [f"-I{ROOT / 'include'}"]
    newest = max(LIB.stat().st_mtime, DROPIN_SRC.stat().st_mtime,
                 (ROOT / "include" / "trv_dropin.hpp").stat().st_mtime,
                 (ROOT / "include" / "trvg.h").stat().st_mtime)
    if force or not DROPIN_LIB.exists() or \
            DROPIN_LIB.stat().st_mtime < newest:
        tmp = DROPIN_LIB.with_suffix(".so.tmp")
        _run([cxx, "-std=c++17", "-O2", "-fPIC", "-shared",
              "-ffp-contract=off", *inc, str(DROPIN_SRC), "-o", str(tmp),
              f"-L{PKG}", "-ltrvg", "-Wl,-rpath,$ORIGIN"],
             "drop-in library build")
        os.replace(tmp, DROPIN_LIB)
    BUILD.mkdir(exist_ok=True)
    if force or not DROPIN_TEST.exists() or \
            DROPIN_TEST.stat().st_mtime < max(
                DROPIN_LIB.stat().st_mtime,
                DROPIN_TEST_SRC.stat().st_mtime):
        _run([cxx, "-std=c++17", "-O2", *inc, str(DROPIN_TEST_SRC), "-o",
              str(DROPIN_TEST), f"-L{PKG}", "-ltrv_dropin", "-ltrvg",
              f"-Wl,-rpath,{PKG}"], "drop-in test program build")
    return DROPIN_LIB


if __name__ == "__main__":
    build(verbose="-v" in sys.argv, force="-f" in sys.argv)
    print(LIB)
