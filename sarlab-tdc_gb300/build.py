"""Build recipe of the GB300 TDC engine: ``libtdc_gb300.so`` (in-tree).

Every CUDA translation unit is compiled for sm_103a only
(``-gencode arch=compute_103a,code=sm_103a``), in parallel, then linked with
the static CUDA runtime into one shared library exporting the C ABI of
``include/tdc_gb300.h``. ptxas resource usage of each kernel goes to
``_build/ptxas.log``.
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
INCLUDE = ROOT / "include"
BUILD = PKG / "_build"
LIB = PKG / "libtdc_gb300.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_SOURCES = ["tdc_focus.cu", "tdc_general.cu", "tdc_motion.cu", "tdc_fp64.cu", "tdc_prep.cu", "tdc_probe.cu",
              "tdc_noalloc.cu", "tdc_adjoint.cu"]
CPP_SOURCES = ["tdc_capi.cpp", "tdc_server.cpp"]


def nvcc() -> str:
    cand = shutil.which("nvcc") or os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found: the GB300 TDC engine needs the CUDA toolkit to build")
    return cand


def _deps() -> list[Path]:
    return sorted(CSRC.glob("*")) + sorted(INCLUDE.glob("*.h")) + [Path(__file__)]


def _stale(out: Path, deps: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps if d.exists())


def _compile(src: str, out_dir: Path, defines: tuple[str, ...]) -> tuple[Path, str]:
    obj = out_dir / (src + ".o")
    common = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-I", str(INCLUDE), "-I", str(CSRC), *defines]
    if src.endswith(".cu"):
        cmd = [nvcc(), *ARCH, "-lineinfo", "-Xptxas", "-v", *common, "-c", str(CSRC / src), "-o", str(obj)]
    else:
        cmd = [nvcc(), *common, "-x", "c++", "-c", str(CSRC / src), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile of {src} failed:\n{r.stdout}\n{r.stderr}")
    return obj, r.stderr


def build(force: bool = False, verbose: bool = False, defines: tuple[str, ...] = (), out_dir: Path = BUILD,
          lib: Path = LIB) -> Path:
    """Compile and link the engine. ``defines`` (``-DNAME=VALUE`` flags) select compile-time
    variants of the kernels, built into ``out_dir`` / ``lib`` (the focus-kernel tuning sweep)."""
    deps = _deps()
    if not force and not defines and not _stale(lib, deps):
        return lib
    out_dir.mkdir(parents=True, exist_ok=True)
    srcs = CU_SOURCES + CPP_SOURCES
    with ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 1)) as ex:
        results = list(ex.map(lambda s: _compile(s, out_dir, tuple(defines)), srcs))
    (out_dir / "ptxas.log").write_text("".join(log for _, log in results))
    objs = [str(o) for o, _ in results]
    tmp = lib.with_name(lib.name + ".tmp%d" % os.getpid())
    cmd = [nvcc(), *ARCH, "-shared", "-cudart", "static", "-o", str(tmp), *objs, "-lpthread", "-ldl", "-lrt"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, lib)
    if verbose:
        print((out_dir / "ptxas.log").read_text())
    return lib


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
