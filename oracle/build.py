"""Build recipe for the oracle (test infrastructure only).

* ``oracle/_build/libtdc_oracle.so`` -- the FP64 C restatement in
  ``oracle/tdc_oracle.c`` (gcc -O2 -fopenmp).
* ``oracle/_ref/tdckernels.ptx`` -- the reference's own GPU kernels
  (``tdc-lib/src/tdckernels.cu``) compiled to PTX by nvcc from where the source
  lies in the reference checkout (fmt from torch's bundled headers). PTX is
  architecture-neutral text, so it can be loaded on any machine with a GB300, where
  tests/golden/make_ref_gpu_golden.py runs those kernels to record golden images.
* ``oracle/_ref/libtdc_refmath.so`` -- the reference's own host-side math
  (``tdc-lib/include/gpumath.h`` and ``windowing.h``, compiled from where they
  lie in the reference checkout by g++, through ``oracle/ref_math_shim.cpp``).
  Built only when the reference checkout is present (``TDC_REFERENCE_ROOT`` or
  ``/root/reference``); it is used to pin the oracle's window and quaternion
  math to the reference's, never by the product.

Both outputs are git-ignored build products.
"""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
REF_OUT = HERE / "_ref"
ORACLE_SO = BUILD / "libtdc_oracle.so"
REFMATH_SO = REF_OUT / "libtdc_refmath.so"


def reference_root() -> Path | None:
    root = Path(os.environ.get("TDC_REFERENCE_ROOT", "/root/reference"))
    inc = root / "tdc-lib" / "include"
    if (inc / "gpumath.h").is_file() and (inc / "windowing.h").is_file():
        return root
    return None


def _stale(out: Path, srcs: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(s.stat().st_mtime > t for s in srcs)


def build_oracle(force: bool = False) -> Path:
    src = HERE / "tdc_oracle.c"
    if force or _stale(ORACLE_SO, [src, Path(__file__)]):
        BUILD.mkdir(exist_ok=True)
        tmp = ORACLE_SO.with_suffix(".so.tmp%d" % os.getpid())
        cmd = ["gcc", "-O2", "-fopenmp", "-fPIC", "-shared", "-std=c11", "-Wall",
               "-o", str(tmp), str(src), "-lm"]
        subprocess.run(cmd, check=True)
        os.replace(tmp, ORACLE_SO)
    return ORACLE_SO


def build_refmath(force: bool = False) -> Path | None:
    root = reference_root()
    if root is None:
        return REFMATH_SO if REFMATH_SO.exists() else None
    inc = root / "tdc-lib" / "include"
    shim = HERE / "ref_math_shim.cpp"
    srcs = [shim, inc / "gpumath.h", inc / "windowing.h", inc / "tuning.h", Path(__file__)]
    if force or _stale(REFMATH_SO, srcs):
        REF_OUT.mkdir(exist_ok=True)
        cuda_inc = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda")) / "include"
        tmp = REFMATH_SO.with_suffix(".so.tmp%d" % os.getpid())
        # -ffp-contract=off: the host build of the reference math does plain
        # IEEE float operations, no fused multiply-adds.
        cmd = ["g++", "-O2", "-fPIC", "-shared", "-std=c++17", "-ffp-contract=off",
               "-I", str(inc), "-I", str(cuda_inc), "-o", str(tmp), str(shim)]
        subprocess.run(cmd, check=True)
        os.replace(tmp, REFMATH_SO)
    return REFMATH_SO


REF_PTX = REF_OUT / "tdckernels.ptx"


def build_ref_ptx(force: bool = False) -> Path | None:
    """PTX of the reference's tdckernels.cu (built only where the checkout is present)."""
    root = reference_root()
    if root is None:
        return REF_PTX if REF_PTX.exists() else None
    src = root / "tdc-lib" / "src" / "tdckernels.cu"
    inc = root / "tdc-lib" / "include"
    if not force and not _stale(REF_PTX, [src, inc / "gpumath.h", inc / "windowing.h", inc / "tuning.h",
                                          Path(__file__)]):
        return REF_PTX
    try:
        import torch.utils.cpp_extension as ext
        torch_inc = ext.include_paths()[0]
    except Exception:
        return None
    REF_OUT.mkdir(exist_ok=True)
    nvcc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    tmp = REF_PTX.with_suffix(".ptx.tmp%d" % os.getpid())
    cmd = [nvcc, "-ptx", "-arch=compute_103a", "-std=c++17", "-DFMT_HEADER_ONLY", "-I", str(inc), "-I", torch_inc,
           "-w", str(src), "-o", str(tmp)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        return None
    os.replace(tmp, REF_PTX)
    return REF_PTX


REF_HOST_LOOP = REF_OUT / "ref_host_loop"
HOST_LOOP_SRC = HERE.parent / "tests" / "golden" / "ref_host_loop.cpp"


def build_ref_host_loop(force: bool = False) -> Path | None:
    """The timing harness of the reference's GPU path (tests/golden/ref_host_loop.cpp: its host
    loop restated, its kernels from REF_PTX, NPP's sum) for this machine, or None where the CUDA
    toolkit's NPP headers or libraries are missing. Built from our own source, on any machine."""
    cuda = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))
    if not (cuda / "include" / "npps.h").is_file():
        return None
    if not force and not _stale(REF_HOST_LOOP, [HOST_LOOP_SRC, Path(__file__)]):
        return REF_HOST_LOOP
    REF_OUT.mkdir(exist_ok=True)
    tmp = REF_HOST_LOOP.with_suffix(".tmp%d" % os.getpid())
    libdirs = [cuda / "lib64", cuda / "lib64" / "stubs", cuda / "targets" / "sbsa-linux" / "lib",
               cuda / "targets" / "sbsa-linux" / "lib" / "stubs"]
    cmd = ["g++", "-O2", "-std=c++17", "-I", str(cuda / "include"), str(HOST_LOOP_SRC), "-o", str(tmp)]
    for d in libdirs:
        if d.is_dir():
            cmd += ["-L", str(d)]
    cmd += ["-lnpps", "-lnppc", "-lcudart", "-lcuda"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        return None
    os.replace(tmp, REF_HOST_LOOP)
    return REF_HOST_LOOP


def main(argv: list[str]) -> int:
    force = "--force" in argv
    print(build_oracle(force))
    print(build_refmath(force))
    print(build_ref_ptx(force))
    print(build_ref_host_loop(force))
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv[1:]))
