"""CPU tests of the C-ABI boundary and the host-side mirror of the reference's
Python interface (no compute: no GPU here)."""
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
HEADERS = sorted((ROOT / "include").glob("*.h"))


def _declared_c_functions():
    names = set()
    for h in HEADERS:
        text = h.read_text()
        if 'extern "C"' not in text:
            continue
        body = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        body = re.sub(r"//[^\n]*", "", body)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(tdc_\w+)\s*\(", body, flags=re.M):
            names.add(m.group(1))
    return names


def test_library_builds_and_exports_every_declared_symbol(engine_lib):
    declared = _declared_c_functions()
    assert "tdc_processor_start" in declared and "tdc_processor_focus_device" in declared
    for name in sorted(declared):
        assert hasattr(engine_lib, name), f"{name} declared in include/ but not exported"
    out = subprocess.run(["nm", "-D", "--defined-only", engine_lib._name], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (tdc_\w+)", out))
    assert declared <= exported
    assert engine_lib.tdc_abi_version() == 1


def test_c_abi_header_compiles_as_c99():
    """include/tdc_gb300.h is a C header (what a cgo / JNI / ctypes binding includes): it must
    compile as plain C99, not only as C++."""
    r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-Werror", "-fsyntax-only", "-x", "c",
                        str(ROOT / "include" / "tdc_gb300.h")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_binding_signatures_cover_the_header():
    import _tdc_capi

    bound = {name for name, _, _ in _tdc_capi.SIGNATURES}
    assert _declared_c_functions() <= bound


def test_library_is_sm103a_only(engine_lib):
    log = (ROOT / "sarlab-tdc_gb300" / "_build" / "ptxas.log").read_text()
    assert "sm_103a" in log
    assert "spill stores" in log
    # no kernel spills registers
    assert not re.search(r"[1-9]\d* bytes spill stores", log)


def test_error_mapping(engine_lib):
    import _tdc_capi as L

    L.check(0)
    with pytest.raises(ValueError):
        L.check(L.TDC_ERR_INVALID_ARGUMENT)
    with pytest.raises(RuntimeError):
        L.check(L.TDC_ERR_CUDA)
    with pytest.raises(RuntimeError):
        L.check(L.TDC_ERR_TIMEOUT)
    with pytest.raises(MemoryError):
        L.check(L.TDC_ERR_NO_MEMORY)


def test_null_processor_is_rejected(engine_lib):
    import _tdc_capi as L

    rc = engine_lib.tdc_processor_start(None, 0.0, 1.0, 0, 0, 1)
    assert rc == L.TDC_ERR_INVALID_ARGUMENT
    assert "null processor" in L.last_error()
    assert engine_lib.tdc_processor_image_buffer(None) is None


def _unbound_processor():
    import _sarlabtdc

    p = object.__new__(_sarlabtdc.TdcProcessor)
    p._h = None
    return p


def _args(C=4, S=8):
    return dict(rawData=np.zeros((C, S), np.complex64), priTimes=np.zeros(C, np.float32),
                sampleTimes=np.zeros(S, np.float32), position=np.zeros((C, S, 3), np.float32),
                velocity=np.zeros((C, S, 3), np.float32), attitude=np.zeros((C, S, 4), np.float32),
                modRate=1.0, startFreq=1.0, bodyBoresight=np.zeros(3, np.float32))


@pytest.mark.parametrize("key,bad,msg", [
    ("rawData", np.zeros(8, np.complex64), "rawData must be 2D"),
    ("priTimes", np.zeros((4, 1), np.float32), "priTimes must be 1D"),
    ("sampleTimes", np.zeros((8, 1), np.float32), "sampleTimes must be 1D"),
    ("position", np.zeros((4, 8), np.float32), "position must be 3D"),
    ("velocity", np.zeros((4, 8), np.float32), "velocity must be 3D"),
    ("attitude", np.zeros((4, 8), np.float32), "attitude must be 3D"),
    ("bodyBoresight", np.zeros((3, 1), np.float32), "bodyBoresight must be 1D"),
    ("priTimes", np.zeros(5, np.float32), "priTimes shape is incorrect"),
    ("sampleTimes", np.zeros(7, np.float32), "sampleTimes shape is incorrect"),
    ("position", np.zeros((4, 8, 4), np.float32), "position shape is incorrect"),
    ("velocity", np.zeros((4, 7, 3), np.float32), "velocity shape is incorrect"),
    ("attitude", np.zeros((4, 8, 3), np.float32), "attitude shape is incorrect"),
    ("bodyBoresight", np.zeros(4, np.float32), "bodyBoresight shape is incorrect"),
])
def test_setrawdata_shape_checks_mirror_the_reference(key, bad, msg):
    """tdcprocessor_wrapper.cpp:54-113: the same checks, order and messages."""
    p = _unbound_processor()
    a = _args()
    a[key] = bad
    with pytest.raises(RuntimeError, match=msg):
        p.setRawData(*a.values())


def test_setfocusgrid_shape_checks():
    p = _unbound_processor()
    with pytest.raises(RuntimeError, match="focusGrid must be 3D"):
        p.setFocusGrid(np.zeros((4, 3), np.float32))
    with pytest.raises(RuntimeError, match="focusGrid shape is incorrect"):
        p.setFocusGrid(np.zeros((4, 4, 2), np.float32))


def test_setrawdata_positional_only_like_pybind():
    import _sarlabtdc

    p = _unbound_processor()
    with pytest.raises(TypeError):
        p.setRawData(**_args())
    assert _sarlabtdc.TdcProcessor.start.__defaults__ == (True,)


def test_product_never_touches_the_oracle():
    pkg = ROOT / "sarlab-tdc_gb300"
    for f in list(pkg.rglob("*.py")) + list(pkg.rglob("*.cu")) + list(pkg.rglob("*.cpp")) + \
            list(pkg.rglob("*.h")) + list(pkg.rglob("*.cuh")):
        text = f.read_text()
        assert not re.search(r"(import\s+oracle|from\s+oracle|libtdc_oracle|libtdc_refmath|oracle/)", text), \
            f"{f} imports or loads the oracle"


def test_no_closed_copy_calls_in_sources():
    # one cudaMemcpyAsync per copy; batch-copy entry points are not used anywhere
    pkg = ROOT / "sarlab-tdc_gb300" / "csrc"
    for f in pkg.iterdir():
        assert "BatchAsync" not in f.read_text()


def _cpp_build(tmp_path):
    exe = tmp_path / "tdcprocessor_smoke"
    lib_dir = ROOT / "sarlab-tdc_gb300"
    cmd = ["g++", "-std=c++17", "-O1", "-I", str(ROOT / "include"), "-I", "/usr/local/cuda/include",
           str(ROOT / "tests" / "cpp" / "tdcprocessor_smoke.cpp"), "-L", str(lib_dir), "-ltdc_gb300",
           f"-Wl,-rpath,{lib_dir}", "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_cpp_header_compiles_and_links(engine_lib, tmp_path):
    """include/tdcprocessor.h is a drop-in for the reference's class: a tdctest-shaped program builds."""
    assert _cpp_build(tmp_path).exists()


def test_wait_timeout_selftest_rejects_bad_limits_before_any_cuda_call(engine_lib):
    import ctypes as C

    import _tdc_capi

    flag = C.c_int(7)
    for limit in (0, -5, 3_000_000):
        assert engine_lib.tdc_selftest_wait_timeout(0, limit, C.byref(flag), None) == _tdc_capi.TDC_ERR_INVALID_ARGUMENT
    assert engine_lib.tdc_selftest_wait_timeout(0, 1000, None, None) == _tdc_capi.TDC_ERR_INVALID_ARGUMENT
    assert flag.value == 7


def test_device_buffers_are_checked_before_any_kernel_writes_them():
    """focusDevice / adjointDevice / setChirpOffsetsDevice validate a CUDA array's dtype,
    contiguity and size (the kernels write every element) -- checked here with fake
    __cuda_array_interface__ objects, no GPU needed."""
    import _sarlabtdc as S

    class Fake:
        def __init__(self, shape, typestr, strides=None, ptr=0x1000):
            self.__cuda_array_interface__ = {"shape": shape, "typestr": typestr, "strides": strides,
                                             "data": (ptr, False), "version": 3}

    assert S._device_buffer(Fake((100,), "<c8"), "complex64", 100, "image") == 0x1000
    assert S._device_buffer(Fake((10, 10), "<c8", strides=(80, 8)), "complex64", 100, "image") == 0x1000
    assert S._device_buffer(0x2000, "complex64", 100, "image") == 0x2000
    with pytest.raises(ValueError):
        S._device_buffer(Fake((99,), "<c8"), "complex64", 100, "image")          # too small
    with pytest.raises(ValueError):
        S._device_buffer(Fake((100,), "<c16"), "complex64", 100, "image")        # wrong dtype
    with pytest.raises(ValueError):
        S._device_buffer(Fake((100,), "<c8", strides=(16,)), "complex64", 100, "image")  # strided
    with pytest.raises(ValueError):
        S._device_buffer(np.zeros(100, np.complex64), "complex64", 100, "image")  # host array
    assert S._device_buffer(Fake((7, 3), "<f8"), "float64", 21, "offsets") == 0x1000


def test_kernels_compile_without_register_spills(engine_lib):
    """ptxas resource report of the build (sarlab-tdc_gb300/_build/ptxas.log): every
    focus (including the anchored-range kernel), adjoint and general-kernel instance fits
    its registers (no spill stores or loads, <= 168 registers for 3 CTAs of 128 threads), so
    a change that pushes a hot loop into local memory fails here, before it reaches a GPU."""
    import re

    log = (ROOT / "sarlab-tdc_gb300" / "_build" / "ptxas.log").read_text()
    blocks = re.split(r"ptxas info\s*: Compiling entry function '", log)[1:]
    seen = {}
    for b in blocks:
        name = b.split("'", 1)[0]
        m_sp = re.search(r"(\d+) bytes spill stores, (\d+) bytes spill loads", b)
        m_rg = re.search(r"Used (\d+) registers", b)
        assert m_sp and m_rg, name
        seen[name] = (int(m_sp.group(1)), int(m_sp.group(2)), int(m_rg.group(1)))
    hot = {n: v for n, v in seen.items()
           if any(k in n for k in ("focus_fp32", "focus_general", "focus_motion", "adjoint_fp32_kernel",
                                   "focus_fp64"))}
    # 4 bulk + 1 anchored + 2 segmented + 7 general + 2 smooth-motion + 2 FP64 + 2 adjoint instances
    assert len(hot) >= 20, sorted(hot)
    assert any("focus_fp32_anchored_kernel" in n for n in hot)
    for name, (st, ld, regs) in hot.items():
        assert st == 0 and ld == 0, f"{name}: {st} B spill stores, {ld} B spill loads"
        assert regs <= 168 or "focus_fp64" in name, f"{name}: {regs} registers"


def test_binding_constants_match_the_header():
    """The Python binding's copies of the header's size limits are the header's values."""
    import _tdc_capi

    text = (ROOT / "include" / "tdc_gb300.h").read_text()
    scratch = re.search(r"#define TDC_NOALLOC_SCRATCH_BYTES \((\d+)u << (\d+)\)", text)
    assert scratch and int(scratch.group(1)) << int(scratch.group(2)) == _tdc_capi.NOALLOC_SCRATCH_BYTES
    max_s = re.search(r"#define TDC_NOALLOC_MAX_SAMPLES (\d+)", text)
    assert max_s and int(max_s.group(1)) == _tdc_capi.NOALLOC_MAX_SAMPLES


def test_bench_command_line_parses():
    """bench.py loads and lists its options without a GPU (its arms and configs)."""
    import sys

    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--help"], capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    for opt in ("--gpus", "--steps", "--warmup", "--impl", "--config"):
        assert opt in r.stdout
