"""The C-ABI library loads and exports every entry point declared in include/vivsim_gb300.h.

Runs without a GPU: loading the library makes no CUDA call.
"""

import os
import re

import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "vivsim_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\s*\*?\s*(vs_[a-z_0-9]+)\s*\(", text, flags=re.M)))


@pytest.fixture(scope="module")
def lib():
    from vivsim_gb300 import _build, _lib
    if not os.path.exists(_build.lib_path()):
        _build.build()
    return _lib.load()


def test_header_declares_entry_points():
    names = declared_functions()
    assert "vs_step" in names and "vs_ib_mdf" in names and len(names) >= 35


def test_every_declared_symbol_is_exported(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_matches_header(lib):
    from vivsim_gb300 import _lib
    assert set(_lib.exported_symbols()) <= set(declared_functions())


def test_status_strings(lib):
    assert lib.vs_status_string(0) == b"ok"
    assert lib.vs_version() >= 100


def test_invalid_arguments_return_status_without_gpu(lib):
    # argument validation happens before any CUDA call
    import ctypes as C
    rc = lib.vs_streaming(7, 0, None, None, 4, 4, 1, None)
    assert rc == 1
    assert b"distinct" in lib.vs_last_error() or b"q must" in lib.vs_last_error()
    rc = lib.vs_collision(9, 5, 0, C.c_void_p(8), C.c_void_p(8), 1.0, C.c_void_p(8), 4, None)
    assert rc == 1 and b"dtype" in lib.vs_last_error()


def test_refinement_and_watchdog_validation_without_gpu(lib):
    """Shape and argument checks of the refinement transfers, the watchdog scan and the
    self-test run before any CUDA call (the pointers below are never dereferenced)."""
    import ctypes as C
    p = C.c_void_p(64)
    # fine extent 12 along the interface onto a coarse extent of 5: the reference's shape error
    assert lib.vs_fine_to_coarse(0, p, 5, 12, p, 7, 5, 0, None) == 1
    assert b"does not match" in lib.vs_last_error()
    assert lib.vs_coarse_to_fine(0, p, 7, 4, p, 5, 12, 0, None) == 1
    assert b"does not match" in lib.vs_last_error()
    assert lib.vs_fine_to_coarse(0, p, 1, 12, p, 7, 6, 0, None) == 1  # one fine node across
    assert lib.vs_fine_to_coarse(0, p, 5, 12, p, 7, 6, 7, None) == 1  # no such direction
    assert b"dir must be" in lib.vs_last_error()
    assert lib.vs_check_finite(0, None, 10, p, None) == 1
    assert lib.vs_selftest_bounded_wait(0, p, None) == 1
    assert lib.vs_selftest_bounded_wait(1 << 21, p, None) == 1


def test_run_form_and_batch_shape_queries_without_gpu(lib):
    """vs_run_persistent answers without a CUDA call (0 for no plan or fewer than two steps),
    and the batch's nodes-per-thread setter validates its arguments first."""
    import ctypes as C
    assert lib.vs_run_persistent(None, None, 100) == 0
    assert lib.vs_run_persistent(C.c_void_p(64), None, 1) == 0
    assert lib.vs_batch_set_nodes_per_thread(None, 2) == 1
    assert b"null plan" in lib.vs_last_error()
    assert lib.vs_batch_set_nodes_per_thread(C.c_void_p(64), 3) == 1
    assert b"1 or 2" in lib.vs_last_error()
    assert lib.vs_lattice_set_run_form(None, 1) == 1
    assert lib.vs_lattice_set_run_form(C.c_void_p(64), 2) == 1
    assert b"VS_RUN_STEPS or VS_RUN_PERSISTENT" in lib.vs_last_error()


def test_plan_validation_without_gpu(lib):
    """A lattice plan is validated before it allocates: bad wall combinations raise."""
    from vivsim_gb300 import _lib as V
    from vivsim_gb300 import solver as S
    with pytest.raises(V.VivsimError, match="characteristic wall is imposed by NEE"):
        S.LatticeStep(9, (16, 16), "bgk", 1.0, boundaries=[S.boundary("bounce_back", "right", mode="characteristic")])
    with pytest.raises(V.VivsimError, match="too small"):
        S.LatticeStep(9, (3, 16), "bgk", 1.0)


def test_jax_adapter_needs_jax():
    """The XLA FFI adapter imports without JAX and refuses to run without it."""
    from vivsim_gb300 import jax_ffi
    try:
        import jax  # noqa: F401
        pytest.skip("JAX is installed here")
    except ImportError:
        pass
    with pytest.raises(ImportError):
        jax_ffi.lbm.collision_kbc(None, None, 1.7)
    with pytest.raises(ImportError):
        jax_ffi.ib.interpolate(None, None, None)


def test_xla_ffi_handlers_match_their_bindings():
    """Every custom-call target of jax_ffi has a handler symbol in xla/vs_xla_ffi.cc, every
    handler is registered, and the handlers compile (g++ -fsyntax-only) against a
    stand-in FFI header that checks each handler's parameters against its binding."""
    import shutil
    import subprocess
    from vivsim_gb300 import jax_ffi
    src = os.path.join(ROOT, "vivsim_gb300", "xla", "vs_xla_ffi.cc")
    symbols = set(re.findall(r"XLA_FFI_DEFINE_HANDLER_SYMBOL\((\w+),", open(src).read()))
    assert symbols == set(jax_ffi.TARGETS.values())
    if shutil.which("g++") is None:
        pytest.skip("no g++")
    cuda_inc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")
    cmd = ["g++", "-std=c++17", "-fsyntax-only", "-I", os.path.join(ROOT, "tests", "c_host", "xla_ffi_standin"),
           "-I", os.path.join(ROOT, "include"), "-I", cuda_inc, src]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]


def test_plain_c_host(tmp_path):
    """A C99 program includes the header, links the library and runs its argument checks
    (tests/c_host/abi_check.c; no GPU needed)."""
    import shutil
    import subprocess
    from vivsim_gb300 import _build
    cc = shutil.which("gcc")
    if cc is None:
        pytest.skip("no C compiler")
    lib = _build.lib_path()
    if not os.path.exists(lib):
        _build.build()
    exe = str(tmp_path / "abi_check")
    subprocess.run([cc, "-std=c99", "-Wall", os.path.join(ROOT, "tests", "c_host", "abi_check.c"), "-o", exe,
                    "-I", os.path.join(ROOT, "include"), "-L", os.path.dirname(lib), "-lvivsim_gb300",
                    "-Wl,-rpath," + os.path.dirname(lib)], check=True)
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr


def test_solver_rejects_unknown_names():
    """Unknown schemes, wall modes, faces, collisions and forcings raise ValueError (as the
    reference raises on an unknown face) before anything is allocated."""
    from vivsim_gb300 import solver as S
    for bad in (S.boundary("neex", "left"), S.boundary("nee", "leftish"), S.boundary("nee", "left", mode="fast")):
        with pytest.raises(ValueError):
            S.LatticeStep(9, (16, 16), "bgk", 1.0, boundaries=[bad])
    with pytest.raises(ValueError):
        S.LatticeStep(9, (16, 16), "lbgk", 1.0)
    with pytest.raises(ValueError):
        S.LatticeStep(9, (16, 16), "bgk", 1.0, forcing="shan_chen")
    with pytest.raises(ValueError):
        S.LatticeStep(9, (16, 16), "bgk", 1.0, variant="fastest")
    with pytest.raises(ValueError):  # a boundary without its face
        S.LatticeStep(9, (16, 16), "bgk", 1.0, boundaries=[dict(kind="nee", mode="given")])
