"""The C ABI library: loads without a GPU, exports every symbol that
include/sbpgpu.h declares, and rejects bad descriptions before touching CUDA."""
import ctypes as C
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared_functions():
    text = open(os.path.join(ROOT, "include", "sbpgpu.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(sbp_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_expected_surface():
    names = _declared_functions()
    for required in ("sbp_create", "sbp_destroy", "sbp_rhs", "sbp_apply", "sbp_ts_rk4", "sbp_rk4",
                     "sbp_error_norms", "sbp_hnorm", "sbp_last_error"):
        assert required in names


def test_library_exports_every_declared_symbol(sbp):
    lib = sbp.load()
    for name in _declared_functions():
        assert hasattr(lib, name), f"{name} declared in include/sbpgpu.h but not exported"
    assert set(_declared_functions()) == set(sbp.EXPORTS)


def test_step_rule_without_gpu(sbp):
    assert sbp.rk4_nsteps(1.8, 0.001) == (1800, 0.001)
    n, dt = sbp.rk4_nsteps(1.0, 0.3)
    assert n == 3 and abs(dt - 1.0 / 3) < 1e-15
    d = C.c_double(-1.0)
    assert sbp.load().sbp_rk4_nsteps(1.0, C.byref(d)) == sbp.ERR_INVALID


@pytest.mark.parametrize("kw,msg", [
    (dict(problem=9, order=4, nx=33, ny=33), "unknown problem"),
    (dict(problem=1, order=5, nx=33, ny=33), "order"),
    (dict(problem=1, order=6, nx=11, ny=33), "minimum"),
    (dict(problem=1, order=4, nx=33, ny=7), "minimum"),
    (dict(problem=4, order=4, nx=33, ny=33, bc=1), "characteristic"),
    (dict(problem=2, order=4, nx=33, ny=33, precision=1), "FP64 only"),
    (dict(problem=6, order=4, nx=33, ny=33), "rho and K"),
])
def test_invalid_descriptions_rejected(sbp, kw, msg):
    problem, order, nx, ny = kw.pop("problem"), kw.pop("order"), kw.pop("nx"), kw.pop("ny")
    with pytest.raises(sbp.SbpError) as ei:
        sbp.Context(problem, order, nx, ny, **kw)
    assert ei.value.code == sbp.ERR_INVALID
    assert msg in str(ei.value)


def test_null_context_calls_fail_cleanly(sbp):
    lib = sbp.load()
    assert lib.sbp_destroy(None) == sbp.ERR_INVALID
    assert lib.sbp_rhs(None, 0.0, None, None, 0) == sbp.ERR_INVALID
    assert lib.sbp_dofs(None) == sbp.ERR_INVALID
