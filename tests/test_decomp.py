"""The decomposed path (sbp_decomp_*): one 2D wave grid as px x py subdomains
with ghost lines and the halo exchange fused into the stage kernels, the reference's
DMDA block decomposition with its VecScatter ghost update on one GPU.

CPU: descriptions the path does not take are rejected before any device work.
GPU: RHS and RK4 against the oracle (1e-12, norm-wise relative, the bar of the
single-grid parity tests) and against the single-grid context (1e-12), for
decompositions with uneven subdomains, orders 2/4/6, free-surface and
characteristic SAT (the oracle's characteristic SAT for rho = K = 1 is its
variable-coefficient problem with unit fields)."""
import ctypes as C

import numpy as np
import pytest

import oracle as O


def relerr(a, b):
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


def _desc(sbp, order, nx, ny, precision=None, problem=None):
    return sbp.Desc(sbp.WAVE_HOM_2D if problem is None else problem, order, 0,
                    sbp.FP64 if precision is None else precision, nx, ny, (C.c_double * 2)(-1.0, -1.0),
                    (C.c_double * 2)(1.0, 1.0), 0.0, 0.0, None, None, None, 0, 1, -1.0, 1.0)


@pytest.mark.parametrize("case", [(4, 20, 20, 4, 1, -1), (6, 40, 17, 2, 2, -1), (4, 30, 30, 2, 2, -4, "fp32"),
                                  (4, 30, 30, 2, 2, -4, "adv"), (4, 7, 30, 1, 1, -1), (6, 40, 11, 1, 1, -1)],
                         ids=["too_narrow_x", "too_narrow_y", "fp32", "other_problem", "below_min_points_x",
                              "below_min_points_y"])
def test_decomp_rejects_unsupported_descriptions(sbp, case):
    order, nx, ny, px, py, code = case[:6]
    kw = {}
    if len(case) > 6 and case[6] == "fp32":
        kw["precision"] = sbp.FP32
    if len(case) > 6 and case[6] == "adv":
        kw["problem"] = sbp.ADVECTION_2D
    L = sbp.load()
    h = C.c_void_p()
    assert L.sbp_decomp_create(C.byref(_desc(sbp, order, nx, ny, **kw)), px, py, C.byref(h)) == code
    assert not h.value
    assert L.sbp_decomp_last_error(None)  # says why


@pytest.mark.gpu
def test_decomp_rejects_unknown_where(sbp):
    """A `where` that is neither SBP_HOST nor SBP_DEVICE is refused before any copy."""
    L = sbp.load()
    v = np.zeros(3 * 20 * 20)
    with sbp.Decomp(4, 20, 20, 2, 2) as dec:
        assert L.sbp_decomp_set_state(dec._h, v.ctypes.data, 7) == sbp.ERR_INVALID
        assert L.sbp_decomp_get_state(dec._h, v.ctypes.data, 7) == sbp.ERR_INVALID
        assert L.sbp_decomp_rhs(dec._h, v.ctypes.data, v.ctypes.data, 7) == sbp.ERR_INVALID
        assert b"where" in L.sbp_decomp_last_error(dec._h)
        dec.set_state(v)  # still usable


CASES = [(2, 37, 29, 2, 3), (4, 40, 40, 4, 4), (4, 65, 33, 3, 2), (6, 27, 60, 1, 5), (6, 50, 41, 2, 2), (4, 33, 33, 1, 1)]
IDS = ["o2_37x29_2x3", "o4_40x40_4x4", "o4_65x33_3x2", "o6_27x60_1x5", "o6_50x41_2x2", "o4_33x33_1x1"]


def _oracle_problem(order, nx, ny, char):
    if char:
        ones = np.ones(nx * ny)
        return O.Problem(O.WAVE_VAR_2D, order, nx, ny, rho=ones, K=ones, bc=O.BC_CHARACTERISTIC)
    return O.Problem(O.WAVE_HOM_2D, order, nx, ny)


@pytest.mark.gpu
@pytest.mark.parametrize("char", [False, True], ids=["free_surface", "characteristic"])
@pytest.mark.parametrize("case", CASES, ids=IDS)
def test_decomp_rhs_matches_oracle(sbp, port, case, char):
    order, nx, ny, px, py = case
    bc = sbp.BC_CHARACTERISTIC if char else sbp.BC_REFERENCE
    src = np.random.default_rng(order + px + 7 * py).standard_normal(3 * nx * ny)
    with sbp.Decomp(order, nx, ny, px, py, bc=bc) as dec:
        got = dec.rhs(src)
    assert relerr(got, port.rhs(_oracle_problem(order, nx, ny, char), src)) < 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("char", [False, True], ids=["free_surface", "characteristic"])
@pytest.mark.parametrize("case", CASES, ids=IDS)
def test_decomp_rk4_matches_oracle_and_single_grid(sbp, port, case, char):
    order, nx, ny, px, py = case
    bc = sbp.BC_CHARACTERISTIC if char else sbp.BC_REFERENCE
    v0 = port.init_wave_pulse(nx, ny, 0.1, -0.2, 0.3, 1.0)
    v0 = v0 + 0.05 * np.random.default_rng(3).standard_normal(v0.size)
    dt = 0.2 * 2.0 / (max(nx, ny) - 1)
    with sbp.Decomp(order, nx, ny, px, py, bc=bc) as dec:
        got = dec.rk4(v0, dt, 9)
    ref = port.rk4(_oracle_problem(order, nx, ny, char), v0, 0.0, dt, 9)
    assert relerr(got, ref) < 1e-12
    with sbp.Context(sbp.WAVE_HOM_2D, order, nx, ny, bc=bc) as c:
        single = c.rk4(v0, 0.0, dt, 9)
    assert relerr(got, single) < 1e-12


@pytest.mark.gpu
def test_decomp_graphs_reused_across_chunk_lengths_and_time_steps(sbp):
    """One context runs 57 steps (a 50-step and a 7-step graph), then 7 steps at another dt
    (the graphs are dropped and recaptured), then 57 steps again: the repeated run reproduces
    the first bit for bit, and each run matches the single grid to 1e-12."""
    order, nx, ny, px, py = 4, 40, 40, 2, 2
    bc = sbp.BC_CHARACTERISTIC
    v0 = np.random.default_rng(11).standard_normal(3 * nx * ny)
    dt = 0.2 * 2.0 / (nx - 1)
    with sbp.Decomp(order, nx, ny, px, py, bc=bc) as dec:
        a = dec.rk4(v0, dt, 57)
        b = dec.rk4(v0, 0.5 * dt, 7)
        c = dec.rk4(v0, dt, 57)
    assert np.array_equal(a, c)
    with sbp.Context(sbp.WAVE_HOM_2D, order, nx, ny, bc=bc) as s:
        assert relerr(a, s.rk4(v0, 0.0, dt, 57)) < 1e-12
        assert relerr(b, s.rk4(v0, 0.0, 0.5 * dt, 7)) < 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("case", [(4, 1024, 1024, 8, 8), (6, 1000, 1030, 3, 5), (2, 1024, 1024, 2, 1)],
                         ids=["o4_1024_8x8", "o6_1000x1030_3x5", "o2_1024_2x1"])
def test_decomp_production_size_matches_single_grid_and_oracle(sbp, port, case):
    """At 1024^2 every CTA walks many tiles of several subdomains: the tile-geometry slots, the
    exchange queue's slot reuse and barrier phases, and the dynamic tile queue are all exercised.
    One RHS against the oracle, and 57 RK4 steps (across a 50-step graph chunk) against the single
    grid, characteristic SAT, 1e-12 norm-wise relative."""
    order, nx, ny, px, py = case
    bc = sbp.BC_CHARACTERISTIC
    rng = np.random.default_rng(order * 100 + px)
    src = rng.standard_normal(3 * nx * ny)
    v0 = port.init_wave_pulse(nx, ny, 0.1, -0.2, 0.3, 1.0) + 0.01 * rng.standard_normal(3 * nx * ny)
    dt = 0.2 * 2.0 / (max(nx, ny) - 1)
    with sbp.Decomp(order, nx, ny, px, py, bc=bc) as dec:
        got_rhs = dec.rhs(src)
        got = dec.rk4(v0, dt, 57)
    assert relerr(got_rhs, port.rhs(_oracle_problem(order, nx, ny, True), src)) < 1e-12
    with sbp.Context(sbp.WAVE_HOM_2D, order, nx, ny, bc=bc) as c:
        single = c.rk4(v0, 0.0, dt, 57)
    assert relerr(got, single) < 1e-12
