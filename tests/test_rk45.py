"""Adaptive Runge-Kutta-Fehlberg 4(5) (the reference's ts_rk45,
code/src/time_stepping/ts_rk.cpp:41-52, PETSc TSRK5F + TSADAPTBASIC).

CPU: the oracle's restatement (orc_rk45) against properties of the method:
5th-order convergence at fixed steps, agreement with a finely stepped RK4 at
tight tolerances, error falling with the tolerance, recovery from rejected
attempts, landing on t_end exactly, and the step limit.

GPU: sbp_rk45_resident / sbp_ts_rk45 (graph-captured attempts, device-side
controller) against orc_rk45 on the same inputs.
- Fixed steps (every attempt accepted, dt_max = the step): the tableau and the
  stage arithmetic, at the RK4 parity bar (1e-12 relative, max norm).
- Adaptive runs: the accepted and rejected counts and the final time are
  equal; the state agrees within max(1e-10, 100 s), s = the oracle's own
  change when its initial state is perturbed at 1e-16 relative. The error
  estimate is the difference of two nearly equal solutions, so last-bit
  differences (the RHS's FMA contraction, the error sum's order) shift the
  step sequence; s measures how far that moves the answer (2e-9 to 5e-8 on
  some of these cases).
"""
import numpy as np
import pytest

import oracle as O

TOL = 1e-10


def relerr(a, b):
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


def _adv1d(n, order=4):
    pb = O.Problem(O.ADVECTION_1D, order, n, a=1.0)
    x = np.linspace(-1, 1, n)
    return pb, np.exp(-(x / 0.2) ** 2)


def _pulse2d(nx, ny, dofs=3, w=0.2):
    x = np.linspace(-1, 1, nx)
    y = np.linspace(-1, 1, ny)
    v = np.zeros((ny, nx, dofs))
    v[:, :, dofs - 1] = np.exp(-((x[None, :] - 0.1) ** 2 + (y[:, None] + 0.05) ** 2) / w**2)
    return v.ravel()


def test_rk45_lands_on_t_end_and_matches_fine_rk4(port):
    pb, v0 = _adv1d(101)
    v, st = port.rk45(pb, v0, 0.0, 0.5, 0.01, atol=1e-11, rtol=1e-11)
    assert st["status"] == 0 and st["t"] == 0.5 and st["accepted"] > 10
    fine = port.rk4(pb, v0, 0.0, 0.5 / 4000, 4000)
    assert relerr(v, fine) < 1e-8


def test_rk45_error_falls_with_tolerance(port):
    pb, v0 = _adv1d(101)
    ref, _ = port.rk45(pb, v0, 0.0, 0.5, 0.01, atol=1e-12, rtol=1e-12)
    errs, steps = [], []
    for tol in (1e-3, 1e-5, 1e-7):
        v, st = port.rk45(pb, v0, 0.0, 0.5, 0.01, atol=tol, rtol=tol)
        errs.append(relerr(v, ref))
        steps.append(st["accepted"])
    assert errs[0] > errs[1] > errs[2]
    assert steps[0] < steps[1] < steps[2]


def test_rk45_fifth_order_at_fixed_steps(port):
    """With tolerances so loose that every attempt is accepted and dt_max = h, RKF45 is the
    fixed-step 5th-order Fehlberg method: halving h divides the error by about 2^5."""
    pb, v0 = _adv1d(51, order=2)
    t_end = 0.2
    ref, _ = port.rk45(pb, v0, 0.0, t_end, 1e-3, atol=1e-13, rtol=1e-13)
    errs = []
    for m in (16, 32):
        h = t_end / m
        v, st = port.rk45(pb, v0, 0.0, t_end, h, atol=1e6, rtol=0.0, dt_max=h)
        assert st["rejected"] == 0 and st["accepted"] == m and st["t"] == t_end
        errs.append(relerr(v, ref))
    assert 20 < errs[0] / errs[1] < 45


def test_rk45_recovers_from_rejected_attempts(port):
    pb, v0 = _adv1d(101)
    v, st = port.rk45(pb, v0, 0.0, 0.3, 0.5)  # the first attempt spans most of the interval
    assert st["rejected"] >= 1 and st["status"] == 0 and st["t"] == 0.3
    ref, _ = port.rk45(pb, v0, 0.0, 0.3, 0.01, atol=1e-11, rtol=1e-11)
    assert relerr(v, ref) < 1e-2


def test_rk45_step_limit(port):
    pb, v0 = _adv1d(101)
    _, st = port.rk45(pb, v0, 0.0, 1.0, 1e-3, max_steps=3)
    assert st["status"] == 1 and st["accepted"] + st["rejected"] == 3 and st["t"] < 1.0


# ---------------------------------------------------------------- GPU parity
CASES = [
    # (name, problem, order, nx, ny, extra kwargs, t_end, dt0)
    ("adv1d_o2", O.ADVECTION_1D, 2, 201, 1, {}, 0.4, 0.01),
    ("adv1d_o4", O.ADVECTION_1D, 4, 201, 1, {}, 0.4, 0.01),
    ("adv1d_o6", O.ADVECTION_1D, 6, 201, 1, {}, 0.4, 0.01),
    ("adv2d_o4", O.ADVECTION_2D, 4, 64, 64, {"a": 1.0, "b": -0.5}, 0.3, 0.01),
    ("refl_o4", O.REFLECTION_1D, 4, 101, 1, {}, 0.3, 0.01),
    ("wave_hom_o2", O.WAVE_HOM_2D, 2, 65, 65, {}, 0.3, 0.01),
    ("wave_hom_o4", O.WAVE_HOM_2D, 4, 65, 65, {}, 0.3, 0.01),
    ("wave_hom_o6", O.WAVE_HOM_2D, 6, 65, 65, {}, 0.3, 0.01),
    ("wave_mms_o4", O.WAVE_MMS_2D, 4, 41, 41, {}, 0.2, 0.01),
    ("wave_var_char_o4", O.WAVE_VAR_2D, 4, 70, 45, {"char": True}, 0.3, 0.01),
    ("wave_2block_o4", O.WAVE_2BLOCK_2D, 4, 49, 66, {"char": True}, 0.3, 0.01),
]


def _case_state(problem, nx, ny):
    if problem == O.ADVECTION_1D:
        return np.exp(-(np.linspace(-1, 1, nx) / 0.2) ** 2)
    if problem == O.REFLECTION_1D:
        x = np.linspace(-1, 1, nx)
        return np.stack([np.exp(-(x / 0.2) ** 2), 0.5 * np.exp(-((x - 0.2) / 0.15) ** 2)], axis=1).ravel()
    if problem == O.ADVECTION_2D:
        return _pulse2d(nx, ny, 1)
    return _pulse2d(nx, ny, 3)


def _fields(nx, ny):
    x = np.linspace(-1, 1, nx)
    y = np.linspace(-1, 1, ny)
    X, Y = np.meshgrid(x, y)
    return (1.0 + 0.3 * np.sin(2 * X) * np.cos(Y)).ravel(), (1.2 + 0.4 * np.cos(X - 2 * Y)).ravel()


def _pair(sbp, problem, order, nx, ny, kw):
    ckw, okw = {}, {}
    if "a" in kw:
        ckw["a"] = okw["a"] = kw["a"]
        ckw["b"] = okw["b"] = kw["b"]
    if kw.get("char"):
        rho, K = _fields(nx, ny)
        ckw.update(rho=rho, K=K, bc=sbp.BC_CHARACTERISTIC)
        okw.update(rho=rho, K=K, bc=O.BC_CHARACTERISTIC)
    ctx = sbp.Context(problem, order, nx, ny, **ckw)
    pb = O.Problem(problem, order, nx, ny, **okw)
    return ctx, pb


def _sensitivity(port, pb, v0, t_end, dt0, **opts):
    """Relative change of the oracle's answer when v0 is perturbed at 1e-16 relative."""
    ref, _ = port.rk45(pb, v0, 0.0, t_end, dt0, **opts)
    v1 = v0 * (1.0 + 1e-16 * np.random.default_rng(0).standard_normal(v0.size))
    out, _ = port.rk45(pb, v1, 0.0, t_end, dt0, **opts)
    return relerr(out, ref)


@pytest.mark.gpu
@pytest.mark.parametrize("name,problem,order,nx,ny,kw,t_end,dt0", CASES, ids=[c[0] for c in CASES])
def test_gpu_rk45_fixed_steps_match_oracle(sbp, port, name, problem, order, nx, ny, kw, t_end, dt0):
    ctx, pb = _pair(sbp, problem, order, nx, ny, kw)
    v0 = _case_state(problem, nx, ny)
    h = 0.25 * dt0
    fixed = dict(atol=1e6, rtol=0.0, dt_max=h)
    with ctx:
        ctx.set_state(v0)
        st = ctx.rk45_resident(0.0, 0.5 * t_end, h, **fixed)
        got = ctx.get_state()
    ref, rst = port.rk45(pb, v0, 0.0, 0.5 * t_end, h, **fixed)
    assert st["rejected"] == rst["rejected"] == 0 and st["accepted"] == rst["accepted"]
    assert relerr(got, ref) < 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("name,problem,order,nx,ny,kw,t_end,dt0", CASES, ids=[c[0] for c in CASES])
def test_gpu_rk45_matches_oracle(sbp, port, name, problem, order, nx, ny, kw, t_end, dt0):
    ctx, pb = _pair(sbp, problem, order, nx, ny, kw)
    v0 = _case_state(problem, nx, ny)
    with ctx:
        ctx.set_state(v0)
        st = ctx.rk45_resident(0.0, t_end, dt0)
        got = ctx.get_state()
    ref, rst = port.rk45(pb, v0, 0.0, t_end, dt0)
    assert (st["accepted"], st["rejected"], st["status"]) == (rst["accepted"], rst["rejected"], rst["status"])
    assert st["t"] == rst["t"] == t_end
    assert relerr(got, ref) < max(TOL, 100 * _sensitivity(port, pb, v0, t_end, dt0))


@pytest.mark.gpu
def test_gpu_rk45_rejections_tolerances_and_host_entry(sbp, port):
    ctx, pb = _pair(sbp, O.WAVE_HOM_2D, 4, 65, 65, {})
    v0 = _case_state(O.WAVE_HOM_2D, 65, 65)
    with ctx:
        # a first attempt far beyond the stable step: rejections, then recovery
        ctx.set_state(v0)
        st = ctx.rk45_resident(0.0, 0.25, 0.2, atol=1e-6, rtol=1e-6)
        got = ctx.get_state()
        ref, rst = port.rk45(pb, v0, 0.0, 0.25, 0.2, atol=1e-6, rtol=1e-6)
        assert st["rejected"] >= 1 and (st["accepted"], st["rejected"]) == (rst["accepted"], rst["rejected"])
        assert relerr(got, ref) < max(TOL, 100 * _sensitivity(port, pb, v0, 0.25, 0.2, atol=1e-6, rtol=1e-6))
        # the host-array entry point (ts_rk45: t from 0, default options)
        host = ctx.ts_rk45(v0, 0.25, 0.01)
        ref2, _ = port.rk45(pb, v0, 0.0, 0.25, 0.01)
        assert relerr(host, ref2) < max(TOL, 100 * _sensitivity(port, pb, v0, 0.25, 0.01))


@pytest.mark.gpu
def test_gpu_rk45_step_limit_and_unsupported(sbp, port):
    ctx, pb = _pair(sbp, O.ADVECTION_1D, 4, 201, 1, {})
    v0 = _case_state(O.ADVECTION_1D, 201, 1)
    with ctx:
        ctx.set_state(v0)
        st = ctx.rk45_resident(0.0, 1.0, 1e-3, check=False, max_steps=5)
        got = ctx.get_state()
    ref, rst = port.rk45(pb, v0, 0.0, 1.0, 1e-3, max_steps=5)
    assert st["rc"] == sbp.ERR_DIVERGED and st["status"] == rst["status"] == 1
    assert st["accepted"] + st["rejected"] == 5
    assert relerr(got, ref) < max(TOL, 100 * _sensitivity(port, pb, v0, 1.0, 1e-3, max_steps=5))
    with sbp.Context(O.WAVE_HOM_2D, 4, 33, 33, precision=sbp.FP32) as c32:
        c32.set_state(_case_state(O.WAVE_HOM_2D, 33, 33))
        with pytest.raises(sbp.SbpError):
            c32.rk45_resident(0.0, 0.1, 0.01)


@pytest.mark.gpu
@pytest.mark.parametrize("name,problem,order,nx,ny,kw,t_end,dt0", [CASES[1], CASES[4], CASES[6], CASES[10]],
                         ids=[CASES[i][0] for i in (1, 4, 6, 10)])
def test_gpu_rk45_error_norm_of_one_attempt(sbp, port, name, problem, order, nx, ny, kw, t_end, dt0):
    """The weighted error of a single attempt (its 1/tol from a refined FP32 reciprocal, the
    sum in per-CTA partials) against the oracle's (FP64 division, sequential sum). Each
    difference u5 - u4 inherits the last-bit differences of the stage derivatives (a couple
    of ulps of u), which moves wlte by up to about 4 eps max|u| / tol; the rest must agree
    to 1e-13 relative (an FP32-accurate reciprocal would be off by about 1e-7)."""
    v0 = _case_state(problem, nx, ny)
    for tol in (1e-4, 1e-9):
        ctx, pb = _pair(sbp, problem, order, nx, ny, kw)
        with ctx:
            ctx.set_state(v0)
            st = ctx.rk45_resident(0.0, t_end, dt0, check=False, max_steps=1, atol=tol, rtol=tol)
        _, rst = port.rk45(pb, v0, 0.0, t_end, dt0, max_steps=1, atol=tol, rtol=tol)
        assert st["accepted"] + st["rejected"] == 1
        bound = 1e-13 * rst["wlte"] + 4 * np.finfo(float).eps * np.abs(v0).max() / tol
        assert abs(st["wlte"] - rst["wlte"]) <= bound
