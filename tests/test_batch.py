"""Batched form: every instance of a batch must evolve exactly as a
single-instance context of the same problem does (same per-point arithmetic),
for uneven sizes, orders, speeds and time steps, FP64 and FP32."""
import json
import os

import numpy as np
import pytest

import fields


def _instances(sbp, seed, count):
    rng = np.random.default_rng(seed)
    out = []
    for k in range(count):
        order = int(rng.choice([2, 4, 6]))
        nx = int(rng.integers(12, 150))
        ny = int(rng.integers(12, 150))
        c = float(rng.uniform(0.5, 2.0))
        h = min(2.0 / (nx - 1), 2.0 / (ny - 1))
        if k % 2 == 0:
            out.append(dict(problem=sbp.WAVE_HOM_2D, order=order, nx=nx, ny=ny, c=c, dt=0.2 * h / c,
                            bc=int(rng.integers(0, 2))))
        else:
            ang = rng.uniform(0, 2 * np.pi)
            out.append(dict(problem=sbp.ADVECTION_2D, order=order, nx=nx, ny=ny, a=c * np.cos(ang),
                            b=c * np.sin(ang), dt=0.2 * h / c))
    return out


def _state(d, seed):
    if d["problem"] == 1:
        x0, y0 = np.random.default_rng(seed).uniform(-0.5, 0.5, 2)
        return fields.gaussian_pulse(d["nx"], d["ny"], x0, y0, 0.2, 1.0)
    x = np.linspace(-1, 1, d["nx"])
    y = np.linspace(-1, 1, d["ny"])
    return np.exp(-(x[None, :] ** 2 + y[:, None] ** 2) / 0.1).ravel()


def _single(sbp, d, v0, steps, precision):
    if d["problem"] == sbp.WAVE_HOM_2D:
        ones = np.ones(d["nx"] * d["ny"])
        ctx = sbp.Context(sbp.WAVE_VAR_2D, d["order"], d["nx"], d["ny"], rho=ones, K=ones * d["c"] ** 2,
                          bc=d["bc"], precision=precision)
    else:
        ctx = sbp.Context(sbp.ADVECTION_2D, d["order"], d["nx"], d["ny"], a=d["a"], b=d["b"], precision=precision)
    with ctx:
        return ctx.rk4(v0, 0.0, d["dt"], steps)


def test_batch_rejects_bad_instances(sbp):
    with pytest.raises(sbp.SbpError) as ei:
        sbp.Batch([dict(problem=sbp.WAVE_HOM_2D, order=5, nx=40, ny=40, c=1.0, dt=0.01)])
    assert "order" in str(ei.value)
    with pytest.raises(sbp.SbpError):
        sbp.Batch([dict(problem=sbp.WAVE_MMS_2D, order=4, nx=40, ny=40, c=1.0, dt=0.01)])


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [0, 1])
def test_batch_matches_single_instances(sbp, precision):
    insts = _instances(sbp, 11 + precision, 12)
    steps = 130  # one 100-step graph chunk and a 30-step chunk
    with sbp.Batch(insts, precision=precision) as b:
        v0 = [_state(d, k) for k, d in enumerate(insts)]
        for k, v in enumerate(v0):
            b.set_state(k, v)
        b.step_resident(steps)
        b.synchronize()
        got = [b.get_state(k) for k in range(len(insts))]
    tol = 1e-12 if precision == 0 else 1e-6
    for k, d in enumerate(insts):
        ref = _single(sbp, d, v0[k], steps, precision)
        err = np.max(np.abs(got[k] - ref)) / np.max(np.abs(ref))
        assert err <= tol, (k, d, err)


@pytest.mark.gpu
def test_batch_autotune_keeps_states_and_caches(sbp, tmp_path):
    insts = _instances(sbp, 5, 8)
    cache = os.path.join(tmp_path, "tiles.json")
    with sbp.Batch(insts) as b:
        v0 = [_state(d, k) for k, d in enumerate(insts)]
        for k, v in enumerate(v0):
            b.set_state(k, v)
        b.autotune(cache)
        for order in (2, 4, 6):
            assert b.tile_height(order) in (0, 8, 14, 16)  # the FP64 wave table's rows
            for problem in (sbp.WAVE_HOM_2D, sbp.ADVECTION_2D):
                cfg = b.kernel_config(order, problem)
                assert cfg == dict(rows=0, warps=0, ring=0, ctas_per_sm=0, converters=0) or (
                    cfg["rows"] % cfg["warps"] == 0 and 2 <= cfg["ring"] <= 8 and cfg["ctas_per_sm"] in (1, 2)), cfg
        b.step_resident(20)
        b.synchronize()
        got = [b.get_state(k) for k in range(len(insts))]
    entries = json.load(open(cache))
    assert entries and all(v in range(4) for v in entries.values())
    for k, d in enumerate(insts):
        ref = _single(sbp, d, v0[k], 20, 0)
        assert np.max(np.abs(got[k] - ref)) <= 1e-12 * np.max(np.abs(ref))


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [0, 1])
def test_every_kernel_configuration_gives_the_same_bits(sbp, precision):
    """Each of the four table entries of every group (tile rows, warps, ring depth, CTAs per SM)
    computes each point with the same operations in the same order: the states agree bit for bit
    after steps that cross a graph chunk -- except the FP64 waves' fixed-point entry, whose exact
    integer stencils round differently from FP64 taps: within 1e-12 of them."""
    insts = _instances(sbp, 21 + precision, 12)
    v0 = [_state(d, k) for k, d in enumerate(insts)]
    results = []
    for index in range(4):
        with sbp.Batch(insts, precision=precision) as b:
            for k, v in enumerate(v0):
                b.set_state(k, v)
            for order in (2, 4, 6):
                for problem in (sbp.WAVE_HOM_2D, sbp.ADVECTION_2D):
                    b.select_config(order, problem, index)
            b.step_resident(105)
            b.synchronize()
            results.append([b.get_state(k) for k in range(len(insts))])
    fixed = []
    wave_order = next(d["order"] for d in insts if d["problem"] == sbp.WAVE_HOM_2D)
    with sbp.Batch(insts, precision=precision) as b:
        for index in range(4):
            b.select_config(wave_order, sbp.WAVE_HOM_2D, index)
            fixed.append(b.kernel_config(wave_order, sbp.WAVE_HOM_2D)["converters"] > 0)
    assert any(fixed) == (precision == 0)  # the fixed-point entry is an FP64 form
    for index in range(1, 4):
        for k in range(len(insts)):
            a, r = results[index][k], results[0][k]
            if fixed[index] and insts[k]["problem"] == sbp.WAVE_HOM_2D:
                assert np.max(np.abs(a - r)) <= 1e-12 * np.max(np.abs(r)), (index, k, insts[k])
            else:
                assert np.array_equal(a, r), (index, k, insts[k])


def test_select_config_rejects_bad_arguments(sbp):
    """Argument checks run before any device work."""
    assert sbp.load().sbp_batch_select_config(None, 4, sbp.WAVE_HOM_2D, 0) == sbp.ERR_INVALID


@pytest.mark.gpu
def test_batch_state_copies_reject_unknown_where(sbp):
    """A `where` that is neither SBP_HOST nor SBP_DEVICE is refused before any copy."""
    L = sbp.load()
    v = np.zeros(3 * 40 * 40)
    with sbp.Batch([dict(problem=sbp.WAVE_HOM_2D, order=4, nx=40, ny=40, c=1.0, dt=0.01)]) as b:
        assert L.sbp_batch_set_state(b._h, 0, v.ctypes.data, 7) == sbp.ERR_INVALID
        assert L.sbp_batch_get_state(b._h, 0, v.ctypes.data, 7) == sbp.ERR_INVALID
        assert b"where" in L.sbp_batch_last_error(b._h)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "fp64_fixed", "fp32"])
def test_batched_configuration_sample_against_oracle(sbp, port, precision):
    """The benchmark's batched configuration -- 512 uneven wave and advection instances
    (fields.batched_instances) -- advanced 20 RK4 steps in one batch; 16 of its instances (the
    smallest, the largest, a wave and an advection instance of each order, the rest drawn) against
    the oracle: waves as the variable-coefficient problem with rho = 1, K = c^2 and the
    characteristic SAT, advection with its (a, b). FP64 1e-12 (the wave groups on FP64 taps, or
    on the fixed-point stencil kernel), FP32 1e-5 norm-wise relative."""
    import oracle as O

    insts, states = fields.batched_instances(512)
    sample = fields.batched_sample(insts, 16)
    assert len(sample) == 16
    steps = 20
    prec, tol = (sbp.FP32, 1e-5) if precision == "fp32" else (sbp.FP64, 1e-12)
    with sbp.Batch(insts, precision=prec) as b:
        if precision == "fp64_fixed":
            for order in (2, 4, 6):
                for index in range(4):
                    b.select_config(order, sbp.WAVE_HOM_2D, index)
                    if b.kernel_config(order, sbp.WAVE_HOM_2D)["converters"]:
                        break
                assert b.kernel_config(order, sbp.WAVE_HOM_2D)["converters"] > 0
        for k, v in enumerate(states):
            b.set_state(k, v)
        b.step_resident(steps)
        b.synchronize()
        got = {k: b.get_state(k) for k in sample}
    orders = set()
    for k in sample:
        d = insts[k]
        orders.add(d["order"])
        if d["problem"] == sbp.WAVE_HOM_2D:
            ones = np.ones(d["nx"] * d["ny"])
            pb = O.Problem(O.WAVE_VAR_2D, d["order"], d["nx"], d["ny"], rho=ones, K=ones * d["c"] ** 2,
                           bc=O.BC_CHARACTERISTIC)
        else:
            pb = O.Problem(O.ADVECTION_2D, d["order"], d["nx"], d["ny"], a=d["a"], b=d["b"])
        ref = port.rk4(pb, states[k], 0.0, d["dt"], steps)
        err = np.max(np.abs(got[k] - ref)) / np.max(np.abs(ref))
        assert err <= tol, (k, d, err)
    assert orders == {2, 4, 6}
