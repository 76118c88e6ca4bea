"""The SAT of x-face points in the 2D wave stage kernels runs in a separate pass
per tile: a point on x = 0 or x = nx - 1 (not on a y face or an interface line)
leaves its RHS in shared memory and one warp applies SAT and stage update to all
of them. These cases put x faces where the tile layout (64 columns per tile)
makes them special: a last tile one column wide (65, 129), a face on a tile's
last column (64), both faces in one tile (63), and the interface lines of the
two-block problem, through every stage kind: RK4 (first, middle, last stage)
in FP64 (1e-12 against the oracle, the bar of the other parity tests) and
compensated FP32 (1e-5), and the fused Fehlberg stages at fixed steps (1e-12).
"""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


def relerr(a, b):
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


def _fields(nx, ny, seed, two_layer=False):
    rng = np.random.default_rng(seed)
    rho = 1.0 + rng.uniform(0, 1, (ny, nx))
    K = 1.0 + rng.uniform(0, 1, (ny, nx))
    if two_layer:
        rho[ny // 2:] *= 4.0
        K[ny // 2:] *= 4.0
    return rho.ravel(), K.ravel()


def _state(port, nx, ny, seed):
    v = port.init_wave_pulse(nx, ny, 0.1, -0.1, 0.3, 1.0)
    return v + 0.05 * np.random.default_rng(seed).standard_normal(v.size)


CASES = [("hom", 65, 40), ("hom", 129, 20), ("hom", 64, 33), ("var", 63, 70), ("var", 129, 37),
         ("two_block", 65, 2 * 24), ("two_block", 129, 2 * 17)]


def _pair(sbp, kind, order, nx, ny, precision=None):
    kw = {"bc": 1}
    if precision is not None:
        kw["precision"] = precision
    if kind == "hom":
        # the oracle's rho = K = 1 problem carries only the reference's free-surface SAT;
        # with characteristic SAT it is the variable-coefficient problem with unit fields
        ones = np.ones(nx * ny)
        return (sbp.Context(sbp.WAVE_HOM_2D, order, nx, ny, bc=sbp.BC_CHARACTERISTIC,
                            **({"precision": precision} if precision is not None else {})),
                O.Problem(O.WAVE_VAR_2D, order, nx, ny, rho=ones, K=ones, bc=O.BC_CHARACTERISTIC))
    rho, K = _fields(nx, ny, order + nx, two_layer=kind == "two_block")
    sprob = sbp.WAVE_VAR_2D if kind == "var" else sbp.WAVE_2BLOCK_2D
    oprob = O.WAVE_VAR_2D if kind == "var" else O.WAVE_2BLOCK_2D
    return (sbp.Context(sprob, order, nx, ny, rho=rho, K=K, **kw),
            O.Problem(oprob, order, nx, ny, rho=rho, K=K, bc=1))


@pytest.mark.parametrize("order", [2, 4, 6])
@pytest.mark.parametrize("case", CASES, ids=[f"{k}_{nx}x{ny}" for k, nx, ny in CASES])
def test_xface_rk4_fp64_and_fp32(sbp, port, order, case):
    kind, nx, ny = case
    ctx, pb = _pair(sbp, kind, order, nx, ny)
    v0 = _state(port, nx, ny, order)
    dt = 0.1 * 2.0 / (max(nx, ny) - 1)
    with ctx:
        got = ctx.rk4(v0, 0.0, dt, 7)
        rhs = ctx.rhs(v0)
    ref = port.rk4(pb, v0, 0.0, dt, 7)
    assert relerr(got, ref) < 1e-12
    assert relerr(rhs, port.rhs(pb, v0)) < 1e-12
    ctx32, _ = _pair(sbp, kind, order, nx, ny, precision=sbp.FP32)
    with ctx32:
        got32 = ctx32.rk4(v0, 0.0, dt, 7)
    assert relerr(got32, ref) < 1e-5


@pytest.mark.parametrize("order", [2, 4, 6])
@pytest.mark.parametrize("case", [CASES[0], CASES[3], CASES[5]], ids=["hom_65x40", "var_63x70", "two_block_65x48"])
def test_xface_fused_fehlberg_fixed_steps(sbp, port, order, case):
    kind, nx, ny = case
    ctx, pb = _pair(sbp, kind, order, nx, ny)
    v0 = _state(port, nx, ny, 3 + order)
    h = 0.1 * 2.0 / (max(nx, ny) - 1)
    fixed = dict(atol=1e6, rtol=0.0, dt_max=h)
    with ctx:
        ctx.set_state(v0)
        st = ctx.rk45_resident(0.0, 6 * h, h, **fixed)
        got = ctx.get_state()
    ref, rst = port.rk45(pb, v0, 0.0, 6 * h, h, **fixed)
    assert st["accepted"] == rst["accepted"] == 6 and st["rejected"] == 0
    assert relerr(got, ref) < 1e-12
