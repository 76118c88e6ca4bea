"""The 3D acoustic wave system (SBP_WAVE_3D; the reference leaves 3D as a TODO,
code/include/partitioned_rhs/rhs.h:400-402): u_t = -p_x, v_t = -p_y, w_t = -p_z,
p_t = -(u_x + v_y + w_z), rho = K = 1, free-surface or characteristic SAT on
the six faces.

CPU: the oracle's 3D restatement. It reduces to the 2D wave_eq_hom RHS (pinned
to the reference's headers) on states constant in z; its semi-discrete energy
rate is zero to rounding with free-surface faces and negative with
characteristic ones; it converges to a standing mode at the operators' order.

GPU: the 3D stage kernels (the plane-ring kernel; the column kernel where
SBP_WAVE3D_COLUMN selects it) through the C ABI against the oracle on the same
inputs: RHS and matrix-free apply (FP64 1e-12, norm-wise relative, the bar of
the 2D parity tests; FP32 2e-6 on FP32-representable inputs), RK4 (FP64
1e-12; compensated FP32 1e-5), RK45 at fixed steps (1e-12), the error norms and
the 3D H-norm (1e-13).
"""
import numpy as np
import pytest

import oracle as O

SIZES = [(13, 14, 15), (33, 20, 17), (16, 12, 40)]


def relerr(a, b):
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


def _hweights(port, n, order, h):
    """Diagonal of the 1D quadrature H (from the oracle's H-norm of unit vectors)."""
    w = np.zeros(n)
    for i in range(n):
        e = np.zeros(n)
        e[i] = 1.0
        w[i] = port.hnorm(e, n, 1, 1, h, 1.0, order) ** 2
    return w


@pytest.mark.parametrize("order", [2, 4, 6])
def test_oracle_3d_reduces_to_2d_on_z_constant_states(port, order):
    nx, ny, nz = 17, 15, 13
    rng = np.random.default_rng(order)
    q2 = rng.standard_normal((ny, nx, 3))  # (u, v, p) of the 2D system
    v3 = np.zeros((nz, ny, nx, 4))
    v3[..., 0], v3[..., 1], v3[..., 3] = q2[..., 0], q2[..., 1], q2[..., 2]
    F3 = port.rhs(O.Problem(O.WAVE_3D, order, nx, ny, nz), v3.ravel()).reshape(nz, ny, nx, 4)
    F2 = port.rhs(O.Problem(O.WAVE_HOM_2D, order, nx, ny), q2.ravel()).reshape(ny, nx, 3)
    for k in range(nz):
        assert np.array_equal(F3[k, ..., 0], F2[..., 0])
        assert np.array_equal(F3[k, ..., 1], F2[..., 1])
        assert np.array_equal(F3[k, ..., 3], F2[..., 2])
    # w: -D1z of a z-constant p vanishes up to rounding; the z faces carry -/+ bw p
    scale = np.abs(F2).max()
    assert np.abs(F3[1:-1, ..., 2]).max() < 1e-12 * scale


@pytest.mark.parametrize("order", [2, 4, 6])
def test_oracle_3d_energy_rates(port, order):
    nx, ny, nz = 14, 13, 15
    rng = np.random.default_rng(10 + order)
    v = rng.standard_normal(nx * ny * nz * 4)
    for bc, sign in ((O.BC_REFERENCE, 0), (O.BC_CHARACTERISTIC, -1)):
        pb = O.Problem(O.WAVE_3D, order, nx, ny, nz, bc=bc)
        F = port.rhs(pb, v)
        W = (_hweights(port, nz, order, 1 / pb.hiz)[:, None, None] * _hweights(port, ny, order, 1 / pb.hiy)[None, :, None]
             * _hweights(port, nx, order, 1 / pb.hix)[None, None, :])
        rate = np.sum(W[..., None] * v.reshape(nz, ny, nx, 4) * F.reshape(nz, ny, nx, 4))
        energy = np.sum(W[..., None] * v.reshape(nz, ny, nx, 4) ** 2)
        hn = port.hnorm3d(v, nx, ny, nz, 4, 1 / pb.hix, 1 / pb.hiy, 1 / pb.hiz, order)
        assert abs(hn * hn - energy) <= 1e-12 * energy
        if sign == 0:
            assert abs(rate) <= 1e-13 * energy * pb.hix  # conserved to rounding
        else:
            assert rate < -1e-3 * energy


@pytest.mark.parametrize("order,sizes,rate", [(2, (17, 33, 65), 1.8), (4, (17, 33, 65), 3.5)])
def test_oracle_3d_standing_mode_converges(port, order, sizes, rate):
    T = 0.1
    errs = []
    for n in sizes:
        pb = O.Problem(O.WAVE_3D, order, n, n, n)
        h = 2.0 / (n - 1)
        nsteps, dt = port.rk4_nsteps(T, 0.1 * h)
        v = port.rk4(pb, port.init_wave3d_mode(n, n, n, 0.0), 0.0, dt, nsteps)
        errs.append(port.error_l2(v, port.init_wave3d_mode(n, n, n, T), h**3))
    assert errs[0] > errs[1] > errs[2]
    assert np.log2(errs[1] / errs[2]) > rate


# ---------------------------------------------------------------- GPU parity
def _pair(sbp, order, n, bc_char, precision=None):
    nx, ny, nz = n
    kw = {"bc": sbp.BC_CHARACTERISTIC} if bc_char else {}
    if precision is not None:
        kw["precision"] = precision
    ctx = sbp.Context(sbp.WAVE_3D, order, nx, ny, nz, **kw)
    pb = O.Problem(O.WAVE_3D, order, nx, ny, nz, bc=O.BC_CHARACTERISTIC if bc_char else O.BC_REFERENCE)
    return ctx, pb


def _pulse(n, seed=0):
    nx, ny, nz = n
    x, y, z = np.linspace(-1, 1, nx), np.linspace(-1, 1, ny), np.linspace(-1, 1, nz)
    v = np.zeros((nz, ny, nx, 4))
    v[..., 3] = np.exp(-((x[None, None, :] - 0.1) ** 2 + (y[None, :, None] + 0.05) ** 2 + z[:, None, None] ** 2) / 0.3**2)
    v[..., 0] = 0.1 * np.random.default_rng(seed).standard_normal((nz, ny, nx))
    return v.ravel()


@pytest.mark.gpu
@pytest.mark.parametrize("order", [2, 4, 6])
@pytest.mark.parametrize("bc_char", [False, True], ids=["free_surface", "characteristic"])
@pytest.mark.parametrize("n", SIZES, ids=["x".join(map(str, s)) for s in SIZES])
def test_gpu_wave3d_rhs_matches_oracle(sbp, port, order, bc_char, n):
    ctx, pb = _pair(sbp, order, n, bc_char)
    v = np.random.default_rng(order + 7 * bc_char).standard_normal(pb.size)
    with ctx:
        got = ctx.rhs(v)
        got_apply = ctx.apply(v)
    assert relerr(got, port.rhs(pb, v)) < 1e-12
    assert relerr(got_apply, port.apply(pb, v)) < 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("order", [2, 4, 6])
@pytest.mark.parametrize("bc_char", [False, True], ids=["free_surface", "characteristic"])
@pytest.mark.parametrize("n", SIZES + [(70, 30, 35)], ids=["x".join(map(str, s)) for s in SIZES + [(70, 30, 35)]])
def test_gpu_wave3d_rhs_fp32_matches_oracle(sbp, port, order, bc_char, n):
    """The FP32 state's RHS (shared-memory tiles with halos, register windows along z,
    closure rows from global memory) against the FP64 oracle on FP32-representable inputs."""
    ctx, pb = _pair(sbp, order, n, bc_char, precision=sbp.FP32)
    v = np.random.default_rng(order + 3 * bc_char).standard_normal(pb.size).astype(np.float32).astype(np.float64)
    with ctx:
        got = ctx.rhs(v)
        got_apply = ctx.apply(v)
    assert relerr(got, port.rhs(pb, v)) < 2e-6
    assert relerr(got_apply, port.apply(pb, v)) < 2e-6


@pytest.mark.gpu
@pytest.mark.parametrize("order", [2, 4, 6])
def test_gpu_wave3d_rk4_matches_oracle(sbp, port, order):
    n = (24, 20, 18)
    for bc_char in (False, True):
        ctx, pb = _pair(sbp, order, n, bc_char)
        v0 = _pulse(n)
        dt = 0.2 * 2.0 / (max(n) - 1)
        with ctx:
            got = ctx.rk4(v0, 0.0, dt, 12)
        ref = port.rk4(pb, v0, 0.0, dt, 12)
        assert relerr(got, ref) < 1e-12
        ctx, pb = _pair(sbp, order, n, bc_char, precision=sbp.FP32)
        with ctx:
            got32 = ctx.rk4(v0, 0.0, dt, 12)
        assert relerr(got32, ref) < 1e-5


@pytest.mark.gpu
@pytest.mark.parametrize("order", [2, 4, 6])
def test_gpu_wave3d_column_kernel_matches_oracle(sbp, port, order, monkeypatch):
    """The column form (every tap a global load), which runs where the plane-ring
    kernel's 32-bit offsets or 16-byte alignment do not hold, selected here by
    SBP_WAVE3D_COLUMN: RHS and RK4 in FP64 and compensated FP32."""
    monkeypatch.setenv("SBP_WAVE3D_COLUMN", "1")
    n = (33, 20, 17)
    for bc_char in (False, True):
        ctx, pb = _pair(sbp, order, n, bc_char)
        v = np.random.default_rng(order).standard_normal(pb.size)
        v0 = _pulse(n)
        dt = 0.2 * 2.0 / (max(n) - 1)
        with ctx:
            got = ctx.rhs(v)
            got_rk = ctx.rk4(v0, 0.0, dt, 6)
        assert relerr(got, port.rhs(pb, v)) < 1e-12
        ref = port.rk4(pb, v0, 0.0, dt, 6)
        assert relerr(got_rk, ref) < 1e-12
        ctx, pb = _pair(sbp, order, n, bc_char, precision=sbp.FP32)
        with ctx:
            got32 = ctx.rk4(v0, 0.0, dt, 6)
        assert relerr(got32, ref) < 1e-5


@pytest.mark.gpu
def test_gpu_wave3d_rk45_adaptive(sbp, port):
    """Adaptive steps: the weighted error norm counts every scalar of the 3D state."""
    n = (20, 17, 15)
    ctx, pb = _pair(sbp, 4, n, True)
    v0 = _pulse(n, 5)
    with ctx:
        ctx.set_state(v0)
        st = ctx.rk45_resident(0.0, 0.3, 0.01, atol=1e-6, rtol=1e-6)
        got = ctx.get_state()
    ref, rst = port.rk45(pb, v0, 0.0, 0.3, 0.01, atol=1e-6, rtol=1e-6)
    assert (st["accepted"], st["rejected"]) == (rst["accepted"], rst["rejected"]) and st["accepted"] > 5
    assert abs(st["wlte"] - rst["wlte"]) <= 1e-6 * rst["wlte"]
    assert relerr(got, ref) < 1e-9


@pytest.mark.gpu
def test_gpu_wave3d_rk45_norms(sbp, port):
    n = (21, 18, 16)
    ctx, pb = _pair(sbp, 4, n, True)
    v0 = _pulse(n, 3)
    h = 0.02
    fixed = dict(atol=1e6, rtol=0.0, dt_max=h)
    with ctx:
        ctx.set_state(v0)
        st = ctx.rk45_resident(0.0, 8 * h, h, **fixed)
        got = ctx.get_state()
        ref, rst = port.rk45(pb, v0, 0.0, 8 * h, h, **fixed)
        assert st["accepted"] == rst["accepted"] == 8 and st["rejected"] == 0
        assert relerr(got, ref) < 1e-12
        # H-norm and error norms of the resident state against the oracle's
        hn = port.hnorm3d(got, n[0], n[1], n[2], 4, ctx.hx, ctx.hy, ctx.hz, 4)
        assert abs(ctx.hnorm() - hn) <= 1e-13 * hn
        exact = v0
        l2, mx = ctx.error_norms(exact)
        assert abs(l2 - port.error_l2(got, exact, ctx.hx * ctx.hy * ctx.hz)) <= 1e-12 * l2
        assert abs(mx - port.error_max(got, exact)) <= 1e-14 * mx
