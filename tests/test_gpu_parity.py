"""Parity of the CUDA path (called through the C ABI) with the oracle.

Tolerance (FP64): norm-wise relative max error ||gpu - oracle||_inf / ||oracle||_inf
<= 1e-12. The GPU folds 1/h into the stencil weights and contracts products
into FMAs, so results differ from the reference's rounding in the last bits;
the stencil sums cancel, so the bound is norm-wise, not pointwise.
FP32 state: <= 1e-5 relative for one RHS (stencil arithmetic in FP32).
"""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

TOL64 = 1e-12
TOL32 = 1e-5


def relerr(a, b):
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


def _fields(n_x, n_y, seed):
    rng = np.random.default_rng(seed)
    x = np.linspace(-1, 1, n_x)
    y = np.linspace(-1, 1, n_y)
    X, Y = np.meshgrid(x, y)
    rho = 1.0 + 0.4 * np.tanh(np.sin(3 * X + rng.uniform()) * np.cos(2 * Y))
    K = 1.2 + 0.5 * np.tanh(np.cos(2 * X - Y + rng.uniform()))
    return rho.ravel(), K.ravel()


def _ctx(sbp, prob, order, nx, ny=1, **kw):
    return sbp.Context(prob, order, nx, ny, **kw)


SIZES_2D = [(None, None), (33, 33), (64, 64), (97, 45), (130, 71)]


@pytest.mark.parametrize("order", [2, 4, 6])
@pytest.mark.parametrize("size", SIZES_2D)
def test_wave_hom_rhs(sbp, port, order, size):
    nx, ny = size
    if nx is None:
        nx = ny = {2: 3, 4: 8, 6: 12}[order]
    rng = np.random.default_rng(order * 1000 + nx)
    src = rng.standard_normal(3 * nx * ny)
    pb = O.Problem(O.WAVE_HOM_2D, order, nx, ny)
    with _ctx(sbp, sbp.WAVE_HOM_2D, order, nx, ny) as c:
        assert relerr(c.rhs(src), port.rhs(pb, src)) <= TOL64
        assert relerr(c.apply(src), port.apply(pb, src)) <= TOL64


@pytest.mark.parametrize("order", [2, 4, 6])
@pytest.mark.parametrize("size", [(33, 33), (70, 41)])
def test_wave_mms_rhs(sbp, port, order, size):
    nx, ny = size
    rng = np.random.default_rng(5 + order)
    src = rng.standard_normal(3 * nx * ny)
    pb = O.Problem(O.WAVE_MMS_2D, order, nx, ny)
    with _ctx(sbp, sbp.WAVE_MMS_2D, order, nx, ny) as c:
        for t in (0.0, 0.37):
            assert relerr(c.rhs(src, t), port.rhs(pb, src, t)) <= TOL64


@pytest.mark.parametrize("order", [2, 4, 6])
@pytest.mark.parametrize("bc", [0, 1])
@pytest.mark.parametrize("size", [(37, 37), (129, 66)])
def test_wave_var_rhs(sbp, port, order, bc, size):
    nx, ny = size
    rho, K = _fields(nx, ny, order + 10 * bc)
    rng = np.random.default_rng(11)
    src = rng.standard_normal(3 * nx * ny)
    pb = O.Problem(O.WAVE_VAR_2D, order, nx, ny, rho=rho, K=K, bc=bc)
    with _ctx(sbp, sbp.WAVE_VAR_2D, order, nx, ny, rho=rho, K=K, bc=bc) as c:
        assert relerr(c.rhs(src), port.rhs(pb, src)) <= TOL64


@pytest.mark.parametrize("order", [2, 4, 6])
def test_wave_hom_characteristic_matches_unit_coefficients(sbp, port, order):
    nx, ny = 75, 40
    ones = np.ones(nx * ny)
    src = np.random.default_rng(2).standard_normal(3 * nx * ny)
    pb = O.Problem(O.WAVE_VAR_2D, order, nx, ny, rho=ones, K=ones, bc=O.BC_CHARACTERISTIC)
    with _ctx(sbp, sbp.WAVE_HOM_2D, order, nx, ny, bc=sbp.BC_CHARACTERISTIC) as c:
        assert relerr(c.rhs(src), port.rhs(pb, src)) <= TOL64


@pytest.mark.parametrize("order", [2, 4, 6])
@pytest.mark.parametrize("n", [None, 33, 201])
def test_advection_1d_rhs(sbp, port, order, n):
    n = n or {2: 3, 4: 8, 6: 12}[order]
    for a in (1.0, 1.5, -0.8):
        src = np.random.default_rng(n).standard_normal(n)
        pb = O.Problem(O.ADVECTION_1D, order, n, a=a)
        with _ctx(sbp, sbp.ADVECTION_1D, order, n, a=a) as c:
            assert relerr(c.rhs(src), port.rhs(pb, src)) <= TOL64


@pytest.mark.parametrize("order", [2, 4, 6])
@pytest.mark.parametrize("size", [(12, 12), (33, 33), (80, 47)])
def test_advection_2d_rhs(sbp, port, order, size):
    nx, ny = size
    if nx < {2: 3, 4: 8, 6: 12}[order]:
        pytest.skip("below minimum size")
    src = np.random.default_rng(nx * ny).standard_normal(nx * ny)
    for a, b in ((1.5, -1.0), (-0.5, 0.7)):
        pb = O.Problem(O.ADVECTION_2D, order, nx, ny, a=a, b=b)
        with _ctx(sbp, sbp.ADVECTION_2D, order, nx, ny, a=a, b=b) as c:
            assert relerr(c.rhs(src), port.rhs(pb, src)) <= TOL64


@pytest.mark.parametrize("order", [2, 4, 6])
@pytest.mark.parametrize("n", [None, 40, 201])
def test_reflection_rhs(sbp, port, order, n):
    n = n or {2: 3, 4: 8, 6: 12}[order]
    src = np.random.default_rng(n + 1).standard_normal(2 * n)
    pb = O.Problem(O.REFLECTION_1D, order, n)
    with _ctx(sbp, sbp.REFLECTION_1D, order, n) as c:
        assert relerr(c.rhs(src), port.rhs(pb, src)) <= TOL64


@pytest.mark.parametrize("order", [2, 4, 6])
@pytest.mark.parametrize("prob", ["hom", "var_char", "mms"])
def test_rk4_steps_match_oracle(sbp, port, order, prob):
    nx, ny = 90, 77
    h = 2.0 / (nx - 1)
    kw, okw = {}, {}
    if prob == "var_char":
        rho, K = _fields(nx, ny, 3)
        kw = dict(rho=rho, K=K, bc=1)
        okw = dict(rho=rho, K=K, bc=1)
        P, OP = sbp.WAVE_VAR_2D, O.WAVE_VAR_2D
    elif prob == "mms":
        P, OP = sbp.WAVE_MMS_2D, O.WAVE_MMS_2D
    else:
        P, OP = sbp.WAVE_HOM_2D, O.WAVE_HOM_2D
    v0 = port.init_wave_pulse(nx, ny, 0.1, -0.2, 0.3, 1.0) + 0.1 * port.init_wave_mms(nx, ny, 0.05)
    dt = 0.2 * h
    pb = O.Problem(OP, order, nx, ny, **okw)
    with _ctx(sbp, P, order, nx, ny, **kw) as c:
        # 57 steps: one 50-step graph chunk plus a 7-step chunk
        got = c.rk4(v0, 0.0, dt, 57)
    ref = port.rk4(pb, v0, 0.0, dt, 57)
    assert relerr(got, ref) <= TOL64


@pytest.mark.parametrize("prob", ["adv1d", "adv2d", "refl"])
def test_rk4_line_problems_match_oracle(sbp, port, prob):
    order = 4
    if prob == "adv1d":
        n = 201
        c = sbp.Context(sbp.ADVECTION_1D, order, n, a=1.0)
        pb = O.Problem(O.ADVECTION_1D, order, n, a=1.0)
        v0 = port.init_adv1d(n, 1.0, 0.0)
    elif prob == "adv2d":
        n = 65
        c = sbp.Context(sbp.ADVECTION_2D, order, n, n, a=1.5, b=-1.0)
        pb = O.Problem(O.ADVECTION_2D, order, n, n, a=1.5, b=-1.0)
        v0 = port.init_adv2d(n, n, 1.5, -1.0, 0.0)
    else:
        n = 101
        c = sbp.Context(sbp.REFLECTION_1D, order, n)
        pb = O.Problem(O.REFLECTION_1D, order, n)
        v0 = port.init_reflection(n, 0.0)
    dt = 0.1 * 2.0 / (n - 1)
    with c:
        got = c.rk4(v0, 0.0, dt, 120)
    assert relerr(got, port.rk4(pb, v0, 0.0, dt, 120)) <= TOL64


def test_kat_advection_config_on_gpu(sbp, port):
    """1D advection, a = 1, N = 201, order 4, CFL 0.1, T = 1.8, through ts_rk4's replacement:
    L2 = 3.930261e-04, the reference operators' known answer."""
    n, a = 201, 1.0
    with sbp.Context(sbp.ADVECTION_1D, 4, n, a=a) as c:
        v = c.ts_rk4(port.init_adv1d(n, a, 0.0), 1.8, 0.1 * 2.0 / (n - 1))
        c.set_state(v)
        l2, mx = c.error_norms(port.init_adv1d(n, a, 1.8))
    assert l2 == pytest.approx(3.930261e-04, rel=1e-6)
    assert mx == pytest.approx(9.271863e-04, rel=1e-6)


@pytest.mark.parametrize("order,expected", [(2, 1.113e-1), (4, 4.090e-3), (6, 5.975e-3)])
def test_kat_wave_mms_on_gpu(sbp, port, order, expected):
    n, T = 81, 0.5
    h = 2.0 / (n - 1)
    with sbp.Context(sbp.WAVE_HOM_2D, order, n, n) as c:
        v = c.ts_rk4(port.init_wave_mms(n, n, 0.0), T, 0.2 * h)
        c.set_state(v)
        l2, _ = c.error_norms(port.init_wave_mms(n, n, T))
    assert l2 == pytest.approx(expected, rel=2e-3)


def test_device_norms_match_oracle(sbp, port):
    nx, ny, order = 150, 97, 6
    rng = np.random.default_rng(9)
    v, ex = rng.standard_normal(3 * nx * ny), rng.standard_normal(3 * nx * ny)
    hx, hy = 2.0 / (nx - 1), 2.0 / (ny - 1)
    with sbp.Context(sbp.WAVE_HOM_2D, order, nx, ny) as c:
        c.set_state(v)
        l2, mx = c.error_norms(ex)
        hn = c.hnorm()
    assert l2 == pytest.approx(port.error_l2(v, ex, hx * hy), rel=1e-13)
    assert mx == port.error_max(v, ex)
    assert hn == pytest.approx(port.hnorm(v, nx, ny, 3, hx, hy, order), rel=1e-13)


@pytest.mark.parametrize("order", [2, 4, 6])
def test_fp32_rhs(sbp, port, order):
    nx, ny = 101, 88
    x = np.linspace(-1, 1, nx)
    y = np.linspace(-1, 1, ny)
    X, Y = np.meshgrid(x, y)
    src = np.stack([np.sin(2 * X) * np.cos(Y), np.cos(X + Y), np.exp(-4 * (X**2 + Y**2))], axis=-1).ravel()
    pb = O.Problem(O.WAVE_HOM_2D, order, nx, ny)
    with _ctx(sbp, sbp.WAVE_HOM_2D, order, nx, ny, precision=sbp.FP32) as c:
        assert relerr(c.rhs(src), port.rhs(pb, src)) <= TOL32


def test_fp32_compensated_rk4_close_to_fp64(sbp, port):
    n, order = 257, 4
    h = 2.0 / (n - 1)
    v0 = port.init_wave_pulse(n, n, 0.0, 0.0, 0.1, 1.0)
    with sbp.Context(sbp.WAVE_HOM_2D, order, n, n, bc=1) as c64, \
            sbp.Context(sbp.WAVE_HOM_2D, order, n, n, bc=1, precision=sbp.FP32) as c32:
        a = c64.rk4(v0, 0.0, 0.2 * h, 400)
        b = c32.rk4(v0, 0.0, 0.2 * h, 400)
    assert relerr(b, a) < 2e-5


def test_large_grid_energy_and_symmetry(sbp, port):
    """At a production size (1024^2, order 4) with the characteristic SAT:
    the discrete energy never grows, and a centred pulse stays symmetric in p
    under x -> -x (exact for the symmetric operator pair)."""
    n, order = 1024, 4
    h = 2.0 / (n - 1)
    v = port.init_wave_pulse(n, n, 0.0, 0.0, 0.05, 1.0)
    ones = np.ones(n * n)
    with sbp.Context(sbp.WAVE_HOM_2D, order, n, n, bc=1) as c:
        c.set_state(v)
        e_prev = c.hnorm()
        for _ in range(5):
            c.step_resident(0.0, 0.2 * h, 40)
            c.synchronize()
            e = c.hnorm()
            assert np.isfinite(e) and e <= e_prev * (1 + 1e-12)
            e_prev = e
        out = c.get_state().reshape(n, n, 3)
    p = out[:, :, 2]
    assert np.max(np.abs(p - p[:, ::-1])) <= 1e-10 * np.max(np.abs(p))
    assert np.max(np.abs(p - p.T)) <= 1e-10 * np.max(np.abs(p))


def _two_layer_fields(nx, ny, seed):
    rng = np.random.default_rng(seed)
    rho = 1.0 + rng.uniform(0, 2, (ny, nx))
    K = 1.0 + rng.uniform(0, 2, (ny, nx))
    rho[ny // 2:] *= 4.0
    K[ny // 2:] *= 4.0
    return rho.ravel(), K.ravel()


@pytest.mark.parametrize("order", [2, 4, 6])
@pytest.mark.parametrize("bc", [0, 1])
@pytest.mark.parametrize("size", [(40, 2 * 29), (130, 2 * 70)])
def test_two_block_interface_rhs(sbp, port, order, bc, size):
    nx, ny = size
    rho, K = _two_layer_fields(nx, ny, order + bc)
    src = np.random.default_rng(13).standard_normal(3 * nx * ny)
    pb = O.Problem(O.WAVE_2BLOCK_2D, order, nx, ny, rho=rho, K=K, bc=bc)
    with _ctx(sbp, sbp.WAVE_2BLOCK_2D, order, nx, ny, rho=rho, K=K, bc=bc) as c:
        assert relerr(c.rhs(src), port.rhs(pb, src)) <= TOL64
        assert relerr(c.apply(src), port.apply(pb, src)) <= TOL64


@pytest.mark.parametrize("order", [4, 6])
def test_two_block_rk4_and_energy(sbp, port, order):
    nx, ny = 96, 2 * 64
    rho, K = _two_layer_fields(nx, ny, 5)
    pb = O.Problem(O.WAVE_2BLOCK_2D, order, nx, ny, rho=rho, K=K, bc=1)
    v0 = port.init_wave_pulse(nx, ny, 0.0, -0.2, 0.2, 1.0)
    hy = 1.0 / (ny // 2 - 1)
    dt = 0.2 * hy / np.sqrt((K / rho).max())
    with _ctx(sbp, sbp.WAVE_2BLOCK_2D, order, nx, ny, rho=rho, K=K, bc=1) as c:
        got = c.rk4(v0, 0.0, dt, 60)
        c.set_state(got)
        hn = c.hnorm()
    assert relerr(got, port.rk4(pb, v0, 0.0, dt, 60)) <= TOL64
    assert hn == pytest.approx(port.hnorm_2block(got, nx, ny, 3, 2.0 / (nx - 1), hy, order), rel=1e-13)


def test_two_block_reflection_coefficient_on_gpu(sbp):
    """Impedance ratio 4 across y = 0 (equal speeds): R = 0.6, T = 1.6."""
    nx, nb, order = 81, 161, 4
    ny = 2 * nb
    rho = np.ones((ny, nx))
    rho[nb:] = 4.0
    rho = rho.ravel()
    y = np.concatenate([np.linspace(-1, 0, nb), np.linspace(0, 1, nb)])
    p = np.exp(-((y + 0.35) / 0.06) ** 2)
    v = np.zeros((ny, nx, 3))
    v[:, :, 2] = p[:, None]
    v[:, :, 1] = p[:, None]
    with sbp.Context(sbp.WAVE_2BLOCK_2D, order, nx, ny, rho=rho, K=rho.copy(), bc=1) as c:
        out = c.ts_rk4(v.ravel(), 0.7, 0.2 / (nb - 1)).reshape(ny, nx, 3)
    col = out[:, nx // 2, 2]
    assert col[:nb].max() == pytest.approx(0.6, abs=0.01)
    assert col[nb:].max() == pytest.approx(1.6, abs=0.01)


@pytest.mark.parametrize("order", [2, 4, 6])
def test_advection_velocity_fields_against_reference_fixtures(sbp, golden, order):
    """Velocities at every point (the reference's callables a(i), a(i,j), b(i,j)): the CUDA
    path against the reference's own RHS in tests/golden (its out-of-bounds boundary reads
    masked), 1e-12 norm-wise."""
    vmeta = golden["vmeta"]
    seen = 0
    for k, (prob, o, n) in enumerate(vmeta):
        prob, o, n = int(prob), int(o), int(n)
        if o != order:
            continue
        src, ref = golden[f"vsrc{k}"], golden[f"vdst{k}"]
        if prob == O.ADVECTION_1D:
            ctx = sbp.Context(sbp.ADVECTION_1D, order, n, a_field=golden[f"va{k}"])
            mask = np.zeros(n, dtype=bool)
            mask[n - 1] = True
        else:
            ctx = sbp.Context(sbp.ADVECTION_2D, order, n, n, a_field=golden[f"va{k}"], b_field=golden[f"vb{k}"])
            mask = np.zeros(n * n, dtype=bool)
            mask[:n] = True
        with ctx as c:
            got = c.rhs(src)
        assert relerr(got[~mask], ref[~mask]) <= TOL64
        seen += 1
    assert seen >= 4


@pytest.mark.parametrize("order", [2, 4, 6])
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_advection_velocity_fields_rhs_and_rk4(sbp, port, order, precision):
    """Fields whose sign changes along every boundary (inflow and outflow on each side), a
    non-square 2D grid and a 1D field changing sign inside: RHS and 20 RK4 steps against
    the oracle."""
    prec, tol = (sbp.FP64, TOL64) if precision == "fp64" else (sbp.FP32, TOL32)
    nx, ny = 83, 57
    x, y = np.linspace(-1, 1, nx), np.linspace(-1, 1, ny)
    X, Y = np.meshgrid(x, y)
    a = np.sin(2 * X + Y) + 0.2
    b = np.cos(X - 2 * Y) - 0.3
    rng = np.random.default_rng(order)
    src = rng.standard_normal(nx * ny)
    v0 = np.exp(-((X - 0.1) ** 2 + (Y + 0.2) ** 2) / 0.2 ** 2).ravel()
    pb = O.Problem(O.ADVECTION_2D, order, nx, ny, a_field=a, b_field=b)
    dt = 0.1 * 2.0 / (nx - 1)
    with sbp.Context(sbp.ADVECTION_2D, order, nx, ny, a_field=a, b_field=b, precision=prec) as c:
        assert relerr(c.rhs(src), port.rhs(pb, src)) <= tol
        assert relerr(c.rk4(v0, 0.0, dt, 20), port.rk4(pb, v0, 0.0, dt, 20)) <= tol
    n = 101
    x = np.linspace(-1, 1, n)
    a1 = 0.1 - np.sin(3 * x)  # > 0 at the left end and < 0 at the right: inflow through both ends
    src1 = rng.standard_normal(n)
    pb1 = O.Problem(O.ADVECTION_1D, order, n, a_field=a1)
    w0 = np.exp(-(x / 0.2) ** 2)
    with sbp.Context(sbp.ADVECTION_1D, order, n, a_field=a1, precision=prec) as c:
        assert relerr(c.rhs(src1), port.rhs(pb1, src1)) <= tol
        assert relerr(c.rk4(w0, 0.0, 0.1 * 2.0 / (n - 1), 20), port.rk4(pb1, w0, 0.0, 0.1 * 2.0 / (n - 1), 20)) <= tol


def test_velocity_fields_rejected_for_other_problems(sbp):
    with pytest.raises(sbp.SbpError) as e:
        sbp.Context(sbp.WAVE_HOM_2D, 4, 20, 20, a_field=np.ones(400))
    assert e.value.code == sbp.ERR_INVALID
