"""Oracle parity at the production grid sizes of the 2D wave workload.

The smaller parity grids (tests/test_gpu_parity.py) hold at most a few dozen
tiles, so every CTA of the persistent stage kernel handles one tile. At
1024^2 and 4096^2 each CTA walks many tiles through its shared-memory ring:
these tests check the ring reuse, the mbarrier phase flips and the reuse of
the deferred x-face boxes against the oracle, on the reference's path
(wave_eq_hom_serial + the SAT, code/demo/wave_hom/wave_eq_hom_rhs.h:365,443)
with the free-surface SAT and with the characteristic SAT of the benchmark.

Tolerances as in tests/test_gpu_parity.py: FP64 1e-12 norm-wise relative in
the max norm; the FP32 state against the FP64 oracle 1e-5.
"""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

TOL64 = 1e-12
TOL32 = 1e-5


def relerr(a, b):
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


def _state(n: int, seed: int) -> np.ndarray:
    """Three offset Gaussian pulses (p width 0.05, the benchmark's) plus seeded
    noise of 1e-3 so that every point's arithmetic matters, AoS (j, i, comp)."""
    x = np.linspace(-1.0, 1.0, n)
    X, Y = np.meshgrid(x, x)
    v = np.empty((n, n, 3))
    v[..., 0] = 0.5 * np.exp(-((X + 0.2) ** 2 + (Y - 0.1) ** 2) / 0.08 ** 2)
    v[..., 1] = 0.3 * np.exp(-((X - 0.05) ** 2 + (Y - 0.3) ** 2) / 0.1 ** 2)
    v[..., 2] = np.exp(-((X - 0.1) ** 2 + (Y + 0.05) ** 2) / 0.05 ** 2)
    v += 1e-3 * np.random.default_rng(seed).standard_normal(v.shape)
    return v.ravel()


def _bc(sbp, name):
    return (sbp.BC_CHARACTERISTIC, O.BC_CHARACTERISTIC) if name == "char" else (sbp.BC_REFERENCE, O.BC_REFERENCE)


@pytest.fixture(scope="module")
def port_all_cores(port):
    import os

    port.set_threads(os.cpu_count() or 1)
    return port


@pytest.mark.parametrize("order", [2, 4, 6])
@pytest.mark.parametrize("bc", ["free_surface", "char"])
def test_1024_rhs_and_ten_rk4_steps(sbp, port_all_cores, order, bc):
    n = 1024
    port = port_all_cores
    gbc, obc = _bc(sbp, bc)
    pb = O.Problem(O.WAVE_HOM_2D, order, n, n, bc=obc)
    v0 = _state(n, order)
    dt = 0.2 * 2.0 / (n - 1)
    with sbp.Context(sbp.WAVE_HOM_2D, order, n, n, bc=gbc) as c:
        assert relerr(c.rhs(v0), port.rhs(pb, v0)) <= TOL64
        assert relerr(c.rk4(v0, 0.0, dt, 10), port.rk4(pb, v0, 0.0, dt, 10)) <= TOL64


def test_4096_order4_characteristic_rhs_and_two_rk4_steps(sbp, port_all_cores):
    """The benchmark's grid, order and SAT."""
    n, order = 4096, 4
    port = port_all_cores
    pb = O.Problem(O.WAVE_HOM_2D, order, n, n, bc=O.BC_CHARACTERISTIC)
    v0 = _state(n, 40)
    dt = 0.2 * 2.0 / (n - 1)
    with sbp.Context(sbp.WAVE_HOM_2D, order, n, n, bc=sbp.BC_CHARACTERISTIC) as c:
        assert relerr(c.rhs(v0), port.rhs(pb, v0)) <= TOL64
        assert relerr(c.rk4(v0, 0.0, dt, 2), port.rk4(pb, v0, 0.0, dt, 2)) <= TOL64


@pytest.mark.parametrize("n", [1024, 4096])
def test_fp32_against_fp64_oracle(sbp, port_all_cores, n):
    """The compensated FP32 form at both production sizes, characteristic SAT,
    order 4: one RHS and two RK4 steps against the FP64 oracle."""
    order = 4
    port = port_all_cores
    pb = O.Problem(O.WAVE_HOM_2D, order, n, n, bc=O.BC_CHARACTERISTIC)
    v0 = _state(n, 7)
    dt = 0.2 * 2.0 / (n - 1)
    ref = port.rhs(pb, v0)
    # The FP32 inputs carry 2^-24 relative rounding, which a derivative amplifies by
    # 1/h times the stencil's weight sum (1.5 at order 4): at 4096^2 that bound is
    # above 1e-5 of the RHS's max norm, so the RHS is held to the larger of the two.
    hi = (n - 1) / 2.0
    tol_rhs = max(TOL32, 2.0 * 2.0 ** -24 * 1.5 * hi * np.max(np.abs(v0)) / np.max(np.abs(ref)))
    with sbp.Context(sbp.WAVE_HOM_2D, order, n, n, bc=sbp.BC_CHARACTERISTIC, precision=sbp.FP32) as c:
        assert relerr(c.rhs(v0), ref) <= tol_rhs
        assert relerr(c.rk4(v0, 0.0, dt, 2), port.rk4(pb, v0, 0.0, dt, 2)) <= TOL32
