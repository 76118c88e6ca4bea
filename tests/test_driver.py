"""The demo driver (hpc-reading-course_gb300/drivers/sbp_demo.cpp): the reference's main
programs re-expressed as plain C++ calls into the C ABI (sbp_create, sbp_ts_rk4,
sbp_error_norms), printing the reference programs' result lines. Known answers: the
1D advection case a = 1, N = 201, order 4, CFL 0.1, T = 1.8 gives L2 = 3.930261e-04
(the reference operators with RK4); the 2D standing mode agrees with the oracle."""
import os
import re
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def driver():
    sys.path.insert(0, os.path.join(ROOT, "hpc-reading-course_gb300"))
    import build

    return build.build_driver()


def _run(driver, *args):
    r = subprocess.run([driver, *map(str, args)], capture_output=True, text=True, timeout=600)
    return r


def _errors(out):
    m = re.search(r"The l2-error is: (\S+), and the maximum error is (\S+)", out)
    assert m, out
    return float(m.group(1)), float(m.group(2))


def test_driver_rejects_bad_arguments(driver):
    for args in ((), ("wave_hom", 10), ("nonsense", 1, 2, 3), ("advection_1d", -5, 1.0, 0.1)):
        r = _run(driver, *args)
        assert r.returncode == 1 and "usage" in r.stderr


@pytest.mark.gpu
def test_driver_advection_known_answer(driver):
    r = _run(driver, "advection_1d", 201, 1.8, 0.1, 4, 1.0)
    assert r.returncode == 0, r.stderr
    assert "Elapsed time:" in r.stdout
    l2, _ = _errors(r.stdout)
    assert l2 == pytest.approx(3.930261e-04, rel=1e-5)  # the driver prints six significant digits (%g)


@pytest.mark.gpu
@pytest.mark.parametrize("order", [2, 4, 6])
def test_driver_wave_hom_matches_oracle(driver, port, order):
    import oracle as O

    n, T, cfl = 81, 0.5, 0.2
    r = _run(driver, "wave_hom", n, n, T, cfl, order)
    assert r.returncode == 0, r.stderr
    l2, mx = _errors(r.stdout)
    h = 2.0 / (n - 1)
    nsteps, dt = port.rk4_nsteps(T, cfl * h)
    v = port.rk4(O.Problem(O.WAVE_HOM_2D, order, n, n), port.init_wave_mms(n, n, 0.0), 0.0, dt, nsteps)
    exact = port.init_wave_mms(n, n, T)
    assert l2 == pytest.approx(port.error_l2(v, exact, h * h), rel=1e-5)  # the driver prints six significant digits (%g)
    assert mx == pytest.approx(port.error_max(v, exact), rel=1e-5)  # the driver prints six significant digits (%g)
