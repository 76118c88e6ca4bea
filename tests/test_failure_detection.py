"""Failure detection of the stage kernels, exercised without a GPU fault.

Every mbarrier wait in the 2D wave stage kernels is bounded by %globaltimer.
sbp_test_drop_tile makes the producer warp of the next RHS evaluation issue no
load for one tile, so the consumers' wait for that tile runs out after the
context's wait limit (set to a few milliseconds here): the kernel sets the
error word, lets its copies in flight land and returns. The call must return
SBP_ERR_DEVICE, and the same context must then give the oracle's results.
Nothing here faults, traps or hangs the GPU: the missing tile is a load that
is never issued, and every wait has a limit.

CPU: the test aid's arguments are checked before any GPU work.
"""
import numpy as np
import pytest

import oracle as O

TOL64 = 1e-12


def relerr(a, b):
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


def test_test_aid_rejects_bad_arguments(sbp):
    L = sbp.load()
    assert L.sbp_set_wait_limit(None, 1000) == sbp.ERR_INVALID
    assert L.sbp_test_drop_tile(None, 0) == sbp.ERR_INVALID


@pytest.mark.gpu
@pytest.mark.parametrize("n,tile", [(256, 5), (1024, 700)], ids=["one_tile_per_cta", "many_tiles_per_cta"])
def test_dropped_tile_times_out_and_context_stays_usable(sbp, port, n, tile):
    """256^2: each CTA owns one tile, the consumers' wait runs out. 1024^2: each
    CTA walks several tiles, so the producer's wait for the stage the stalled
    consumers never release runs out as well, with the next tile's copy in flight."""
    order = 4
    rng = np.random.default_rng(n)
    src = rng.standard_normal(3 * n * n)
    pb = O.Problem(O.WAVE_HOM_2D, order, n, n, bc=O.BC_CHARACTERISTIC)
    expected = port.rhs(pb, src)
    with sbp.Context(sbp.WAVE_HOM_2D, order, n, n, bc=sbp.BC_CHARACTERISTIC) as c:
        c.set_wait_limit(5_000_000)  # 5 ms: a tile load takes microseconds
        assert relerr(c.rhs(src), expected) <= TOL64
        c.test_drop_tile(tile)
        with pytest.raises(sbp.SbpError) as e:
            c.rhs(src)
        assert e.value.code == sbp.ERR_DEVICE
        assert "timed out" in str(e.value)
        # the same context, the same stream: full results again, the error word cleared
        assert relerr(c.rhs(src), expected) <= TOL64
        c.synchronize()
        h = 2.0 / (n - 1)
        v0 = port.init_wave_pulse(n, n, 0.1, -0.1, 0.1, 1.0)
        assert relerr(c.rk4(v0, 0.0, 0.2 * h, 3), port.rk4(pb, v0, 0.0, 0.2 * h, 3)) <= TOL64


@pytest.mark.gpu
def test_drop_tile_argument_range(sbp):
    with sbp.Context(sbp.WAVE_HOM_2D, 4, 64, 64) as c:
        with pytest.raises(sbp.SbpError) as e:
            c.test_drop_tile(10 ** 6)
        assert e.value.code == sbp.ERR_INVALID
        with pytest.raises(sbp.SbpError):
            c.set_wait_limit(-1)
