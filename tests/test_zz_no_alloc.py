"""sbp_wave_rhs_noalloc: the wave RHS for callers that cannot allocate device memory.

Such callers -- a host framework that owns all device memory through its own
pool, or a latency-bound loop that cannot take cudaMalloc's device
synchronisation -- cannot create a context (sbp_create allocates). The entry
point keeps its scratch in a static device array instead, and must give what
sbp_rhs and the oracle give. Two calls in a row on different grids check that
the contents the first call leaves in the shared array do not leak into the
second.

This file is collected last so a run that stops at the first failure has run
every other test before it.
"""
import numpy as np
import pytest

TOL64 = 1e-12  # the FP64 parity tolerance of tests/test_gpu_parity.py


def relerr(a, b):
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


def test_noalloc_rejects_grids_beyond_the_static_scratch(sbp):
    # roundup(257, 64) * 256 = 81920 > SBP_NOALLOC_MAX_PLANE: rejected before any GPU work
    rc = sbp.wave_rhs_noalloc(4, 257, 256, 0.0, 1, 1)
    assert rc == sbp.ERR_TOO_LARGE
    assert sbp.wave_rhs_noalloc(5, 64, 64, 0.0, 1, 1) == sbp.ERR_INVALID
    assert sbp.wave_rhs_noalloc(4, 64, 64, 0.0, 0, 0) == sbp.ERR_INVALID


@pytest.mark.gpu
def test_noalloc_matches_sbp_rhs_on_two_calls_in_a_row(sbp, port):
    import torch

    import oracle as O

    rng = np.random.default_rng(2026)
    cases = [  # (order, nx, ny, bc): a larger grid first, then a smaller one
        (4, 256, 256, sbp.BC_REFERENCE),
        (6, 97, 61, sbp.BC_CHARACTERISTIC),
    ]
    for order, nx, ny, bc in cases:
        src = rng.standard_normal(3 * nx * ny)
        with sbp.Context(sbp.WAVE_HOM_2D, order, nx, ny, bc=bc) as ctx:
            expected = ctx.rhs(src, 0.25)
        d_src = torch.from_numpy(src).to("cuda:0")
        d_dst = torch.full_like(d_src, float("nan"))
        torch.cuda.synchronize()
        rc = sbp.wave_rhs_noalloc(order, nx, ny, 0.25, d_src.data_ptr(), d_dst.data_ptr(), bc=bc)
        assert rc == sbp.OK
        got = d_dst.cpu().numpy()
        assert np.isfinite(got).all()
        assert relerr(got, expected) <= TOL64
        obc = O.BC_CHARACTERISTIC if bc == sbp.BC_CHARACTERISTIC else O.BC_REFERENCE
        assert relerr(got, port.rhs(O.Problem(O.WAVE_HOM_2D, order, nx, ny, bc=obc), src, 0.25)) <= TOL64
