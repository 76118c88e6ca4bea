"""The learned correction of the coarse two-layer solve: trained on fine
trajectories this solver generates, it must beat the plain coarse solve on
held-out trajectories; with corrupted weights (injected on the host) the
energy check must reject its corrections and the fine solve must answer."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _small():
    import learned

    return learned.Setup(nxc=65, nbc=33)


def test_learned_correction_beats_plain_coarse_solve(sbp):
    import learned

    s = _small()
    sv = learned.Solvers(s)
    X, Y, scale = learned.make_dataset(sv, range(1000, 1024), windows=6, keep=3)
    with sbp.Cnn(2 * s.nbc, s.nxc, 8) as net:
        losses = learned.train(net, X, Y, epochs=25, batch=8, lr=2e-3)
        assert np.mean(losses[-10:]) < 0.5 * np.mean(losses[:10])
        solver = learned.LearnedSolver(sv, net, scale)
        res = learned.evaluate(sv, solver, range(5000, 5004), windows=6)
    assert np.mean(res["learned"]) < np.mean(res["coarse"])


def test_energy_guard_falls_back_to_fine_solve(sbp):
    import learned

    s = _small()
    sv = learned.Solvers(s)
    with sbp.Cnn(2 * s.nbc, s.nxc, 1) as net:
        p = net.get_params()
        rng = np.random.default_rng(0)
        net.set_params((p + 5.0 * rng.standard_normal(p.size)).astype(np.float32))  # corrupted weights
        solver = learned.LearnedSolver(sv, net, scale=1.0)
        res = learned.evaluate(sv, solver, [5000], windows=3)
    assert solver.fallbacks == 1
    assert res["learned"][0] == 0.0  # the answer came from the fine solve, the judge itself


def test_features_and_zero_state_gives_zero_correction(sbp):
    """Features are (u, v, p, p log(rho)/log 4) / s; a trained network (biases held at zero)
    maps the zero state to an exactly zero correction."""
    import learned
    import torch

    s = _small()
    sv = learned.Solvers(s)
    x0, y0, w, a = learned.trajectory_params(5000)
    st = torch.from_numpy(learned.pulse_state(s.nxc, s.nbc, x0, y0, w, a)).to(sv.dev)
    x = sv.features(st).view(-1, 4).cpu().numpy()
    q = st.view(-1, 3).cpu().numpy()
    rho = sv.rho_c.cpu().numpy()
    expect = np.concatenate([q, (q[:, 2] * np.log(rho) / np.log(4.0))[:, None]], axis=1)
    np.testing.assert_allclose(x, expect.astype(np.float32), rtol=1e-6, atol=1e-30)
    X, Y, scale = learned.make_dataset(sv, range(1000, 1004), windows=4, keep=2)
    with sbp.Cnn(2 * s.nbc, s.nxc, 2) as net:
        learned.train(net, X, Y, epochs=3, batch=2, lr=2e-3)
        zero = torch.zeros(sv.npc * 4, dtype=torch.float32, device=sv.dev)
        out = torch.full((sv.npc * 3,), 7.0, dtype=torch.float32, device=sv.dev)
        net.forward(zero.data_ptr(), 1, out.data_ptr())
        torch.cuda.synchronize()
    assert float(out.abs().max()) == 0.0
