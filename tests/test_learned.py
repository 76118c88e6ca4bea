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
    X, Y, scales = learned.make_dataset(sv, range(1000, 1024), windows=6, keep=3)
    with sbp.Cnn(2 * s.nbc, s.nxc, 8) as net:
        losses = learned.train(net, X, Y, epochs=25, batch=8, lr=2e-3)
        assert np.mean(losses[-10:]) < 0.5 * np.mean(losses[:10])
        solver = learned.LearnedSolver(sv, net, scales)
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
        solver = learned.LearnedSolver(sv, net, learned.Scales())
        res = learned.evaluate(sv, solver, [5000], windows=3)
    assert solver.fallbacks == 1
    assert res["learned"][0] == 0.0  # the answer came from the fine solve, the reference itself


def _features_np(q_aos, rho, K, nx, ny, nb):
    """Numpy restatement of sbp_cnn_features (inv_scale 1)."""
    st = q_aos.reshape(ny, nx, 3)
    z = np.sqrt(rho * K).reshape(ny, nx)
    q = np.stack([z * st[..., 0], z * st[..., 1], st[..., 2]], axis=-1)
    f = np.zeros((ny, nx, 24))
    i1 = np.clip(np.arange(nx), 1, nx - 2)
    i2 = np.clip(np.arange(nx), 2, nx - 3)
    f[:, :, 0:3] = q[:, i1 - 1] - 2 * q[:, i1] + q[:, i1 + 1]
    f[:, :, 6:9] = q[:, i2 - 2] - 4 * q[:, i2 - 1] + 6 * q[:, i2] - 4 * q[:, i2 + 1] + q[:, i2 + 2]
    for b in range(ny // nb):
        rows = slice(b * nb, (b + 1) * nb)
        r1 = np.clip(np.arange(nb), 1, nb - 2) + b * nb
        r2 = np.clip(np.arange(nb), 2, nb - 3) + b * nb
        f[rows, :, 3:6] = q[r1 - 1] - 2 * q[r1] + q[r1 + 1]
        f[rows, :, 9:12] = q[r2 - 2] - 4 * q[r2 - 1] + 6 * q[r2] - 4 * q[r2 + 1] + q[r2 + 2]
        f[rows, :, 12:24] = (1.0 if b == 0 else -1.0) * f[rows, :, 0:12]
    return f.reshape(-1, 24)


def test_features_and_zero_state_gives_zero_correction(sbp):
    """Features are undivided second and fourth differences of (Z u, Z v, p) within each block
    plus a layer-tagged copy; a trained network (biases held at zero) maps the zero state to an
    exactly zero correction."""
    import learned
    import torch

    s = _small()
    sv = learned.Solvers(s)
    rng = np.random.default_rng(3)
    st = torch.from_numpy(rng.standard_normal(sv.npc * 3)).to(sv.dev)
    x = sv.features(st).view(-1, 24).cpu().numpy()
    expect = _features_np(st.cpu().numpy(), sv.rho_c.cpu().numpy(), sv.K_c.cpu().numpy(), s.nxc, 2 * s.nbc, s.nbc)
    np.testing.assert_allclose(x, expect.astype(np.float32), rtol=1e-5, atol=1e-5)
    X, Y, scales = learned.make_dataset(sv, range(1000, 1004), windows=4, keep=2)
    with sbp.Cnn(2 * s.nbc, s.nxc, 2) as net:
        learned.train(net, X, Y, epochs=3, batch=2, lr=2e-3)
        zero = torch.zeros(sv.npc * 24, dtype=torch.float32, device=sv.dev)
        out = torch.full((sv.npc * 3,), 7.0, dtype=torch.float32, device=sv.dev)
        torch.cuda.synchronize()
        net.forward(zero.data_ptr(), 1, out.data_ptr())
        torch.cuda.synchronize()
    assert float(out.abs().max()) == 0.0


@pytest.mark.parametrize("shared", [True, False], ids=["net_on_coarse_stream", "net_on_own_stream"])
def test_run_matches_window_by_window_solve(sbp, shared):
    """LearnedSolver.run (state resident in the coarse context, one stream, two host
    waits per window) gives bit for bit the state of the window-by-window path
    (corrected_window), with the network on the coarse context's stream or its own."""
    import learned
    import torch

    s = _small()
    sv = learned.Solvers(s)
    kw = {"stream": sv.stream.cuda_stream} if shared else {}
    with sbp.Cnn(2 * s.nbc, s.nxc, 1, **kw) as net:
        p = net.get_params()
        net.set_params((p + 0.02 * np.random.default_rng(1).standard_normal(p.size)).astype(np.float32))
        solver = learned.LearnedSolver(sv, net, learned.Scales(inp=2.0, out=1e-3), guard=1e9)
        assert solver.shared == shared
        x0, y0, w, a = learned.trajectory_params(5001)
        fine0 = torch.from_numpy(learned.pulse_state(s.nxf, s.nbf, x0, y0, w, a)).to(sv.dev)
        fast = solver.run(fine0, 5)
        state = sv.restrict(fine0)
        for _ in range(5):
            state = solver.corrected_window(state)
        torch.cuda.synchronize()
    assert solver.fallbacks == 0
    assert float((state - sv.restrict(fine0)).abs().max()) > 0.0
    assert torch.equal(fast, state)
