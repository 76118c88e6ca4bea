"""The learned-correction network: the CPU checker (oracle/cnn_oracle.py)
against finite differences, and the GPU kernels (BF16 tcgen05 convolutions --
forward, input gradient, weight gradient -- with FP32 accumulation in tensor
memory) against the checker."""
import numpy as np
import pytest

import cnn_oracle as N


def _small_params(seed):
    rng = np.random.default_rng(seed)
    params = []
    for k, (ci, co, _) in enumerate(N.LAYERS):
        w = rng.standard_normal((co, 9, ci)) * np.sqrt(2.0 / (9 * ci))
        if k == 0:
            w[:, :, N.IN_REAL:] = 0.0
        if k == len(N.LAYERS) - 1:
            w[N.OUT_REAL:] = 0.0
        params.append((w, 0.1 * rng.standard_normal(co)))
    return N.pack(params)


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    vec = _small_params(1)
    x = rng.standard_normal((1, 5, 6, N.IN_REAL))
    t = rng.standard_normal((1, 5, 6, N.OUT_REAL))
    loss, g = N.loss_and_grad(vec, x, t, bf16=False)
    idx = rng.choice(np.flatnonzero(g), size=40, replace=False)
    eps = 1e-6
    for i in idx:
        vp, vm = vec.copy(), vec.copy()
        vp[i] += eps
        vm[i] -= eps
        fd = (N.loss_and_grad(vp, x, t, bf16=False)[0] - N.loss_and_grad(vm, x, t, bf16=False)[0]) / (2 * eps)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(g[i])) + 1e-7


def test_bf16_rounding_is_nearest_even():
    vals = np.array([1.0, 1.0 + 2**-8, 1.0 + 2**-7 + 2**-8, -3.14159, 1e-20])
    r = N.round_bf16(vals)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0 + 2**-6
    assert abs(r[3] + 3.14159) < 0.02 and r[4] != 0.0


def _relerr(a, b):
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-30)


@pytest.mark.gpu
@pytest.mark.parametrize("shape", [(2, 19, 23), (3, 32, 40), (1, 64, 64), (1, 9, 200), (2, 160, 160)],
                         ids=["2x19x23", "3x32x40", "1x64x64", "1x9x200", "2x160x160"])
def test_gpu_forward_and_gradients_match_oracle(sbp, shape):
    """Tolerances from what BF16 storage with FP32 accumulation leaves against the oracle, which
    rounds the same tensors to BF16 and sums in FP64 (measured: output <= 1.9e-3, loss <= 8e-6,
    each layer's weight and bias gradients <= 8e-4, max-norm relative), with a margin of 2.5-6x.
    2 x 160 x 160 has more 128-pixel tiles (400) than the persistent convolutions have CTAs, so
    CTAs take several tiles: ring-slot reuse, both tensor-memory accumulators, and the weight
    gradient's accumulation over tiles are exercised."""
    import torch

    B, H, W = shape
    rng = np.random.default_rng(3 + H)
    x = rng.standard_normal((B, H, W, N.IN_REAL)).astype(np.float32)
    t = rng.standard_normal((B, H, W, 3)).astype(np.float32)
    with sbp.Cnn(H, W, B) as net:
        vec = _small_params(7 + W).astype(np.float32)
        net.set_params(vec)
        dx = torch.from_numpy(x).cuda()
        dt = torch.from_numpy(t).cuda()
        out = torch.empty((B, H, W, 3), dtype=torch.float32, device="cuda")
        net.forward(dx.data_ptr(), B, out.data_ptr())
        loss, g = net.gradients(dx.data_ptr(), dt.data_ptr(), B)
    ref_out, _, _ = N.forward(vec.astype(np.float64), x.astype(np.float64), bf16=True)
    assert _relerr(out.cpu().numpy(), ref_out) < 5e-3
    ref_loss, ref_g = N.loss_and_grad(vec.astype(np.float64), x.astype(np.float64), t.astype(np.float64), bf16=True)
    assert loss == pytest.approx(ref_loss, rel=1e-4)
    o = 0
    for layer, (ci, co, _) in enumerate(N.LAYERS):
        nw = co * 9 * ci
        assert _relerr(g[o:o + nw], ref_g[o:o + nw]) < 5e-3, ("weights", layer)
        assert _relerr(g[o + nw:o + nw + co], ref_g[o + nw:o + nw + co]) < 5e-3, ("bias", layer)
        o += nw + co


@pytest.mark.gpu
def test_gpu_training_fits_a_batch(sbp):
    import torch

    B, H, W = 4, 24, 24
    rng = np.random.default_rng(5)
    x = rng.standard_normal((B, H, W, N.IN_REAL)).astype(np.float32)
    # a target the network can represent: a smoothed function of the inputs
    t = (0.3 * x[..., :3] + 0.1 * np.roll(x[..., 1:4], 1, axis=1)).astype(np.float32)
    with sbp.Cnn(H, W, B) as net:
        dx = torch.from_numpy(x).cuda()
        dt = torch.from_numpy(t).cuda()
        losses = [net.train_step(dx.data_ptr(), dt.data_ptr(), B, 3e-3) for _ in range(300)]
    assert losses[-1] < 0.1 * losses[0]
