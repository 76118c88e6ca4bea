"""Seeded input fields for the wave workloads (host side, numpy).

These produce problem *inputs* (initial data and coefficient fields); they
do no part of the SBP computation, which runs in libsbpgpu.
"""
from __future__ import annotations

import numpy as np


def fourier_field(n: int, seed: int, modes: int = 8, kmax: float = 6.0, xl=(-1.0, -1.0), xr=(1.0, 1.0)):
    """1 + 0.5 * tanh(sum_m A_m cos(k_m . x + phi_m)) on an n x n grid, (j, i) row-major.

    k_m: integer wave vectors, uniform over the nonzero lattice points with
    |k| <= kmax; A_m ~ N(0, 1); phi_m ~ U[0, 2 pi); all drawn from `seed`.
    The range is inside (0.5, 1.5): 1 + 0.5 tanh(.) never reaches 2.
    """
    rng = np.random.default_rng(seed)
    r = int(np.floor(kmax))
    lattice = np.array([(a, b) for a in range(-r, r + 1) for b in range(-r, r + 1)
                        if (a, b) != (0, 0) and a * a + b * b <= kmax * kmax], dtype=np.float64)
    k = lattice[rng.integers(0, len(lattice), size=modes)]
    amp = rng.standard_normal(modes)
    phi = rng.uniform(0.0, 2 * np.pi, size=modes)
    x = np.linspace(xl[0], xr[0], n)
    y = np.linspace(xl[1], xr[1], n)
    X, Y = np.meshgrid(x, y)
    s = np.zeros_like(X)
    for m in range(modes):
        s += amp[m] * np.cos(k[m, 0] * X + k[m, 1] * Y + phi[m])
    return (1.0 + 0.5 * np.tanh(s)).ravel()


def gaussian_pulse(nx: int, ny: int, x0: float = 0.0, y0: float = 0.0, width: float = 0.05, amp: float = 1.0,
                   xl=(-1.0, -1.0), xr=(1.0, 1.0)):
    """Wave state (u, v, p) in the reference's AoS layout: p = amp exp(-|x - x0|^2 / width^2), u = v = 0."""
    x = np.linspace(xl[0], xr[0], nx) - x0
    y = np.linspace(xl[1], xr[1], ny) - y0
    v = np.zeros((ny, nx, 3))
    v[:, :, 2] = amp * np.exp(-(x[None, :] ** 2 + y[:, None] ** 2) / width**2)
    return v.ravel()


def standing_mode(nx: int, ny: int, t: float, n: int = 3, m: int = 4, xl=(-1.0, -1.0), xr=(1.0, 1.0)):
    """Exact solution of the rho = K = 1 wave system with free-surface boundaries (p = 0 on x, y = +-1):
    the standing mode of the reference's wave_hom demo (code/demo/wave_hom/wave_eq_hom_sim.cpp:211-233),
    u = -n cos(n pi x) sin(m pi y) sin(pi w t) / w, v = -m sin(n pi x) cos(m pi y) sin(pi w t) / w,
    p = sin(n pi x) sin(m pi y) cos(pi w t), w = sqrt(n^2 + m^2); AoS (j, i, comp)."""
    x = np.linspace(xl[0], xr[0], nx)[None, :]
    y = np.linspace(xl[1], xr[1], ny)[:, None]
    w = np.sqrt(n * n + m * m)
    out = np.empty((ny, nx, 3))
    out[..., 0] = -n * np.cos(n * np.pi * x) * np.sin(m * np.pi * y) * np.sin(np.pi * w * t) / w
    out[..., 1] = -m * np.sin(n * np.pi * x) * np.cos(m * np.pi * y) * np.sin(np.pi * w * t) / w
    out[..., 2] = np.sin(np.pi * n * x) * np.sin(np.pi * m * y) * np.cos(np.pi * w * t)
    return out.ravel()


def batched_instances(count: int, seed: int = 2):
    """The batched workload: `count` independent instances (512 in the benchmark configuration).
    N = round(exp(U[ln 64, ln 512])) per side, order from {2, 4, 6}, speed c ~ U[0.5, 2];
    even members are waves (rho = 1, K = c^2, characteristic SAT), odd members advection
    with |(a, b)| = c in a random direction; dt = 0.2 h / c; pulses centred in [-0.5, 0.5]^2."""
    import sbpgpu

    rng = np.random.default_rng(seed)
    insts, states = [], []
    for k in range(count):
        nx = int(round(np.exp(rng.uniform(np.log(64), np.log(512)))))
        ny = int(round(np.exp(rng.uniform(np.log(64), np.log(512)))))
        order = int(rng.choice([2, 4, 6]))
        c = float(rng.uniform(0.5, 2.0))
        x0, y0 = rng.uniform(-0.5, 0.5, 2)
        h = min(2.0 / (nx - 1), 2.0 / (ny - 1))
        if k % 2 == 0:
            insts.append(dict(problem=sbpgpu.WAVE_HOM_2D, order=order, nx=nx, ny=ny, c=c, dt=0.2 * h / c,
                              bc=sbpgpu.BC_CHARACTERISTIC))
            states.append(gaussian_pulse(nx, ny, x0, y0, 0.1, 1.0))
        else:
            ang = rng.uniform(0.0, 2 * np.pi)
            insts.append(dict(problem=sbpgpu.ADVECTION_2D, order=order, nx=nx, ny=ny, a=c * np.cos(ang),
                              b=c * np.sin(ang), dt=0.2 * h / c))
            x = np.linspace(-1, 1, nx) - x0
            y = np.linspace(-1, 1, ny) - y0
            states.append(np.exp(-(x[None, :] ** 2 + y[:, None] ** 2) / 0.1**2).ravel())
    return insts, states


def batched_sample(insts, count: int = 16, seed: int = 7):
    """Indices of `count` instances of a batch to check one by one: the smallest and the largest,
    the first wave and the first advection instance of each order, the rest drawn from `seed`."""
    import sbpgpu

    sizes = [d["nx"] * d["ny"] for d in insts]
    pick = [int(np.argmin(sizes)), int(np.argmax(sizes))]
    for o in (2, 4, 6):
        for p in (sbpgpu.WAVE_HOM_2D, sbpgpu.ADVECTION_2D):
            k = next((k for k, d in enumerate(insts) if d["order"] == o and d["problem"] == p), None)
            if k is not None:
                pick.append(k)
    rng = np.random.default_rng(seed)
    for k in rng.permutation(len(insts)):
        if len(set(pick)) >= count:
            break
        pick.append(int(k))
    return sorted(set(pick))[:count]
