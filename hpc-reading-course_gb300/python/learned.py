"""Learned correction of a coarse two-layer wave solve.

The problem: the two-block acoustic wave system (libsbpgpu's SBP_WAVE_2BLOCK_2D)
with rho = K = 1 below y = 0 and rho = K = 4 above (impedance ratio 4, equal
speeds), characteristic SAT on the outer boundary, energy-conserving interface
SAT, SBP order 4. A fine grid (nx_f = 4 (nx_c - 1) + 1 points per row, the same
in y per block) is nested in a 4x coarser one, so restriction is injection.

Every `window` coarse RK4 steps (4 by default) the network (libsbpgpu's
sbp_cnn_*, BF16 tensor-core convolutions) maps high-pass features of the
coarse state (undivided second and fourth differences of Z u, Z v, p,
Z = sqrt(rho K), computed in FP64) to a correction of Z u, Z v, p towards the
restricted fine solution.

Training: pairs (features of a coarse window's result, restricted fine state
minus that result) from seeded pulse trajectories, first from windows started
on the restricted fine state, then from windows started on the corrected
solve's own states (rollout rounds: the states the solver actually meets,
with targets that pull back to the fine solution). The network has no biases
and ReLU activations, so it is positively homogeneous: scaling a sample's
features and target by the same factor leaves the function to learn
unchanged. Each sample is scaled to unit target RMS, so every trajectory
counts equally in relative terms, as in the relative error it is measured by. A correction that raises
the coarse state's H-norm by more than `guard` (relative) fails the energy
check; then the run falls back to the fine solve: the answer is the fine
solver's, restricted to the coarse grid. The fine solve is also the reference:
errors are measured against the restricted fine solution.

Device memory and small glue operations (restriction by slicing, target
differences) use torch on the GPU; the solves and the network run in libsbpgpu.
The library's contexts and network run on their own streams, so every hand-off
of a device array between torch and the library waits for the producer
(`_ready`).
"""
from __future__ import annotations

import time
from dataclasses import dataclass

import numpy as np
import torch

import sbpgpu


@dataclass
class Setup:
    nxc: int = 257          # coarse points per row
    nbc: int = 129          # coarse points per block column (2 blocks)
    order: int = 4
    ratio: float = 4.0      # rho and K above y = 0 (1 below)
    cfl: float = 0.2
    window: int = 4         # coarse steps between corrections

    @property
    def nxf(self):
        return 4 * (self.nxc - 1) + 1

    @property
    def nbf(self):
        return 4 * (self.nbc - 1) + 1

    @property
    def hc(self):
        return 2.0 / (self.nxc - 1)

    @property
    def hf(self):
        return 2.0 / (self.nxf - 1)

    @property
    def dtc(self):
        return self.cfl * min(self.hc, 1.0 / (self.nbc - 1))

    @property
    def dtf(self):
        return self.dtc / 4


def two_layer_fields(nx: int, nb: int, ratio: float):
    rho = np.ones((2 * nb, nx))
    rho[nb:] = ratio
    return rho.ravel(), rho.ravel().copy()


def pulse_state(nx: int, nb: int, x0: float, y0: float, width: float, amp: float):
    """Gaussian pressure pulse on the two-block grid (AoS u, v, p; the interface line in both blocks)."""
    x = np.linspace(-1, 1, nx)
    y = np.concatenate([np.linspace(-1, 0, nb), np.linspace(0, 1, nb)])
    v = np.zeros((2 * nb, nx, 3))
    v[:, :, 2] = amp * np.exp(-((x[None, :] - x0) ** 2 + (y[:, None] - y0) ** 2) / width**2)
    return v.ravel()


def trajectory_params(seed: int):
    """Pulse position U[-0.5, 0.5]^2, width U[0.02, 0.1], amplitude U[0.5, 2] from `seed`."""
    rng = np.random.default_rng(seed)
    x0, y0 = rng.uniform(-0.5, 0.5, 2)
    return float(x0), float(y0), float(rng.uniform(0.02, 0.1)), float(rng.uniform(0.5, 2.0))


def _ready():
    """Wait for all work on the device (the hand-off point between torch's stream and the
    library's streams)."""
    torch.cuda.synchronize()


class Solvers:
    """The fine and coarse two-block contexts plus device buffers; with `mid`, also a plain solve
    at twice the coarse resolution (for the time-against-error comparison); with `truth`, a solve at
    twice the fine resolution that stands in for the exact solution when the fine solve's own error
    is measured."""

    def __init__(self, s: Setup, device: int = 0, mid: bool = False, truth: bool = False):
        self.s = s
        self.dev = torch.device(f"cuda:{device}")
        rf, kf = two_layer_fields(s.nxf, s.nbf, s.ratio)
        rc, kc = two_layer_fields(s.nxc, s.nbc, s.ratio)
        bc = sbpgpu.BC_CHARACTERISTIC
        self.fine = sbpgpu.Context(sbpgpu.WAVE_2BLOCK_2D, s.order, s.nxf, 2 * s.nbf, rho=rf, K=kf, bc=bc,
                                   device=device)
        # the coarse context runs on this stream; a network created on it (Cnn(stream=
        # stream.cuda_stream)) lets the corrected solve run without host syncs between
        # its steps, features, network and correction
        self.stream = torch.cuda.Stream(device=self.dev)
        self.coarse = sbpgpu.Context(sbpgpu.WAVE_2BLOCK_2D, s.order, s.nxc, 2 * s.nbc, rho=rc, K=kc, bc=bc,
                                     stream=self.stream.cuda_stream, device=device)
        self.mid = None
        if mid:
            nxm, nbm = 2 * (s.nxc - 1) + 1, 2 * (s.nbc - 1) + 1
            rm, km = two_layer_fields(nxm, nbm, s.ratio)
            self.mid = sbpgpu.Context(sbpgpu.WAVE_2BLOCK_2D, s.order, nxm, 2 * nbm, rho=rm, K=km, bc=bc,
                                      device=device)
            self.mid_shape = (nxm, nbm)
        self.truth = None
        if truth:
            nxt, nbt = 2 * (s.nxf - 1) + 1, 2 * (s.nbf - 1) + 1
            rt, kt = two_layer_fields(nxt, nbt, s.ratio)
            self.truth = sbpgpu.Context(sbpgpu.WAVE_2BLOCK_2D, s.order, nxt, 2 * nbt, rho=rt, K=kt, bc=bc,
                                        device=device)
            self.truth_shape = (nxt, nbt)
        self.rho_c = torch.from_numpy(rc).to(self.dev)
        self.K_c = torch.from_numpy(kc).to(self.dev)
        self.npc = s.nxc * 2 * s.nbc

    # -- state movement (AoS FP64 device tensors)
    def fine_state(self):
        out = torch.empty(self.s.nxf * 2 * self.s.nbf * 3, dtype=torch.float64, device=self.dev)
        self.fine.get_state_ptr(out.data_ptr(), sbpgpu.DEVICE)
        return out

    def coarse_state(self):
        out = torch.empty(self.npc * 3, dtype=torch.float64, device=self.dev)
        self.coarse.get_state_ptr(out.data_ptr(), sbpgpu.DEVICE)
        return out

    def restrict(self, fine_aos):
        s = self.s
        f = fine_aos.view(2, s.nbf, s.nxf, 3)
        return f[:, ::4, ::4, :].contiguous().view(-1)

    def coarse_steps(self, state, n):
        _ready()
        self.coarse.set_state_ptr(state.data_ptr(), sbpgpu.DEVICE)
        self.coarse.step_resident(0.0, self.s.dtc, n)
        self.coarse.synchronize()
        return self.coarse_state()

    def fine_steps_from(self, fine_state, n):
        _ready()
        self.fine.set_state_ptr(fine_state.data_ptr(), sbpgpu.DEVICE)
        self.fine.step_resident(0.0, self.s.dtf, n)
        self.fine.synchronize()
        return self.fine_state()

    def mid_solve(self, fine_aos, windows: int):
        """Plain solve at twice the coarse resolution from the fine state (restricted by 2), over
        `windows` coarse windows, restricted to the coarse grid."""
        s = self.s
        nxm, nbm = self.mid_shape
        st = fine_aos.view(2, s.nbf, s.nxf, 3)[:, ::2, ::2, :].contiguous().view(-1)
        _ready()
        self.mid.set_state_ptr(st.data_ptr(), sbpgpu.DEVICE)
        self.mid.step_resident(0.0, s.dtc / 2, 2 * s.window * windows)
        self.mid.synchronize()
        out = torch.empty(nxm * 2 * nbm * 3, dtype=torch.float64, device=self.dev)
        self.mid.get_state_ptr(out.data_ptr(), sbpgpu.DEVICE)
        return out.view(2, nbm, nxm, 3)[:, ::2, ::2, :].contiguous().view(-1)

    def truth_solve(self, params, windows: int):
        """The pulse of `params` (trajectory_params) sampled on the truth grid, solved over `windows`
        coarse windows at a quarter of the fine step, restricted to the coarse grid (every 8th point)."""
        s = self.s
        nxt, nbt = self.truth_shape
        x0, y0, w, a = params
        st = torch.from_numpy(pulse_state(nxt, nbt, x0, y0, w, a)).to(self.dev)
        _ready()
        self.truth.set_state_ptr(st.data_ptr(), sbpgpu.DEVICE)
        self.truth.step_resident(0.0, s.dtf / 2, 8 * s.window * windows)
        self.truth.synchronize()
        out = torch.empty(nxt * 2 * nbt * 3, dtype=torch.float64, device=self.dev)
        self.truth.get_state_ptr(out.data_ptr(), sbpgpu.DEVICE)
        return out.view(2, nbt, nxt, 3)[:, ::8, ::8, :].contiguous().view(-1)

    def features(self, coarse_aos, inv_scale: float = 1.0):
        s = self.s
        x = torch.empty(self.npc * 24, dtype=torch.float32, device=self.dev)
        _ready()
        sbpgpu.cnn_features(coarse_aos.data_ptr(), self.rho_c.data_ptr(), self.K_c.data_ptr(), s.nxc, 2 * s.nbc,
                            s.nbc, inv_scale, x.data_ptr())
        _ready()
        return x

    def to_q(self, coarse_aos):
        """(Z u, Z v, p) of an AoS coarse state, Z = sqrt(rho K): the variables the network corrects."""
        z = (self.rho_c * self.K_c).sqrt()
        q = coarse_aos.view(-1, 3).clone()
        q[:, 0] *= z
        q[:, 1] *= z
        return q.view(-1)


@dataclass
class Scales:
    """Feature scale (features are divided by it) and correction scale (outputs are in its units)."""
    inp: float = 1.0
    out: float = 1.0


def collect(sv: Solvers, seeds, windows: int, keep: int | None = None, solver: "LearnedSolver | None" = None):
    """Raw pairs (features of the coarse state after one window, restricted fine state minus that
    coarse state in Z u, Z v, p). Each trajectory runs `windows` windows of the fine solve; `keep`
    of them (drawn from the trajectory's seed; all if None) become samples, so the samples cover
    the whole horizon the solver is used on. Without `solver` every window starts on the
    restricted fine state; with one, windows start on the corrected solve's own state (the
    restricted fine state again where a correction fails the energy check)."""
    s = sv.s
    xs, ys = [], []
    fine_steps = 4 * s.window
    for seed in seeds:
        x0, y0, w, a = trajectory_params(seed)
        picks = set(range(windows)) if keep is None else set(
            np.random.default_rng(seed + 7).choice(windows, size=keep, replace=False).tolist())
        fine = torch.from_numpy(pulse_state(s.nxf, s.nbf, x0, y0, w, a)).to(sv.dev)
        state = sv.restrict(fine)
        last = max(picks) if picks else -1
        for k in range(last + 1):
            if solver is None and k not in picks:
                fine = sv.fine_steps_from(fine, fine_steps)
                continue
            start = sv.restrict(fine) if solver is None else state
            pred = sv.coarse_steps(start, s.window)
            fine = sv.fine_steps_from(fine, fine_steps)
            target = sv.restrict(fine)
            if k in picks:
                xs.append(sv.features(pred))
                ys.append((sv.to_q(target) - sv.to_q(pred)).to(torch.float32))
            if solver is not None:
                corrected = solver.correct(pred)
                state = target if corrected is None else corrected
    return torch.stack(xs), torch.stack(ys)


def normalize(X, Y, scales: Scales | None = None):
    """Scale each sample to unit target RMS (valid for the homogeneous network; the floor keeps
    near-zero targets from dominating), then features and targets by the set's RMS (`scales`,
    computed when None). Returns (X, Y, scales)."""
    a = Y.square().mean(dim=1).sqrt()
    a = torch.clamp(a, min=max(1e-3 * float(a.median()), 1e-30))[:, None]
    X = X / a
    Y = Y / a
    if scales is None:
        scales = Scales(inp=float(X.square().mean().sqrt()) or 1.0, out=float(Y.square().mean().sqrt()) or 1.0)
    return X / scales.inp, Y / scales.out, scales


def make_dataset(sv: Solvers, seeds, windows: int, keep: int | None = None):
    """Windows started on the restricted fine state, normalized: (X, Y, Scales)."""
    return normalize(*collect(sv, seeds, windows, keep))


def train(net: sbpgpu.Cnn, X, Y, *, epochs: int, batch: int, lr: float, seed: int = 0):
    """Adam over shuffled minibatches, learning rate decayed from `lr` to `lr`/10 on a cosine;
    returns the loss history (one entry per step)."""
    n = X.shape[0]
    g = torch.Generator(device="cpu").manual_seed(seed)
    total = epochs * (n // batch)
    losses = []
    for _ in range(epochs):
        perm = torch.randperm(n, generator=g)
        for k in range(0, n - batch + 1, batch):
            idx = perm[k:k + batch].to(X.device)
            xb = X.index_select(0, idx).contiguous()
            yb = Y.index_select(0, idx).contiguous()
            _ready()
            frac = len(losses) / max(total, 1)
            step_lr = lr * (0.1 + 0.45 * (1.0 + np.cos(np.pi * frac)))
            losses.append(net.train_step(xb.data_ptr(), yb.data_ptr(), batch, step_lr))
    return losses


class LearnedSolver:
    """Coarse solve corrected by the network every window, with the energy check."""

    def __init__(self, sv: Solvers, net: sbpgpu.Cnn, scales: Scales, guard: float = 0.01):
        self.sv, self.net, self.scales, self.guard = sv, net, scales, guard
        self.delta = torch.empty(sv.npc * 3, dtype=torch.float32, device=sv.dev)
        self.pred = torch.empty(sv.npc * 3, dtype=torch.float64, device=sv.dev)
        self.x = torch.empty(sv.npc * 24, dtype=torch.float32, device=sv.dev)
        self.shared = getattr(net, "stream", None) == sv.stream.cuda_stream
        self.fallbacks = 0

    def hnorm(self, state):
        _ready()
        self.sv.coarse.set_state_ptr(state.data_ptr(), sbpgpu.DEVICE)
        return self.sv.coarse.hnorm()

    def corrected_window(self, state):
        """One window of the corrected coarse solve; None if the correction fails the energy check."""
        return self.correct(self.sv.coarse_steps(state, self.sv.s.window))

    def correct(self, pred):
        """The network's correction of a coarse window's result; None if it fails the energy check."""
        sv = self.sv
        x = sv.features(pred, 1.0 / self.scales.inp)
        self.net.forward(x.data_ptr(), 1, self.delta.data_ptr())
        e0 = self.hnorm(pred)
        corrected = pred.clone()
        _ready()
        sbpgpu.cnn_correct(corrected.data_ptr(), self.delta.data_ptr(), sv.rho_c.data_ptr(), sv.K_c.data_ptr(), sv.npc,
                           self.scales.out)
        torch.cuda.synchronize()
        e1 = self.hnorm(corrected)
        if not np.isfinite(e1) or e1 > e0 * (1.0 + self.guard):
            return None
        return corrected

    def run(self, fine0, windows: int):
        """`windows` corrected windows from the fine initial state `fine0` (restricted); if a
        correction fails the energy check, the fine solve from `fine0` gives the answer.
        The state stays in the coarse context between windows and all work is ordered on
        its stream: the host waits only for the two H-norms of the energy check (and around
        the network when that runs on another stream). The same operations as
        corrected_window, so the same results."""
        sv, s = self.sv, self.sv.s
        ctx, S = sv.coarse, sv.stream
        _ready()
        with torch.cuda.stream(S):
            start = sv.restrict(fine0)
            ctx.set_state_ptr(start.data_ptr(), sbpgpu.DEVICE)
            for _ in range(windows):
                ctx.step_resident(0.0, s.dtc, s.window)
                e0 = ctx.hnorm()
                ctx.get_state_ptr(self.pred.data_ptr(), sbpgpu.DEVICE)
                sbpgpu.cnn_features(self.pred.data_ptr(), sv.rho_c.data_ptr(), sv.K_c.data_ptr(), s.nxc, 2 * s.nbc,
                                    s.nbc, 1.0 / self.scales.inp, self.x.data_ptr(), S.cuda_stream)
                if not self.shared:
                    S.synchronize()
                self.net.forward(self.x.data_ptr(), 1, self.delta.data_ptr())
                if not self.shared:
                    _ready()
                sbpgpu.cnn_correct(self.pred.data_ptr(), self.delta.data_ptr(), sv.rho_c.data_ptr(), sv.K_c.data_ptr(),
                                   sv.npc, self.scales.out, S.cuda_stream)
                ctx.set_state_ptr(self.pred.data_ptr(), sbpgpu.DEVICE)
                e1 = ctx.hnorm()
                if not np.isfinite(e1) or e1 > e0 * (1.0 + self.guard):
                    break
            else:
                out = self.pred.clone()
                S.synchronize()
                return out
        self.fallbacks += 1
        return sv.restrict(sv.fine_steps_from(fine0, 4 * s.window * windows))

    def run_plain(self, fine0, windows: int):
        """The coarse solve without corrections."""
        sv, s = self.sv, self.sv.s
        return sv.coarse_steps(sv.restrict(fine0), s.window * windows)


def evaluate(sv: Solvers, solver: LearnedSolver, seeds, windows: int):
    """Relative L2 errors against the restricted fine solution after `windows` windows, for
    the plain coarse solve and the corrected one (and the plain solve at twice the coarse
    resolution, if `sv` has it), and the wall time of each form. If `sv` has the truth solve, also
    every form's error, the fine solve's included, against it on the coarse grid points
    (out["vs_truth"])."""
    s = sv.s
    out = {"coarse": [], "learned": [], "mid": [], "t_fine": 0.0, "t_coarse": 0.0, "t_learned": 0.0, "t_mid": 0.0,
           "vs_truth": {"coarse": [], "learned": [], "mid": [], "fine": []}}
    forms = [("coarse", solver.run_plain), ("learned", solver.run)]
    if sv.mid is not None:
        forms.append(("mid", sv.mid_solve))
    for seed in seeds:
        x0, y0, w, a = trajectory_params(seed)
        fine0 = torch.from_numpy(pulse_state(s.nxf, s.nbf, x0, y0, w, a)).to(sv.dev)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        fine = sv.fine_steps_from(fine0, 4 * s.window * windows)
        out["t_fine"] += time.perf_counter() - t0
        ref = sv.restrict(fine)
        truth = sv.truth_solve((x0, y0, w, a), windows) if sv.truth is not None else None
        if truth is not None:
            out["vs_truth"]["fine"].append(float(torch.linalg.norm(ref - truth) / torch.linalg.norm(truth)))
        for key, fn in forms:
            t0 = time.perf_counter()
            st = fn(fine0, windows)
            torch.cuda.synchronize()
            out["t_" + key] += time.perf_counter() - t0
            out[key].append(float(torch.linalg.norm(st - ref) / torch.linalg.norm(ref)))
            if truth is not None:
                out["vs_truth"][key].append(float(torch.linalg.norm(st - truth) / torch.linalg.norm(truth)))
    return out
