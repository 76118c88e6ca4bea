"""ctypes access to the two CPU checkers. TEST INFRASTRUCTURE ONLY.

* ``Port`` loads ``oracle/_build/libsbporacle.so`` -- the C restatement of the
  reference's hot path (oracle/sbp_oracle.c).
* ``Reference`` loads ``oracle/_ref/libsbpref.so`` -- the reference's own
  header-only operators and RHS kernels compiled against two shims
  (oracle/ref_capi.cpp). It exists only where the reference checkout was
  present at build time.

Only tests/, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg
import this module. Arrays are numpy float64 in the reference's AoS layout
(element (j, i, comp) at dofs*(i + nx*j) + comp).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "_build", "libsbporacle.so")
PORT_OPT_SO = os.path.join(HERE, "_build", "libsbporacle_opt.so")  # -O3 -ffast-math: timing only
REF_SO = os.path.join(HERE, "_ref", "libsbpref.so")

WAVE_HOM_2D, WAVE_MMS_2D, ADVECTION_1D, ADVECTION_2D, REFLECTION_1D, WAVE_VAR_2D = 1, 2, 3, 4, 5, 6
WAVE_2BLOCK_2D = 7
WAVE_3D = 8
BC_REFERENCE, BC_CHARACTERISTIC = 0, 1
DOFS = {WAVE_HOM_2D: 3, WAVE_MMS_2D: 3, WAVE_VAR_2D: 3, ADVECTION_1D: 1, ADVECTION_2D: 1, REFLECTION_1D: 2,
        WAVE_2BLOCK_2D: 3, WAVE_3D: 4}
TWO_D = {WAVE_HOM_2D, WAVE_MMS_2D, WAVE_VAR_2D, ADVECTION_2D, WAVE_2BLOCK_2D}

_dp = C.POINTER(C.c_double)


def _ptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_dp)


class _Problem(C.Structure):
    _fields_ = [("problem", C.c_int), ("order", C.c_int), ("bc", C.c_int),
                ("nx", C.c_longlong), ("ny", C.c_longlong),
                ("hix", C.c_double), ("hiy", C.c_double),
                ("xl0", C.c_double), ("xl1", C.c_double),
                ("a", C.c_double), ("b", C.c_double),
                ("rho", _dp), ("K", _dp),
                ("nz", C.c_longlong), ("hiz", C.c_double), ("xl2", C.c_double),
                ("va", _dp), ("vb", _dp)]


def reference_dir() -> str | None:
    """Where the reference checkout is, if anywhere: $REF_DIR, else baseline/_ref/
    beside the repository, else the container's checkout. None when none holds the
    reference's hot-path headers (the GPU machine has none)."""
    root = os.path.dirname(HERE)
    for cand in (os.environ.get("REF_DIR"), os.path.join(root, "baseline", "_ref"), "/root/reference"):
        if cand and os.path.isdir(os.path.join(cand, "code", "include", "sbpops")):
            return cand
    return None


def build(ref_dir: str | None = None, quiet: bool = True) -> None:
    """Build the port (always) and oracle/_ref (when the reference checkout exists)."""
    args = ["make", "-s", "-C", HERE, "-j8", "all"]
    if ref_dir:
        args.append(f"REF_DIR={ref_dir}")
    subprocess.run(args, check=True, stdout=subprocess.DEVNULL if quiet else None)


class Problem:
    """A grid problem on [xl, xr]^d with N points per direction, h = (xr-xl)/(N-1)."""

    def __init__(self, problem: int, order: int, nx: int, ny: int = 1, nz: int = 1, *, xl=(-1.0, -1.0, -1.0),
                 xr=(1.0, 1.0, 1.0), a: float = 1.0, b: float = 0.0, bc: int = BC_REFERENCE, rho=None, K=None,
                 a_field=None, b_field=None):
        self.problem, self.order, self.bc = problem, order, bc
        self.nx, self.ny = nx, (ny if problem in TWO_D or problem == WAVE_3D else 1)
        self.nz = nz if problem == WAVE_3D else 1
        xl, xr = tuple(xl) + (-1.0,) * (3 - len(xl)), tuple(xr) + (1.0,) * (3 - len(xr))
        self.xl, self.xr = xl, xr
        self.hix = (nx - 1) / (xr[0] - xl[0])
        self.hiy = (self.ny - 1) / (xr[1] - xl[1]) if problem in TWO_D or problem == WAVE_3D else 1.0
        self.hiz = (self.nz - 1) / (xr[2] - xl[2]) if problem == WAVE_3D else 1.0
        if problem == WAVE_2BLOCK_2D:  # each block: ny/2 points over half of [xl1, xr1]
            self.hiy = (self.ny // 2 - 1) / ((xr[1] - xl[1]) / 2)
        self.a, self.b = a, b
        self.rho = None if rho is None else np.ascontiguousarray(rho, dtype=np.float64).ravel()
        self.K = None if K is None else np.ascontiguousarray(K, dtype=np.float64).ravel()
        # advection: the velocity at every point (the reference's a(i) / a(i,j), b(i,j))
        self.a_field = None if a_field is None else np.ascontiguousarray(a_field, dtype=np.float64).ravel()
        self.b_field = None if b_field is None else np.ascontiguousarray(b_field, dtype=np.float64).ravel()
        self.dofs = DOFS[problem]

    @property
    def size(self) -> int:
        return self.nx * self.ny * self.nz * self.dofs

    def c_struct(self) -> _Problem:
        s = _Problem(self.problem, self.order, self.bc, self.nx, self.ny, self.hix, self.hiy,
                     self.xl[0], self.xl[1], self.a, self.b, None, None, self.nz, self.hiz, self.xl[2])
        if self.rho is not None:
            s.rho = _ptr(self.rho)
            s.K = _ptr(self.K)
        if self.a_field is not None:
            s.va = _ptr(self.a_field)
        if self.b_field is not None:
            s.vb = _ptr(self.b_field)
        return s


class Rk45Opts(C.Structure):
    _fields_ = [("atol", C.c_double), ("rtol", C.c_double), ("safety", C.c_double), ("reject_safety", C.c_double),
                ("clip_lo", C.c_double), ("clip_hi", C.c_double), ("dt_min", C.c_double), ("dt_max", C.c_double),
                ("max_steps", C.c_longlong), ("max_reject", C.c_int)]


class Rk45Stats(C.Structure):
    _fields_ = [("accepted", C.c_longlong), ("rejected", C.c_longlong), ("t", C.c_double), ("dt_next", C.c_double),
                ("wlte", C.c_double), ("status", C.c_int)]


class Port:
    """The C restatement (oracle/sbp_oracle.c)."""

    def __init__(self, path: str = PORT_SO):
        if not os.path.exists(path):
            build()
        L = self.lib = C.CDLL(path)
        P = C.POINTER(_Problem)
        for name in ("orc_apply", "orc_rhs"):
            getattr(L, name).argtypes = [P, C.c_double, _dp, _dp]
            getattr(L, name).restype = C.c_int
        L.orc_bc.argtypes = [P, _dp, _dp]
        L.orc_rk4.argtypes = [P, C.c_double, C.c_double, C.c_longlong, _dp]
        L.orc_rk45_default_opts.argtypes = [C.POINTER(Rk45Opts)]
        L.orc_rk45_default_opts.restype = None
        L.orc_rk45.argtypes = [P, C.c_double, C.c_double, C.c_double, C.POINTER(Rk45Opts), _dp,
                               C.POINTER(Rk45Stats)]
        L.orc_rk4_nsteps.argtypes = [C.c_double, _dp]
        L.orc_rk4_nsteps.restype = C.c_longlong
        L.orc_hnorm1d_reference.argtypes = [_dp, C.c_longlong, C.c_longlong, C.c_double, C.c_int]
        L.orc_hnorm1d_reference.restype = C.c_double
        L.orc_hnorm.argtypes = [_dp, C.c_longlong, C.c_longlong, C.c_longlong, C.c_double, C.c_double, C.c_int]
        L.orc_hnorm.restype = C.c_double
        L.orc_hnorm_2block.argtypes = L.orc_hnorm.argtypes
        L.orc_hnorm3d.argtypes = [_dp] + [C.c_longlong] * 4 + [C.c_double] * 3 + [C.c_int]
        L.orc_hnorm3d.restype = C.c_double
        L.orc_init_wave3d_mode.argtypes = [_dp] + [C.c_longlong] * 3 + [C.c_double] * 6 + [C.c_int] * 3 + \
            [C.c_double]
        L.orc_hnorm_2block.restype = C.c_double
        L.orc_error_l2.argtypes = [_dp, _dp, C.c_longlong, C.c_double]
        L.orc_error_l2.restype = C.c_double
        L.orc_error_max.argtypes = [_dp, _dp, C.c_longlong]
        L.orc_error_max.restype = C.c_double
        L.orc_init_adv1d.argtypes = [_dp, C.c_longlong] + [C.c_double] * 4
        L.orc_init_adv2d.argtypes = [_dp, C.c_longlong, C.c_longlong] + [C.c_double] * 7
        L.orc_init_wave_mms.argtypes = [_dp, C.c_longlong, C.c_longlong] + [C.c_double] * 5
        L.orc_init_reflection.argtypes = [_dp, C.c_longlong] + [C.c_double] * 4
        L.orc_init_wave_pulse.argtypes = [_dp, C.c_longlong, C.c_longlong] + [C.c_double] * 8
        L.orc_set_threads.argtypes = [C.c_int]
        L.orc_get_threads.restype = C.c_int

    def _call3(self, fn, pb: Problem, t, src):
        src = np.ascontiguousarray(src, dtype=np.float64)
        dst = np.zeros_like(src)
        s = pb.c_struct()
        rc = fn(C.byref(s), t, _ptr(src), _ptr(dst))
        if rc:
            raise ValueError(f"oracle rejected the problem (code {rc})")
        return dst

    def apply(self, pb: Problem, src, t: float = 0.0):
        return self._call3(self.lib.orc_apply, pb, t, src)

    def rhs(self, pb: Problem, src, t: float = 0.0):
        return self._call3(self.lib.orc_rhs, pb, t, src)

    def bc(self, pb: Problem, src, dst):
        src = np.ascontiguousarray(src, dtype=np.float64)
        out = np.array(dst, dtype=np.float64, copy=True)
        s = pb.c_struct()
        rc = self.lib.orc_bc(C.byref(s), _ptr(src), _ptr(out))
        if rc:
            raise ValueError(f"oracle rejected the problem (code {rc})")
        return out

    def rk4(self, pb: Problem, v, t0: float, dt: float, nsteps: int):
        out = np.array(v, dtype=np.float64, copy=True)
        s = pb.c_struct()
        rc = self.lib.orc_rk4(C.byref(s), t0, dt, nsteps, _ptr(out))
        if rc:
            raise ValueError(f"oracle rejected the problem (code {rc})")
        return out

    def rk45(self, pb: Problem, v, t0: float, t_end: float, dt0: float, **opts):
        """Adaptive RKF45 from t0 to t_end (orc_rk45); opts override the defaults.
        Returns (state, stats dict)."""
        o = Rk45Opts()
        self.lib.orc_rk45_default_opts(C.byref(o))
        for k, val in opts.items():
            setattr(o, k, val)
        out = np.array(v, dtype=np.float64, copy=True)
        st = Rk45Stats()
        s = pb.c_struct()
        rc = self.lib.orc_rk45(C.byref(s), t0, t_end, dt0, C.byref(o), _ptr(out), C.byref(st))
        if rc:
            raise ValueError(f"oracle rejected the problem (code {rc})")
        return out, {f: getattr(st, f) for f, _ in Rk45Stats._fields_}

    def rk4_nsteps(self, t_end: float, dt: float):
        d = C.c_double(dt)
        n = self.lib.orc_rk4_nsteps(t_end, C.byref(d))
        return n, d.value

    def hnorm1d_reference(self, v, n, dofs, h, order):
        v = np.ascontiguousarray(v, dtype=np.float64)
        return self.lib.orc_hnorm1d_reference(_ptr(v), n, dofs, h, order)

    def hnorm(self, v, nx, ny, dofs, hx, hy, order):
        v = np.ascontiguousarray(v, dtype=np.float64)
        return self.lib.orc_hnorm(_ptr(v), nx, ny, dofs, hx, hy, order)

    def hnorm3d(self, v, nx, ny, nz, dofs, hx, hy, hz, order):
        v = np.ascontiguousarray(v, dtype=np.float64)
        return self.lib.orc_hnorm3d(_ptr(v), nx, ny, nz, dofs, hx, hy, hz, order)

    def hnorm_2block(self, v, nx, ny, dofs, hx, hy, order):
        v = np.ascontiguousarray(v, dtype=np.float64)
        return self.lib.orc_hnorm_2block(_ptr(v), nx, ny, dofs, hx, hy, order)

    def error_l2(self, v1, v2, hprod):
        v1 = np.ascontiguousarray(v1, dtype=np.float64)
        v2 = np.ascontiguousarray(v2, dtype=np.float64)
        return self.lib.orc_error_l2(_ptr(v1), _ptr(v2), v1.size, hprod)

    def error_max(self, v1, v2):
        v1 = np.ascontiguousarray(v1, dtype=np.float64)
        v2 = np.ascontiguousarray(v2, dtype=np.float64)
        return self.lib.orc_error_max(_ptr(v1), _ptr(v2), v1.size)

    # initial / exact data of the reference demos
    def init_adv1d(self, n, a, t, xl=-1.0, xr=1.0):
        v = np.zeros(n)
        self.lib.orc_init_adv1d(_ptr(v), n, xl, (xr - xl) / (n - 1), a, t)
        return v

    def init_adv2d(self, nx, ny, a, b, t):
        v = np.zeros(nx * ny)
        self.lib.orc_init_adv2d(_ptr(v), nx, ny, -1.0, -1.0, 2.0 / (nx - 1), 2.0 / (ny - 1), a, b, t)
        return v

    def init_wave_mms(self, nx, ny, t):
        v = np.zeros(nx * ny * 3)
        self.lib.orc_init_wave_mms(_ptr(v), nx, ny, -1.0, -1.0, 2.0 / (nx - 1), 2.0 / (ny - 1), t)
        return v

    def init_reflection(self, n, t, W=2.0):
        v = np.zeros(2 * n)
        self.lib.orc_init_reflection(_ptr(v), n, -1.0, 2.0 / (n - 1), t, W)
        return v

    def init_wave_pulse(self, nx, ny, x0=0.0, y0=0.0, w=0.05, amp=1.0):
        v = np.zeros(nx * ny * 3)
        self.lib.orc_init_wave_pulse(_ptr(v), nx, ny, -1.0, -1.0, 2.0 / (nx - 1), 2.0 / (ny - 1), x0, y0, w, amp)
        return v

    def init_wave3d_mode(self, nx, ny, nz, t, a=1, b=2, c=2):
        """Standing mode on [-1, 1]^3 with p = 0 on the faces (orc_init_wave3d_mode)."""
        v = np.zeros(nx * ny * nz * 4)
        self.lib.orc_init_wave3d_mode(_ptr(v), nx, ny, nz, -1.0, -1.0, -1.0, 2.0 / (nx - 1), 2.0 / (ny - 1),
                                      2.0 / (nz - 1), a, b, c, t)
        return v

    def set_threads(self, n: int):
        self.lib.orc_set_threads(n)

    def threads(self) -> int:
        return self.lib.orc_get_threads()


class Reference:
    """The reference's own headers compiled as oracle/_ref/libsbpref.so."""

    def __init__(self, path: str = REF_SO):
        self.lib = C.CDLL(path)
        L = self.lib
        for o in (2, 4, 6):
            for n in ("ref_wave_hom_apply", "ref_wave_apply"):
                getattr(L, f"{n}_o{o}").argtypes = [C.c_longlong, C.c_longlong] + [C.c_double] * 5 + [_dp, _dp]
            for n in ("ref_wave_hom_bc", "ref_wave_bc"):
                getattr(L, f"{n}_o{o}").argtypes = [C.c_longlong, C.c_longlong, C.c_double, C.c_double, _dp, _dp]
            for n in ("ref_adv1d_apply", "ref_adv1d_bc"):
                getattr(L, f"{n}_o{o}").argtypes = [C.c_longlong, C.c_double, C.c_double, _dp, _dp]
            for n in ("ref_adv2d_apply", "ref_adv2d_bc"):
                getattr(L, f"{n}_o{o}").argtypes = [C.c_longlong, C.c_longlong] + [C.c_double] * 4 + [_dp, _dp]
            for n in ("ref_adv1d_apply_var", "ref_adv1d_bc_var"):
                getattr(L, f"{n}_o{o}").argtypes = [C.c_longlong, C.c_double, _dp, _dp, _dp]
            for n in ("ref_adv2d_apply_var", "ref_adv2d_bc_var"):
                getattr(L, f"{n}_o{o}").argtypes = [C.c_longlong, C.c_longlong, C.c_double, C.c_double, _dp, _dp,
                                                     _dp, _dp]
            getattr(L, f"ref_refl_apply_o{o}").argtypes = [C.c_longlong, C.c_double, _dp, _dp]
            getattr(L, f"ref_refl_bc_o{o}").argtypes = [C.c_longlong, _dp, _dp]
            getattr(L, f"ref_hnorm1d_o{o}").argtypes = [C.c_longlong, C.c_longlong, C.c_double, _dp]
            getattr(L, f"ref_hnorm1d_o{o}").restype = C.c_double

    @staticmethod
    def available(path: str = REF_SO) -> bool:
        return os.path.exists(path)

    def rhs(self, pb: Problem, src, t: float = 0.0, with_bc: bool = True):
        """The RHS callback body of the reference demo: *_serial then *_bc_serial."""
        L, o = self.lib, pb.order
        src = np.ascontiguousarray(src, dtype=np.float64)
        dst = np.zeros_like(src)
        if pb.problem in (WAVE_HOM_2D, WAVE_MMS_2D):
            base = "ref_wave_hom" if pb.problem == WAVE_HOM_2D else "ref_wave"
            getattr(L, f"{base}_apply_o{o}")(pb.nx, pb.ny, pb.hix, pb.hiy, pb.xl[0], pb.xl[1], t, _ptr(src), _ptr(dst))
            if with_bc:
                getattr(L, f"{base}_bc_o{o}")(pb.nx, pb.ny, pb.hix, pb.hiy, _ptr(src), _ptr(dst))
        elif pb.problem == ADVECTION_1D and pb.a_field is not None:
            getattr(L, f"ref_adv1d_apply_var_o{o}")(pb.nx, pb.hix, _ptr(pb.a_field), _ptr(src), _ptr(dst))
            if with_bc:
                getattr(L, f"ref_adv1d_bc_var_o{o}")(pb.nx, pb.hix, _ptr(pb.a_field), _ptr(src), _ptr(dst))
        elif pb.problem == ADVECTION_2D and pb.a_field is not None:
            args = (pb.nx, pb.ny, pb.hix, pb.hiy, _ptr(pb.a_field), _ptr(pb.b_field), _ptr(src), _ptr(dst))
            getattr(L, f"ref_adv2d_apply_var_o{o}")(*args)
            if with_bc:
                getattr(L, f"ref_adv2d_bc_var_o{o}")(*args)
        elif pb.problem == ADVECTION_1D:
            getattr(L, f"ref_adv1d_apply_o{o}")(pb.nx, pb.hix, pb.a, _ptr(src), _ptr(dst))
            if with_bc:
                getattr(L, f"ref_adv1d_bc_o{o}")(pb.nx, pb.hix, pb.a, _ptr(src), _ptr(dst))
        elif pb.problem == ADVECTION_2D:
            getattr(L, f"ref_adv2d_apply_o{o}")(pb.nx, pb.ny, pb.hix, pb.hiy, pb.a, pb.b, _ptr(src), _ptr(dst))
            if with_bc:
                getattr(L, f"ref_adv2d_bc_o{o}")(pb.nx, pb.ny, pb.hix, pb.hiy, pb.a, pb.b, _ptr(src), _ptr(dst))
        elif pb.problem == REFLECTION_1D:
            getattr(L, f"ref_refl_apply_o{o}")(pb.nx, pb.hix, _ptr(src), _ptr(dst))
            if with_bc:
                getattr(L, f"ref_refl_bc_o{o}")(pb.nx, _ptr(src), _ptr(dst))
        else:
            raise ValueError("the reference has no counterpart for this problem")
        return dst

    def hnorm1d(self, v, n, dofs, h, order):
        v = np.ascontiguousarray(v, dtype=np.float64)
        return getattr(self.lib, f"ref_hnorm1d_o{order}")(n, dofs, h, _ptr(v))
