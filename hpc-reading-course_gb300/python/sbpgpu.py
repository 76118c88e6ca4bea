"""ctypes binding of libsbpgpu.so (include/sbpgpu.h).

This is the binding a Python caller of the reference's RHS-callback /
ts_rk4 surface uses; it holds no numerics. Every compute call goes to the
CUDA library, and loading fails loudly when the library is missing -- there
is no CPU fallback.

Arrays are numpy float64 in the reference's AoS layout (element (j, i, comp)
at dofs*(i + nx*j) + comp); host arrays are passed with where=HOST. Device
arrays (e.g. torch CUDA tensors) are passed by address with where=DEVICE.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(PKG, "lib", "libsbpgpu.so")

OK, ERR_INVALID, ERR_CUDA, ERR_DEVICE, ERR_UNSUPPORTED, ERR_TOO_LARGE = 0, -1, -2, -3, -4, -5
NOALLOC_MAX_PLANE = 65536
WAVE_HOM_2D, WAVE_MMS_2D, ADVECTION_1D, ADVECTION_2D, REFLECTION_1D, WAVE_VAR_2D = 1, 2, 3, 4, 5, 6
WAVE_2BLOCK_2D = 7
WAVE_3D = 8
BC_REFERENCE, BC_CHARACTERISTIC = 0, 1
FP64, FP32 = 0, 1
HOST, DEVICE = 0, 1
TWO_D = {WAVE_HOM_2D, WAVE_MMS_2D, WAVE_VAR_2D, ADVECTION_2D, WAVE_2BLOCK_2D}
DOFS = {WAVE_HOM_2D: 3, WAVE_MMS_2D: 3, WAVE_VAR_2D: 3, ADVECTION_1D: 1, ADVECTION_2D: 1, REFLECTION_1D: 2,
        WAVE_2BLOCK_2D: 3, WAVE_3D: 4}

# Every exported entry point of include/sbpgpu.h.
EXPORTS = ("sbp_create", "sbp_destroy", "sbp_last_error", "sbp_dofs", "sbp_size", "sbp_rhs", "sbp_apply", "sbp_rk4_nsteps",
           "sbp_ts_rk4", "sbp_rk4", "sbp_set_state", "sbp_get_state", "sbp_rk4_resident", "sbp_synchronize",
           "sbp_error_norms", "sbp_hnorm", "sbp_get_stream", "sbp_launch_count", "sbp_probe_dfma_rate",
           "sbp_set_wait_limit", "sbp_test_drop_tile",
           "sbp_wave_rhs_noalloc", "sbp_write_petsc_vec", "sbp_read_petsc_vec",
           "sbp_batch_create", "sbp_batch_destroy", "sbp_batch_last_error", "sbp_batch_set_state",
           "sbp_batch_get_state", "sbp_batch_rk4_resident", "sbp_batch_synchronize", "sbp_batch_autotune",
           "sbp_batch_tile_height", "sbp_batch_kernel_config", "sbp_batch_select_config", "sbp_batch_get_stream", "sbp_batch_points", "sbp_batch_launch_count",
           "sbp_cnn_create", "sbp_cnn_destroy", "sbp_cnn_last_error", "sbp_cnn_param_count", "sbp_cnn_init",
           "sbp_cnn_get_params", "sbp_cnn_set_params", "sbp_cnn_forward", "sbp_cnn_gradients", "sbp_cnn_train_step",
           "sbp_cnn_features", "sbp_cnn_correct", "sbp_cnn_launch_count",
           "sbp_rk45_default_opts", "sbp_rk45_resident", "sbp_ts_rk45",
           "sbp_decomp_create", "sbp_decomp_destroy", "sbp_decomp_last_error", "sbp_decomp_set_state",
           "sbp_decomp_get_state", "sbp_decomp_rhs", "sbp_decomp_rk4_resident")

_dp = C.POINTER(C.c_double)
ERR_DIVERGED = -6


class Rk45Opts(C.Structure):
    _fields_ = [("atol", C.c_double), ("rtol", C.c_double), ("safety", C.c_double), ("reject_safety", C.c_double),
                ("clip_lo", C.c_double), ("clip_hi", C.c_double), ("dt_min", C.c_double), ("dt_max", C.c_double),
                ("max_steps", C.c_longlong), ("max_reject", C.c_int)]


class Rk45Stats(C.Structure):
    _fields_ = [("accepted", C.c_longlong), ("rejected", C.c_longlong), ("t", C.c_double), ("dt_next", C.c_double),
                ("wlte", C.c_double), ("status", C.c_int)]


class Desc(C.Structure):
    _fields_ = [("problem", C.c_int), ("order", C.c_int), ("bc", C.c_int), ("precision", C.c_int),
                ("nx", C.c_longlong), ("ny", C.c_longlong),
                ("xl", C.c_double * 2), ("xr", C.c_double * 2),
                ("a", C.c_double), ("b", C.c_double),
                ("rho", _dp), ("K", _dp),
                ("stream", C.c_void_p), ("device", C.c_int),
                ("nz", C.c_longlong), ("xl2", C.c_double), ("xr2", C.c_double),
                ("a_field", _dp), ("b_field", _dp)]


class Instance(C.Structure):
    """One member of a batch (sbp_instance)."""
    _fields_ = [("problem", C.c_int), ("order", C.c_int), ("bc", C.c_int),
                ("nx", C.c_longlong), ("ny", C.c_longlong),
                ("xl", C.c_double * 2), ("xr", C.c_double * 2),
                ("c", C.c_double), ("a", C.c_double), ("b", C.c_double), ("dt", C.c_double)]


class SbpError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"libsbpgpu error {code}: {msg}")
        self.code = code


_lib = None


def load(path: str = LIB_PATH) -> C.CDLL:
    """Load the CUDA library (once). Raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise OSError(f"{path} is missing: build it with `python hpc-reading-course_gb300/build.py` "
                      "(the SBP hot path has no CPU implementation in the product)")
    L = C.CDLL(path)
    P = C.c_void_p
    L.sbp_create.argtypes = [C.POINTER(Desc), C.POINTER(P)]
    L.sbp_destroy.argtypes = [P]
    L.sbp_last_error.argtypes = [P]
    L.sbp_last_error.restype = C.c_char_p
    L.sbp_dofs.argtypes = [P]
    L.sbp_size.argtypes = [P]
    L.sbp_size.restype = C.c_longlong
    for n in ("sbp_rhs", "sbp_apply"):
        getattr(L, n).argtypes = [P, C.c_double, C.c_void_p, C.c_void_p, C.c_int]
    L.sbp_rk4_nsteps.argtypes = [C.c_double, _dp]
    L.sbp_rk4_nsteps.restype = C.c_longlong
    L.sbp_ts_rk4.argtypes = [P, C.c_double, C.c_double, C.c_void_p, C.c_int]
    L.sbp_rk4.argtypes = [P, C.c_double, C.c_double, C.c_longlong, C.c_void_p, C.c_int]
    L.sbp_set_state.argtypes = [P, C.c_void_p, C.c_int]
    L.sbp_get_state.argtypes = [P, C.c_void_p, C.c_int]
    L.sbp_rk4_resident.argtypes = [P, C.c_double, C.c_double, C.c_longlong]
    L.sbp_rk45_default_opts.argtypes = [C.POINTER(Rk45Opts)]
    L.sbp_rk45_default_opts.restype = None
    L.sbp_rk45_resident.argtypes = [P, C.c_double, C.c_double, C.c_double, C.POINTER(Rk45Opts),
                                    C.POINTER(Rk45Stats)]
    L.sbp_ts_rk45.argtypes = [P, C.c_double, C.c_double, C.c_void_p, C.c_int]
    L.sbp_synchronize.argtypes = [P]
    L.sbp_error_norms.argtypes = [P, C.c_void_p, C.c_int, _dp, _dp]
    L.sbp_hnorm.argtypes = [P, _dp]
    L.sbp_get_stream.argtypes = [P, C.POINTER(C.c_void_p)]
    L.sbp_launch_count.argtypes = [P]
    L.sbp_launch_count.restype = C.c_longlong
    L.sbp_probe_dfma_rate.argtypes = [C.c_int, _dp]
    L.sbp_set_wait_limit.argtypes = [P, C.c_longlong]
    L.sbp_test_drop_tile.argtypes = [P, C.c_longlong]
    L.sbp_wave_rhs_noalloc.argtypes = [C.POINTER(Desc), C.c_double, C.c_void_p, C.c_void_p]
    L.sbp_batch_create.argtypes = [C.POINTER(Instance), C.c_int, C.c_int, C.c_int, C.c_void_p, C.POINTER(P)]
    L.sbp_batch_destroy.argtypes = [P]
    L.sbp_batch_last_error.argtypes = [P]
    L.sbp_batch_last_error.restype = C.c_char_p
    L.sbp_batch_set_state.argtypes = [P, C.c_int, C.c_void_p, C.c_int]
    L.sbp_batch_get_state.argtypes = [P, C.c_int, C.c_void_p, C.c_int]
    L.sbp_batch_rk4_resident.argtypes = [P, C.c_longlong]
    L.sbp_batch_synchronize.argtypes = [P]
    L.sbp_batch_autotune.argtypes = [P, C.c_char_p]
    L.sbp_batch_tile_height.argtypes = [P, C.c_int]
    L.sbp_batch_kernel_config.argtypes = [P, C.c_int, C.c_int, C.POINTER(C.c_int)]
    L.sbp_batch_select_config.argtypes = [P, C.c_int, C.c_int, C.c_int]
    L.sbp_batch_get_stream.argtypes = [P, C.POINTER(C.c_void_p)]
    L.sbp_batch_points.argtypes = [P]
    L.sbp_batch_points.restype = C.c_longlong
    L.sbp_batch_launch_count.argtypes = [P]
    L.sbp_batch_launch_count.restype = C.c_longlong
    L.sbp_cnn_create.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p, C.POINTER(P)]
    L.sbp_cnn_destroy.argtypes = [P]
    L.sbp_cnn_last_error.argtypes = [P]
    L.sbp_cnn_last_error.restype = C.c_char_p
    L.sbp_cnn_param_count.restype = C.c_longlong
    L.sbp_cnn_init.argtypes = [P, C.c_ulonglong]
    L.sbp_cnn_get_params.argtypes = [P, C.c_void_p, C.c_longlong]
    L.sbp_cnn_set_params.argtypes = [P, C.c_void_p, C.c_longlong]
    L.sbp_cnn_forward.argtypes = [P, C.c_void_p, C.c_int, C.c_void_p]
    L.sbp_cnn_gradients.argtypes = [P, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_longlong,
                                    C.POINTER(C.c_float)]
    L.sbp_cnn_train_step.argtypes = [P, C.c_void_p, C.c_void_p, C.c_int, C.c_float, C.POINTER(C.c_float)]
    L.sbp_cnn_features.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_double,
                                   C.c_void_p, C.c_void_p]
    L.sbp_cnn_correct.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_longlong, C.c_double,
                                  C.c_void_p]
    L.sbp_cnn_launch_count.argtypes = [P]
    L.sbp_cnn_launch_count.restype = C.c_longlong
    L.sbp_decomp_create.argtypes = [C.POINTER(Desc), C.c_int, C.c_int, C.POINTER(P)]
    L.sbp_decomp_destroy.argtypes = [P]
    L.sbp_decomp_last_error.argtypes = [P]
    L.sbp_decomp_last_error.restype = C.c_char_p
    L.sbp_decomp_set_state.argtypes = [P, C.c_void_p, C.c_int]
    L.sbp_decomp_get_state.argtypes = [P, C.c_void_p, C.c_int]
    L.sbp_decomp_rhs.argtypes = [P, C.c_void_p, C.c_void_p, C.c_int]
    L.sbp_decomp_rk4_resident.argtypes = [P, C.c_double, C.c_longlong]
    L.sbp_write_petsc_vec.argtypes = [C.c_char_p, C.c_void_p, C.c_longlong]
    L.sbp_read_petsc_vec.argtypes = [C.c_char_p, C.c_void_p, C.c_longlong, C.POINTER(C.c_longlong)]
    _lib = L
    return L


def rk4_nsteps(t_end: float, dt: float):
    """The reference's step rule: (steps, adjusted dt)."""
    d = C.c_double(dt)
    n = load().sbp_rk4_nsteps(t_end, C.byref(d))
    return n, d.value


def probe_dfma_rate(device: int = 0) -> float:
    r = C.c_double(0.0)
    rc = load().sbp_probe_dfma_rate(device, C.byref(r))
    if rc:
        raise SbpError(rc, "DFMA probe failed")
    return r.value


def wave_rhs_noalloc(order: int, nx: int, ny: int, t: float, src_ptr: int, dst_ptr: int, *,
                     bc: int = BC_REFERENCE, xl=(-1.0, -1.0), xr=(1.0, 1.0), stream: int | None = None,
                     device: int = 0) -> int:
    """sbp_wave_rhs_noalloc on caller-owned device arrays; returns the status code."""
    d = Desc(WAVE_HOM_2D, order, bc, FP64, nx, ny, (C.c_double * 2)(*xl), (C.c_double * 2)(*xr), 0.0, 0.0,
             None, None, stream, device)
    return load().sbp_wave_rhs_noalloc(C.byref(d), t, src_ptr, dst_ptr)


def write_petsc_vec(path: str, v: np.ndarray) -> None:
    """Write a PETSc binary Vec file (what VecView on a binary viewer writes)."""
    v = np.ascontiguousarray(v, dtype=np.float64)
    rc = load().sbp_write_petsc_vec(path.encode(), v.ctypes.data, v.size)
    if rc:
        raise SbpError(rc, f"cannot write {path}")


def read_petsc_vec(path: str) -> np.ndarray:
    """Read a PETSc binary Vec file."""
    L = load()
    n = C.c_longlong(0)
    rc = L.sbp_read_petsc_vec(path.encode(), None, 0, C.byref(n))
    if rc:
        raise SbpError(rc, f"{path} is not a PETSc binary Vec file")
    out = np.empty(n.value)
    rc = L.sbp_read_petsc_vec(path.encode(), out.ctypes.data, out.size, C.byref(n))
    if rc:
        raise SbpError(rc, f"cannot read {path}")
    return out


def _host(a: np.ndarray) -> np.ndarray:
    if a.dtype != np.float64 or not a.flags["C_CONTIGUOUS"]:
        raise TypeError("host arrays must be C-contiguous float64")
    return a


class Context:
    """One problem instance on one device (sbp_create / sbp_destroy)."""

    def __init__(self, problem: int, order: int, nx: int, ny: int = 1, nz: int = 1, *, bc: int = BC_REFERENCE,
                 precision: int = FP64, xl=(-1.0, -1.0, -1.0), xr=(1.0, 1.0, 1.0), a: float = 1.0, b: float = 0.0,
                 rho=None, K=None, stream: int | None = None, device: int = 0, a_field=None, b_field=None):
        L = load()
        self._L = L
        self.problem, self.order, self.nx = problem, order, nx
        self.ny = ny if problem in TWO_D or problem == WAVE_3D else 1
        self.nz = nz if problem == WAVE_3D else 1
        self.dofs = DOFS.get(problem, 0)
        self.precision = precision
        xl = tuple(xl) + (-1.0,) * (3 - len(xl))
        xr = tuple(xr) + (1.0,) * (3 - len(xr))
        self.xl, self.xr = xl, xr
        self._rho = None if rho is None else np.ascontiguousarray(rho, dtype=np.float64).ravel()
        self._K = None if K is None else np.ascontiguousarray(K, dtype=np.float64).ravel()
        d = Desc(problem, order, bc, precision, nx, self.ny, (C.c_double * 2)(*xl[:2]), (C.c_double * 2)(*xr[:2]),
                 a, b, None, None, stream, device, self.nz, xl[2], xr[2])
        if self._rho is not None:
            d.rho = self._rho.ctypes.data_as(_dp)
            d.K = self._K.ctypes.data_as(_dp)
        # advection: velocities at every point (copied by sbp_create)
        self._va = None if a_field is None else np.ascontiguousarray(a_field, dtype=np.float64).ravel()
        self._vb = None if b_field is None else np.ascontiguousarray(b_field, dtype=np.float64).ravel()
        if self._va is not None:
            d.a_field = self._va.ctypes.data_as(_dp)
        if self._vb is not None:
            d.b_field = self._vb.ctypes.data_as(_dp)
        h = C.c_void_p()
        rc = L.sbp_create(C.byref(d), C.byref(h))
        if rc:
            raise SbpError(rc, L.sbp_last_error(None).decode())
        self._h = h

    # -- helpers
    @property
    def size(self) -> int:
        return self.nx * self.ny * self.nz * self.dofs

    @property
    def hx(self) -> float:
        return (self.xr[0] - self.xl[0]) / (self.nx - 1)

    @property
    def hy(self) -> float:
        if self.problem == WAVE_2BLOCK_2D:
            return 0.5 * (self.xr[1] - self.xl[1]) / (self.ny // 2 - 1)
        return (self.xr[1] - self.xl[1]) / (self.ny - 1) if self.problem in TWO_D or self.problem == WAVE_3D else 1.0

    @property
    def hz(self) -> float:
        return (self.xr[2] - self.xl[2]) / (self.nz - 1) if self.problem == WAVE_3D else 1.0

    def _check(self, rc: int):
        if rc:
            raise SbpError(rc, self._L.sbp_last_error(self._h).decode())

    def close(self):
        if getattr(self, "_h", None):
            self._L.sbp_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- the reference surface
    def rhs(self, src: np.ndarray, t: float = 0.0) -> np.ndarray:
        """dst = F(t, src): the RHS callback body (host arrays)."""
        src = _host(src)
        dst = np.empty_like(src)
        self._check(self._L.sbp_rhs(self._h, t, src.ctypes.data, dst.ctypes.data, HOST))
        return dst

    def apply(self, src: np.ndarray, t: float = 0.0) -> np.ndarray:
        """The matrix-free apply without boundary terms (host arrays)."""
        src = _host(src)
        dst = np.empty_like(src)
        self._check(self._L.sbp_apply(self._h, t, src.ctypes.data, dst.ctypes.data, HOST))
        return dst

    def set_wait_limit(self, ns: int):
        """Limit of the stage kernels' bounded device waits (0: the default, 200 ms)."""
        self._check(self._L.sbp_set_wait_limit(self._h, ns))

    def test_drop_tile(self, tile: int):
        """Test aid: the next rhs()/apply() issues no load for this tile, so its
        bounded wait runs out and the call raises SbpError(ERR_DEVICE)."""
        self._check(self._L.sbp_test_drop_tile(self._h, tile))

    def rhs_ptr(self, t: float, src_ptr: int, dst_ptr: int, where: int):
        self._check(self._L.sbp_rhs(self._h, t, src_ptr, dst_ptr, where))

    def ts_rk4(self, v: np.ndarray, t_end: float, dt: float) -> np.ndarray:
        out = np.array(_host(v), copy=True)
        self._check(self._L.sbp_ts_rk4(self._h, t_end, dt, out.ctypes.data, HOST))
        return out

    def rk4(self, v: np.ndarray, t0: float, dt: float, nsteps: int) -> np.ndarray:
        out = np.array(_host(v), copy=True)
        self._check(self._L.sbp_rk4(self._h, t0, dt, nsteps, out.ctypes.data, HOST))
        return out

    def rk4_ptr(self, ptr: int, t0: float, dt: float, nsteps: int, where: int):
        self._check(self._L.sbp_rk4(self._h, t0, dt, nsteps, ptr, where))

    # -- resident state
    def set_state(self, v: np.ndarray):
        self._check(self._L.sbp_set_state(self._h, _host(v).ctypes.data, HOST))

    def set_state_ptr(self, ptr: int, where: int):
        self._check(self._L.sbp_set_state(self._h, ptr, where))

    def get_state(self) -> np.ndarray:
        out = np.empty(self.size)
        self._check(self._L.sbp_get_state(self._h, out.ctypes.data, HOST))
        return out

    def get_state_ptr(self, ptr: int, where: int):
        self._check(self._L.sbp_get_state(self._h, ptr, where))

    def step_resident(self, t0: float, dt: float, nsteps: int):
        self._check(self._L.sbp_rk4_resident(self._h, t0, dt, nsteps))

    def rk45_resident(self, t0: float, t_end: float, dt0: float, check: bool = True, **opts) -> dict:
        """Adaptive RKF45 on the resident state (sbp_rk45_resident); opts override the defaults.
        Returns the stats as a dict; with check=False a stopped run returns its stats too."""
        o = Rk45Opts()
        self._L.sbp_rk45_default_opts(C.byref(o))
        for k, val in opts.items():
            setattr(o, k, val)
        st = Rk45Stats()
        rc = self._L.sbp_rk45_resident(self._h, t0, t_end, dt0, C.byref(o), C.byref(st))
        if rc and (check or rc != ERR_DIVERGED):
            self._check(rc)
        out = {f: getattr(st, f) for f, _ in Rk45Stats._fields_}
        out["rc"] = rc
        return out

    def ts_rk45(self, v: np.ndarray, t_end: float, dt: float) -> np.ndarray:
        out = np.array(_host(v), copy=True)
        self._check(self._L.sbp_ts_rk45(self._h, t_end, dt, out.ctypes.data, HOST))
        return out

    def synchronize(self):
        self._check(self._L.sbp_synchronize(self._h))

    def error_norms(self, exact: np.ndarray):
        l2, mx = C.c_double(), C.c_double()
        self._check(self._L.sbp_error_norms(self._h, _host(exact).ctypes.data, HOST, C.byref(l2), C.byref(mx)))
        return l2.value, mx.value

    def hnorm(self) -> float:
        h = C.c_double()
        self._check(self._L.sbp_hnorm(self._h, C.byref(h)))
        return h.value

    @property
    def stream(self) -> int:
        s = C.c_void_p()
        self._check(self._L.sbp_get_stream(self._h, C.byref(s)))
        return s.value or 0

    @property
    def launches(self) -> int:
        return self._L.sbp_launch_count(self._h)


class Decomp:
    """One SBP_WAVE_HOM_2D grid (FP64) as px x py subdomains with ghost lines and a device halo
    exchange before every stage (sbp_decomp_*); states are the full grid's AoS arrays."""

    def __init__(self, order: int, nx: int, ny: int, px: int, py: int, *, bc: int = BC_REFERENCE,
                 xl=(-1.0, -1.0), xr=(1.0, 1.0), stream: int | None = None, device: int = 0):
        L = load()
        self._L = L
        self.nx, self.ny, self.px, self.py = nx, ny, px, py
        self.size = 3 * nx * ny
        d = Desc(WAVE_HOM_2D, order, bc, FP64, nx, ny, (C.c_double * 2)(*xl[:2]), (C.c_double * 2)(*xr[:2]),
                 0.0, 0.0, None, None, stream, device, 1, -1.0, 1.0)
        h = C.c_void_p()
        rc = L.sbp_decomp_create(C.byref(d), px, py, C.byref(h))
        if rc:
            raise SbpError(rc, L.sbp_decomp_last_error(None).decode())
        self._h = h

    def _check(self, rc):
        if rc:
            raise SbpError(rc, self._L.sbp_decomp_last_error(self._h).decode())

    def close(self):
        if self._h:
            self._L.sbp_decomp_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_state(self, v: np.ndarray):
        self._check(self._L.sbp_decomp_set_state(self._h, _host(v).ctypes.data, HOST))

    def get_state(self) -> np.ndarray:
        out = np.empty(self.size)
        self._check(self._L.sbp_decomp_get_state(self._h, out.ctypes.data, HOST))
        return out

    def rhs(self, src: np.ndarray) -> np.ndarray:
        src = _host(src)
        dst = np.empty_like(src)
        self._check(self._L.sbp_decomp_rhs(self._h, src.ctypes.data, dst.ctypes.data, HOST))
        return dst

    def step_resident(self, dt: float, nsteps: int):
        self._check(self._L.sbp_decomp_rk4_resident(self._h, dt, nsteps))

    def rk4(self, v0: np.ndarray, dt: float, nsteps: int) -> np.ndarray:
        self.set_state(v0)
        self.step_resident(dt, nsteps)
        return self.get_state()


class Batch:
    """Many independent wave / advection instances advanced together (sbp_batch_*).

    instances: dicts with problem (WAVE_HOM_2D or ADVECTION_2D), order, nx, ny,
    dt and c (wave speed) or a, b (advection velocity); optional bc, xl, xr.
    """

    def __init__(self, instances, *, precision: int = FP64, device: int = 0, stream: int | None = None):
        L = load()
        self._L = L
        arr = (Instance * len(instances))()
        self.shapes = []
        for k, d in enumerate(instances):
            xl, xr = d.get("xl", (-1.0, -1.0)), d.get("xr", (1.0, 1.0))
            arr[k] = Instance(d["problem"], d["order"], d.get("bc", BC_REFERENCE), d["nx"], d["ny"],
                              (C.c_double * 2)(*xl), (C.c_double * 2)(*xr), d.get("c", 1.0), d.get("a", 0.0),
                              d.get("b", 0.0), d["dt"])
            self.shapes.append((d["ny"], d["nx"], 3 if d["problem"] == WAVE_HOM_2D else 1))
        h = C.c_void_p()
        rc = L.sbp_batch_create(arr, len(instances), precision, device, stream, C.byref(h))
        if rc:
            raise SbpError(rc, L.sbp_batch_last_error(None).decode())
        self._h = h

    def _check(self, rc):
        if rc:
            raise SbpError(rc, self._L.sbp_batch_last_error(self._h).decode())

    def close(self):
        if getattr(self, "_h", None):
            self._L.sbp_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_state(self, index: int, v: np.ndarray):
        self._check(self._L.sbp_batch_set_state(self._h, index, _host(v).ctypes.data, HOST))

    def get_state(self, index: int) -> np.ndarray:
        out = np.empty(int(np.prod(self.shapes[index])))
        self._check(self._L.sbp_batch_get_state(self._h, index, out.ctypes.data, HOST))
        return out

    def step_resident(self, nsteps: int):
        self._check(self._L.sbp_batch_rk4_resident(self._h, nsteps))

    def synchronize(self):
        self._check(self._L.sbp_batch_synchronize(self._h))

    def autotune(self, cache_path: str | None = None):
        self._check(self._L.sbp_batch_autotune(self._h, cache_path.encode() if cache_path else None))

    def tile_height(self, order: int) -> int:
        return self._L.sbp_batch_tile_height(self._h, order)

    def kernel_config(self, order: int, problem: int) -> dict:
        """The kernel configuration of one (order, problem) group: tile rows, compute warps,
        ring depth, CTAs per SM and converter warps (the FP64 fixed-point wave kernel; zeros
        for an empty group)."""
        cfg = (C.c_int * 5)()
        self._check(self._L.sbp_batch_kernel_config(self._h, order, problem, cfg))
        return dict(zip(("rows", "warps", "ring", "ctas_per_sm", "converters"), list(cfg)))

    def select_config(self, order: int, problem: int, index: int):
        """Runs entry `index` (0..3) of the group's configuration table from now on."""
        self._check(self._L.sbp_batch_select_config(self._h, order, problem, index))

    @property
    def points(self) -> int:
        return self._L.sbp_batch_points(self._h)

    @property
    def launches(self) -> int:
        return self._L.sbp_batch_launch_count(self._h)

    @property
    def stream(self) -> int:
        s = C.c_void_p()
        self._check(self._L.sbp_batch_get_stream(self._h, C.byref(s)))
        return s.value or 0


class Cnn:
    """The learned-correction network (sbp_cnn_*). Device arrays are passed by address
    (e.g. torch CUDA tensors' data_ptr()): features NHWC FP32 with 24 channels, outputs 3."""

    def __init__(self, height: int, width: int, max_batch: int, *, device: int = 0, stream: int | None = None,
                 seed: int = 1234):
        L = load()
        self._L = L
        self.height, self.width, self.max_batch = height, width, max_batch
        h = C.c_void_p()
        rc = L.sbp_cnn_create(height, width, max_batch, device, stream, C.byref(h))
        if rc:
            raise SbpError(rc, L.sbp_cnn_last_error(None).decode())
        self._h = h
        self.stream = stream  # the cudaStream_t it was created on (None: its own)
        if seed != 1234:
            self._check(L.sbp_cnn_init(h, seed))

    def _check(self, rc):
        if rc:
            raise SbpError(rc, self._L.sbp_cnn_last_error(self._h).decode())

    def close(self):
        if getattr(self, "_h", None):
            self._L.sbp_cnn_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @staticmethod
    def param_count() -> int:
        return load().sbp_cnn_param_count()

    def get_params(self) -> np.ndarray:
        out = np.empty(self.param_count(), dtype=np.float32)
        self._check(self._L.sbp_cnn_get_params(self._h, out.ctypes.data, out.size))
        return out

    def set_params(self, v: np.ndarray):
        v = np.ascontiguousarray(v, dtype=np.float32)
        self._check(self._L.sbp_cnn_set_params(self._h, v.ctypes.data, v.size))

    def forward(self, x_ptr: int, batch: int, out_ptr: int):
        self._check(self._L.sbp_cnn_forward(self._h, x_ptr, batch, out_ptr))

    def gradients(self, x_ptr: int, target_ptr: int, batch: int):
        g = np.empty(self.param_count(), dtype=np.float32)
        loss = C.c_float()
        self._check(self._L.sbp_cnn_gradients(self._h, x_ptr, target_ptr, batch, g.ctypes.data, g.size,
                                              C.byref(loss)))
        return loss.value, g

    def train_step(self, x_ptr: int, target_ptr: int, batch: int, lr: float) -> float:
        loss = C.c_float()
        self._check(self._L.sbp_cnn_train_step(self._h, x_ptr, target_ptr, batch, lr, C.byref(loss)))
        return loss.value

    @property
    def launches(self) -> int:
        return self._L.sbp_cnn_launch_count(self._h)


def cnn_features(state_ptr: int, rho_ptr: int, K_ptr: int, nx: int, ny: int, block_rows: int, inv_scale: float,
                 x_ptr: int, stream: int | None = None):
    rc = load().sbp_cnn_features(state_ptr, rho_ptr, K_ptr, nx, ny, block_rows, inv_scale, x_ptr, stream)
    if rc:
        raise SbpError(rc, "sbp_cnn_features failed")


def cnn_correct(state_ptr: int, delta_ptr: int, rho_ptr: int, K_ptr: int, npts: int, scale: float,
                stream: int | None = None):
    rc = load().sbp_cnn_correct(state_ptr, delta_ptr, rho_ptr, K_ptr, npts, scale, stream)
    if rc:
        raise SbpError(rc, "sbp_cnn_correct failed")
