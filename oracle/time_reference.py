"""Times the reference's own wave_hom RHS (its headers compiled in this checkout with the
reference's -O3 -ffast-math, oracle/_ref/libsbpref_opt.so) beside the oracle port built
with the same flags (oracle/_build/libsbporacle_opt.so), one thread each, on the same
input. TEST INFRASTRUCTURE ONLY: it shows whether the port that bench.py times on the
GPU machine's host cores (where the reference checkout does not exist) is slower or faster
than the reference's own code.

    python oracle/time_reference.py [--n 1024] [--repeats 5]

The reference RHS is wave_eq_hom_serial + the free-surface SAT
(code/demo/wave_hom/wave_eq_hom_rhs.h:365,443); the port runs the same problem.
"""
import argparse
import ctypes as C
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import oracle as O  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=1024)
    ap.add_argument("--repeats", type=int, default=5)
    a = ap.parse_args()
    O.build(ref_dir=O.reference_dir())
    ref_so = os.path.join(HERE, "_ref", "libsbpref_opt.so")
    if not os.path.exists(ref_so):
        sys.exit("oracle/_ref/libsbpref_opt.so was not built: the reference checkout is needed")
    n = a.n
    src = np.random.default_rng(0).standard_normal(3 * n * n)
    dst = np.zeros_like(src)
    dp = C.POINTER(C.c_double)
    ref = C.CDLL(ref_so)
    port = O.Port(O.PORT_OPT_SO)
    port.set_threads(1)
    pb = O.Problem(O.WAVE_HOM_2D, 4, n, n)
    out = {}
    for order in (2, 4, 6):
        f_apply = getattr(ref, f"ref_wave_hom_apply_o{order}")
        f_bc = getattr(ref, f"ref_wave_hom_bc_o{order}")
        f_apply.argtypes = [C.c_longlong, C.c_longlong] + [C.c_double] * 5 + [dp, dp]
        f_bc.argtypes = [C.c_longlong, C.c_longlong, C.c_double, C.c_double, dp, dp]
        hi = (n - 1) / 2.0
        ps, ds = src.ctypes.data_as(dp), dst.ctypes.data_as(dp)
        pb = O.Problem(O.WAVE_HOM_2D, order, n, n)
        tr, tp = [], []
        for _ in range(a.repeats):
            t0 = time.perf_counter()
            f_apply(n, n, hi, hi, -1.0, -1.0, 0.0, ps, ds)
            f_bc(n, n, hi, hi, ps, ds)
            tr.append(time.perf_counter() - t0)
            cs = pb.c_struct()
            t0 = time.perf_counter()
            port.lib.orc_rhs(C.byref(cs), 0.0, ps, ds)  # the same preallocated arrays as the reference's
            tp.append(time.perf_counter() - t0)
        out[order] = (n * n / min(tr), n * n / min(tp))
        print(f"order {order}: reference {out[order][0]:.3e} points/s, port {out[order][1]:.3e} points/s, "
              f"port / reference {out[order][1] / out[order][0]:.2f} (one thread, {n}x{n}, best of {a.repeats})")


if __name__ == "__main__":
    main()
