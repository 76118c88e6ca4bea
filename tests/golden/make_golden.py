"""Generate tests/golden/ref_rhs.npz from the reference's own headers.

Runs where the reference checkout exists (it builds oracle/_ref from the
headers where they lie, against the shims in oracle/shim/) and records, for
seeded inputs, the output of the reference's RHS callback body
(``*_serial`` followed by ``*_bc_serial``) and of ``H_central::get_norm_1D``.
The fixtures travel with the repository; the reference checkout does not.

    python tests/golden/make_golden.py [--ref-dir PATH]

Reference defects visible in the fixtures (kept as they are, documented in
the tests): the 1D advection right SAT and the 2D advection south SAT read
``closure_invquad`` out of bounds (code/demo/advection/advection_rhs.h:118,490),
so those boundary entries may be non-finite.
"""
import argparse
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import oracle as O  # noqa: E402

MIN_N = {2: 3, 4: 8, 6: 12}


def cases():
    """(name, problem, order, n, a, b, t, input kind) for every fixture."""
    out = []
    for order in (2, 4, 6):
        for n in sorted({MIN_N[order], 13, 33}):
            for prob in (O.WAVE_HOM_2D, O.WAVE_MMS_2D):
                out.append((prob, order, n, 0.0, 0.0, 0.37, "random"))
            out.append((O.WAVE_HOM_2D, order, n, 0.0, 0.0, 0.0, "mms"))
            out.append((O.ADVECTION_2D, order, n, 1.5, -1.0, 0.0, "random"))
        for n in sorted({MIN_N[order], 33, 201}):
            out.append((O.ADVECTION_1D, order, n, 1.0, 0.0, 0.0, "random"))
            out.append((O.ADVECTION_1D, order, n, 1.5, 0.0, 0.0, "gauss"))
            out.append((O.REFLECTION_1D, order, n, 0.0, 0.0, 0.0, "random"))
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref-dir", default=O.reference_dir(),
                    help="the reference checkout (default: $REF_DIR, baseline/_ref/, the container's checkout)")
    ap.add_argument("--out", default=os.path.join(HERE, "ref_rhs.npz"))
    args = ap.parse_args()
    if not args.ref_dir:
        sys.exit("no reference checkout found: set REF_DIR or pass --ref-dir")
    O.build(ref_dir=args.ref_dir)
    if not O.Reference.available():
        sys.exit("oracle/_ref was not built: the reference checkout is needed")
    ref, port = O.Reference(), O.Port()
    rng = np.random.default_rng(20261203)
    blobs = {}
    meta = []
    for k, (prob, order, n, a, b, t, kind) in enumerate(cases()):
        pb = O.Problem(prob, order, n, n, a=a, b=b)
        if kind == "random":
            src = rng.standard_normal(pb.size)
        elif kind == "mms":
            src = port.init_wave_mms(n, n, 0.21)
        else:
            src = port.init_adv1d(n, a, 0.0)
        dst = ref.rhs(pb, src, t=t)
        blobs[f"src{k}"] = src
        blobs[f"dst{k}"] = dst
        meta.append([prob, order, n, a, b, t])
    # get_norm_1D on one rank: left-closure weights only (H_central.h:70-103)
    hn = []
    for order in (2, 4, 6):
        for n, dofs in ((MIN_N[order], 1), (50, 2), (201, 1)):
            v = rng.standard_normal(n * dofs)
            h = 2.0 / (n - 1)
            blobs[f"hn_v{len(hn)}"] = v
            hn.append([order, n, dofs, h, ref.hnorm1d(v, n, dofs, h, order)])
    blobs["meta"] = np.array(meta, dtype=np.float64)
    blobs["hnorm"] = np.array(hn, dtype=np.float64)
    # advection with a velocity at every point (the reference's callables a(i), a(i,j), b(i,j)),
    # from a generator of their own so the cases above keep their inputs
    vrng = np.random.default_rng(20261204)
    vmeta = []
    for order in (2, 4, 6):
        for n in sorted({MIN_N[order], 33, 201}):
            x = np.linspace(-1.0, 1.0, n)
            a = 0.8 + np.sin(2 * np.pi * x + vrng.uniform(-0.3, 0.3))  # changes sign inside the domain
            k = len(vmeta)
            blobs[f"va{k}"], blobs[f"vb{k}"] = a, np.zeros(1)
            blobs[f"vsrc{k}"] = vrng.standard_normal(n)
            pb = O.Problem(O.ADVECTION_1D, order, n, a_field=a)
            blobs[f"vdst{k}"] = ref.rhs(pb, blobs[f"vsrc{k}"])
            vmeta.append([O.ADVECTION_1D, order, n])
        for n in sorted({max(MIN_N[order], 12), 33}):
            x = np.linspace(-1.0, 1.0, n)
            X, Y = np.meshgrid(x, x)
            a = 1.2 + 0.4 * np.sin(2 * X + Y + vrng.uniform(-0.3, 0.3))
            b = -0.8 + 0.3 * np.cos(X - 2 * Y + vrng.uniform(-0.3, 0.3))
            k = len(vmeta)
            blobs[f"va{k}"], blobs[f"vb{k}"] = a.ravel(), b.ravel()
            blobs[f"vsrc{k}"] = vrng.standard_normal(n * n)
            pb = O.Problem(O.ADVECTION_2D, order, n, n, a_field=a, b_field=b)
            blobs[f"vdst{k}"] = ref.rhs(pb, blobs[f"vsrc{k}"])
            vmeta.append([O.ADVECTION_2D, order, n])
    blobs["vmeta"] = np.array(vmeta, dtype=np.float64)
    np.savez_compressed(args.out, **blobs)
    print(f"wrote {len(meta)} RHS cases, {len(vmeta)} velocity-field cases and {len(hn)} H-norm cases to {args.out}")


if __name__ == "__main__":
    main()
