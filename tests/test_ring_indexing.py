"""CPU restatement of the 3D plane-ring kernel's copy and slot arithmetic
(wave3d_ring_kernel in hpc-reading-course_gb300/csrc/wave3d.cu), run block by
block with the kernel's constants: every value is its own coordinate, so the
test checks that each shared-memory tap, register-window entry and stage-update
operand reads the grid point it should, that every 16-byte chunk stays inside
its row and the state, and that no copy still in flight or issued by a thread
one plane ahead lands in a slot that the current plane's compute reads (ring A
has 2R + D + 2 slots, ring B D + 2, one barrier per plane)."""
import itertools

import pytest

TX, TY, TZ, D = 32, 4, 12, 1  # kR3X, kR3Y, kR3Z, kR3D
W_OF = {2: 3, 4: 5, 6: 7}
CS_OF = {2: 1, 4: 4, 6: 6}


def _check(nx, ny, nz, order, v, nex, tx=TX, ty=TY, tz=TZ, d=D):
    W, CS = W_OF[order], CS_OF[order]
    R = (W - 1) // 2
    HX = (R + v - 1) // v * v
    PX, PY = tx + 2 * HX, ty + 2 * R
    SA, SB = 2 * R + d + 2, d + 2
    A_W = PY * PX
    A_SZ = A_W + ty * tx
    B_V = ty * PX
    B_X = B_V + PY * tx
    B_SZ = B_X + nex * ty * tx
    for x in (tx, A_W, A_SZ, B_V, B_X, B_SZ):
        assert x % v == 0  # 16-byte aligned tile rows
    pitch = (nx + 63) // 64 * 64
    slab, plane = ny * pitch, nz * ny * pitch
    assert 4 * plane < 2**31
    points = 0
    for bx, by, bz in itertools.product(range(-(-nx // tx)), range(-(-ny // ty)), range(-(-nz // tz))):
        i0, j0, k0 = bx * tx, by * ty, bz * tz
        k1 = min(k0 + tz, nz)
        sA, sB = [None] * (SA * A_SZ), [None] * (SB * B_SZ)
        pending = []
        ctr = {"ia": 0, "ib": 0}

        def issue(m, dry=False):
            writes = []

            def box(ring, base, tp, comp, kk, NR, NC, gj0, gi0):
                for idx in range(NR * NC):
                    r, c = divmod(idx, NC)
                    gj, gi = gj0 + r, gi0 + c * v
                    if 0 <= gj < ny and 0 <= gi < nx:
                        assert gi + v <= pitch and (base + r * tp + c * v) % v == 0
                        assert kk * slab + gj * pitch + gi + v <= plane
                        for e in range(v):
                            writes.append((ring, base + r * tp + c * v + e,
                                           (comp, gi + e, gj, kk) if gi + e < nx else ("pad",)))

            ia, ib, kb = ctr["ia"], ctr["ib"], m - R
            assert ia == (m - k0 + R) % SA
            if 0 <= m < nz:
                a = ia * A_SZ
                box("A", a, PX, "p", m, ty + 2 * R, PX // v, j0 - R, i0 - HX)
                box("A", a + A_W, tx, "w", m, ty, tx // v, j0, i0)
            if k0 <= kb < k1:
                assert ib == (kb - k0) % SB
                b = ib * B_SZ
                box("B", b, PX, "u", kb, ty, PX // v, j0, i0 - HX)
                box("B", b + B_V, tx, "v", kb, ty + 2 * R, tx // v, j0 - R, i0)
                for e in range(nex):
                    box("B", b + B_X + e * ty * tx, tx, f"x{e}", kb, ty, tx // v, j0, i0)
            if not dry:
                ctr["ia"] = (ia + 1) % SA
                if k0 <= kb < k1:
                    ctr["ib"] = (ib + 1) % SB
            pending.append((m, writes))

        def land(upto):
            while pending and pending[0][0] <= upto:
                for ring, idx, val in pending.pop(0)[1]:
                    (sA if ring == "A" else sB)[idx] = val

        win = {}
        for m in range(k0 - R, k0 + R + d):
            issue(m)
        kbs, za, ka = 0, 0, R
        for k in range(k0, k1):
            issue(k + R + d)
            land(k + R)  # cp.async.wait_group D, then the block barrier
            reads = set()
            for tyy, txx in itertools.product(range(ty), range(tx)):
                i, j = i0 + txx, j0 + tyy
                if not (i < nx and j < ny):
                    continue
                pc, uc = (tyy + R) * PX + txx + HX, tyy * PX + txx + HX
                vc, wc = (tyy + R) * tx + txx, tyy * tx + txx
                zn = (za + 2 * R) % SA
                if k == k0:
                    win[(txx, tyy)] = ([sA[((za + q) % SA) * A_SZ + pc] for q in range(W - 1)] + [None],
                                       [sA[((za + q) % SA) * A_SZ + A_W + wc] for q in range(W - 1)] + [None])
                    for q in range(W - 1):
                        reads |= {("A", ((za + q) % SA) * A_SZ + pc), ("A", ((za + q) % SA) * A_SZ + A_W + wc)}
                zp, zw = win[(txx, tyy)]
                zp[W - 1], zw[W - 1] = sA[zn * A_SZ + pc], sA[zn * A_SZ + A_W + wc]
                reads |= {("A", zn * A_SZ + pc), ("A", zn * A_SZ + A_W + wc)}
                a, b = ka * A_SZ, kbs * B_SZ
                for q in range(W):
                    if CS <= k < nz - CS or q == R:
                        assert zp[q] == ("p", i, j, k - R + q) and zw[q] == ("w", i, j, k - R + q)
                if CS <= i < nx - CS:
                    for q in range(W):
                        assert sA[a + pc - R + q] == ("p", i - R + q, j, k)
                        assert sB[b + uc - R + q] == ("u", i - R + q, j, k)
                        reads |= {("A", a + pc - R + q), ("B", b + uc - R + q)}
                if CS <= j < ny - CS:
                    for q in range(W):
                        assert sA[a + pc + (q - R) * PX] == ("p", i, j - R + q, k)
                        assert sB[b + B_V + vc + (q - R) * tx] == ("v", i, j - R + q, k)
                        reads |= {("A", a + pc + (q - R) * PX), ("B", b + B_V + vc + (q - R) * tx)}
                assert sB[b + uc] == ("u", i, j, k) and sB[b + B_V + vc] == ("v", i, j, k)
                for e in range(nex):
                    assert sB[b + B_X + e * ty * tx + wc] == (f"x{e}", i, j, k)
                    reads.add(("B", b + B_X + e * ty * tx + wc))
                win[(txx, tyy)] = (zp[1:] + [None], zw[1:] + [None])
                points += 1
            # what may land while plane k is computed: copies in flight and the next plane's issue
            issue(k + 1 + R + d, dry=True)
            for _, writes in pending:
                for ring, idx, _ in writes:
                    assert (ring, idx) not in reads, ("slot reused while read", k, ring, idx)
            pending.pop()
            kbs, za, ka = (kbs + 1) % SB, (za + 1) % SA, (ka + 1) % SA
    assert points == nx * ny * nz


@pytest.mark.parametrize("order", [2, 4, 6])
@pytest.mark.parametrize("v,nex", [(4, 8), (4, 12), (2, 8), (2, 0)], ids=["fp32_mid", "fp32_last", "fp64_mid", "fp64_first"])
@pytest.mark.parametrize("n", [(13, 14, 15), (33, 9, 26), (7, 7, 7)], ids=["13x14x15", "33x9x26", "7x7x7"])
def test_ring_kernel_slots_and_taps(order, v, nex, n):
    _check(*n, order, v, nex)


def test_ring_kernel_other_shapes():
    """Shapes of the sweep that chose the default (32 x 8 threads, 2 planes ahead;
    32 x 2; 64 x 4) keep the same invariants."""
    _check(40, 17, 19, 6, 4, 12, tx=32, ty=8, tz=16, d=2)
    _check(40, 17, 19, 4, 4, 8, tx=32, ty=2, tz=5, d=1)
    _check(70, 9, 13, 2, 2, 8, tx=64, ty=4, tz=12, d=1)
