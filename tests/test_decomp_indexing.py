"""CPU restatement of the decomposed path's index arithmetic
(hpc-reading-course_gb300/csrc/decomp.cu): the subdomain pools with sw ghost
lines, the halo-exchange kernel's copies and every tap d1_sub reads. Values are
their own global coordinates, so the test checks that after the exchange every
interior stencil tap, closure tap and centre value of every point reads the
grid point it should, and that all pool accesses stay inside the subdomain's
own planes."""
import itertools

import pytest

W_OF = {2: 3, 4: 5, 6: 7}
CS_OF = {2: 1, 4: 4, 6: 6}
CW_OF = {2: 2, 4: 6, 6: 9}


def _layout(NX, NY, px, py, sw):
    subs, off = [], 0
    for by, bx in itertools.product(range(py), range(px)):
        xoff, yoff = bx * NX // px, by * NY // py
        nx, ny = (bx + 1) * NX // px - xoff, (by + 1) * NY // py - yoff
        pitch = (nx + 2 * sw + 31) // 32 * 32
        plane = (ny + 2 * sw) * pitch
        subs.append(dict(nx=nx, ny=ny, xoff=xoff, yoff=yoff, pitch=pitch, plane=plane, base=off))
        off += 3 * plane
    return subs, off


def _check(NX, NY, px, py, order):
    W, CS, CW = W_OF[order], CS_OF[order], CW_OF[order]
    sw = (W - 1) // 2
    assert NX // px >= CW and NY // py >= CW
    subs, pool_n = _layout(NX, NY, px, py, sw)
    pool = [None] * pool_n

    def at(S, c, i, j):  # local (i, j), ghosts at -sw.. and n..n+sw-1
        assert -sw <= i < S["nx"] + sw and -sw <= j < S["ny"] + sw
        return S["base"] + c * S["plane"] + (j + sw) * S["pitch"] + (i + sw)

    # scatter: interiors hold their global coordinates
    for S in subs:
        for j, i, c in itertools.product(range(S["ny"]), range(S["nx"]), range(3)):
            pool[at(S, c, i, j)] = (c, S["xoff"] + i, S["yoff"] + j)
    # halo kernel (side 0 west, 1 east, 2 south, 3 north)
    for b, side in itertools.product(range(px * py), range(4)):
        bx, by = b % px, b // px
        nbx = bx - 1 if side == 0 else (bx + 1 if side == 1 else bx)
        nby = by - 1 if side == 2 else (by + 1 if side == 3 else by)
        if not (0 <= nbx < px and 0 <= nby < py):
            continue
        S, N = subs[b], subs[nby * px + nbx]
        length = S["ny"] if side < 2 else S["nx"]
        for idx in range(3 * sw * length):
            c, rem = divmod(idx, sw * length)
            g, p = divmod(rem, length)
            if side == 0:
                di, dj, si, sj = -sw + g, p, N["nx"] - sw + g, p
            elif side == 1:
                di, dj, si, sj = S["nx"] + g, p, g, p
            elif side == 2:
                di, dj, si, sj = p, -sw + g, p, N["ny"] - sw + g
            else:
                di, dj, si, sj = p, S["ny"] + g, p, g
            pool[at(S, c, di, dj)] = pool[at(N, c, si, sj)]

    def d1_taps(S, c, base_local, st_is_x, off, n, I):
        """Global indices d1_sub reads for the line through base_local."""
        R = sw
        if CS <= I < n - CS:
            idx = [I - R + k for k in range(W) if k != R]
        elif I < CS:
            assert off == 0
            idx = list(range(CW))
        else:
            idx = [n - CW + k for k in range(CW)]
        vals = []
        for g in idx:
            li = g - off
            i, j = (li, base_local) if st_is_x else (base_local, li)
            vals.append((pool[at(S, c, i, j)], g))
        return vals

    for b, S in enumerate(subs):
        for j, i in itertools.product(range(S["ny"]), range(S["nx"])):
            I, J = S["xoff"] + i, S["yoff"] + j
            for c in (0, 2):  # x lines of u and p
                for v, g in d1_taps(S, c, j, True, S["xoff"], NX, I):
                    assert v == (c, g, J), (b, i, j, c, v, g)
            for c in (1, 2):  # y lines of v and p
                for v, g in d1_taps(S, c, i, False, S["yoff"], NY, J):
                    assert v == (c, I, g), (b, i, j, c, v, g)
            for c in range(3):
                assert pool[at(S, c, i, j)] == (c, I, J)


@pytest.mark.parametrize("order", [2, 4, 6])
@pytest.mark.parametrize("grid", [(37, 29, 2, 3), (40, 40, 4, 4), (65, 33, 3, 2), (20, 18, 1, 1), (27, 60, 1, 5)],
                         ids=["37x29_2x3", "40x40_4x4", "65x33_3x2", "20x18_1x1", "27x60_1x5"])
def test_decomposition_halo_and_taps(order, grid):
    NX, NY, px, py = grid
    if NX // px < CW_OF[order] or NY // py < CW_OF[order]:
        pytest.skip("subdomains narrower than a closure block are rejected by sbp_decomp_create")
    _check(NX, NY, px, py, order)
