"""CPU restatement of the decomposed path's index arithmetic
(hpc-reading-course_gb300/csrc/decomp.cu, and the decomposed stage kernel of
csrc/wave2d_fixed.cuh): the subdomain pools with sw ghost rows and col0 ghost
columns (sw rounded up to even), the halo-exchange kernel's copies, the TMA box
origins the producer issues, and every tap the compute warps read (interior taps
from the boxes, closure taps from the arrays). Values are their own global
coordinates, so the test checks that after the exchange every interior stencil
tap, closure tap and centre value of every point reads the grid point it should,
that all pool accesses stay inside the subdomain's own planes, and that every
TMA x coordinate is a multiple of 2 doubles (16 bytes)."""
import itertools

import pytest

W_OF = {2: 3, 4: 5, 6: 7}
CS_OF = {2: 1, 4: 4, 6: 6}
CW_OF = {2: 2, 4: 6, 6: 9}


TY_OF = {2: 14, 4: 14, 6: 14}  # the fixed-point tile's rows (SBP_FP64_TILE_ROWS)


def _layout(NX, NY, px, py, sw, col0):
    subs, off = [], 0
    for by, bx in itertools.product(range(py), range(px)):
        xoff, yoff = bx * NX // px, by * NY // py
        nx, ny = (bx + 1) * NX // px - xoff, (by + 1) * NY // py - yoff
        pitch = (nx + 2 * col0 + 31) // 32 * 32
        plane = (ny + 2 * sw) * pitch
        subs.append(dict(nx=nx, ny=ny, xoff=xoff, yoff=yoff, pitch=pitch, plane=plane, base=off))
        off += 3 * plane
    return subs, off


def _check(NX, NY, px, py, order):
    W, CS, CW = W_OF[order], CS_OF[order], CW_OF[order]
    sw = (W - 1) // 2
    col0 = (sw + 1) // 2 * 2  # ghost_x(order)
    HX, HY, TY = col0, sw, TY_OF[order]
    assert NX // px >= CW and NY // py >= CW
    subs, pool_n = _layout(NX, NY, px, py, sw, col0)
    pool = [None] * pool_n

    def at(S, c, i, j):  # local (i, j), ghosts at -sw.. and n..n+sw-1
        assert -sw <= i < S["nx"] + sw and -sw <= j < S["ny"] + sw
        assert S["nx"] + 2 * col0 <= S["pitch"]
        return S["base"] + c * S["plane"] + (j + sw) * S["pitch"] + (i + col0)

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

    # TMA boxes of every tile: origins in array coordinates (the interior starts at
    # column col0, row sw), x a multiple of 2 doubles, and the stencil taps the
    # compute warps read from the boxes land on local indices i - R .. i + R
    for b, S in enumerate(subs):
        assert (S["base"] * 8) % 16 == 0 and (S["pitch"] * 8) % 16 == 0 and (S["plane"] * 8) % 16 == 0
        for j0 in range(0, S["ny"], TY):
            for i0 in range(0, S["nx"], 64):
                for (x, y) in ((i0, j0), (i0, j0 + HY), (i0 + HX, j0), (i0 + HX, j0 + HY)):  # p, u, v, u^n/acc
                    assert x % 2 == 0 and x >= 0 and y >= 0
                for yy, xx in itertools.product(range(TY), range(64)):
                    i, j = i0 + xx, j0 + yy
                    if i >= S["nx"] or j >= S["ny"]:
                        continue
                    for s in range(W):  # box column of tap s (x + HX - R + s) -> array column
                        assert i0 + (xx + HX - sw + s) == col0 + i - sw + s
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


def _halo_writes(subs, px, py, sw, col0):
    """{destination pool index: (source subdomain, c, i, j)} of the halo-exchange kernel."""
    def at(S, c, i, j):
        return S["base"] + c * S["plane"] + (j + sw) * S["pitch"] + (i + col0)
    out = {}
    for b, side in itertools.product(range(px * py), range(4)):
        bx, by = b % px, b // px
        nbx = bx - 1 if side == 0 else (bx + 1 if side == 1 else bx)
        nby = by - 1 if side == 2 else (by + 1 if side == 3 else by)
        if not (0 <= nbx < px and 0 <= nby < py):
            continue
        S, n = subs[b], nby * px + nbx
        N = subs[n]
        length = S["ny"] if side < 2 else S["nx"]
        for c, g, p in itertools.product(range(3), range(sw), range(length)):
            if side == 0:
                di, dj, si, sj = -sw + g, p, N["nx"] - sw + g, p
            elif side == 1:
                di, dj, si, sj = S["nx"] + g, p, g, p
            elif side == 2:
                di, dj, si, sj = p, -sw + g, p, N["ny"] - sw + g
            else:
                di, dj, si, sj = p, S["ny"] + g, p, g
            out[at(S, c, di, dj)] = (n, c, si, sj)
    return out


def _fused_writes(subs, px, py, sw, col0):
    """The same map for the exchange fused into the stage kernels (fx_exchange_tile):
    every point within sw of its subdomain's edge, once per side with a neighbour,
    copies its value into the neighbour's mirroring ghost line."""
    out = {}
    for b, S in enumerate(subs):
        bx, by = b % px, b // px
        nbr = [by * px + bx - 1 if bx > 0 else -1, by * px + bx + 1 if bx < px - 1 else -1,
               (by - 1) * px + bx if by > 0 else -1, (by + 1) * px + bx if by < py - 1 else -1]
        for c, j, i in itertools.product(range(3), range(S["ny"]), range(S["nx"])):
            for side, n in enumerate(nbr):
                if n < 0:
                    continue
                N = subs[n]
                if side == 0 and i < sw:
                    dst = N["base"] + c * N["plane"] + (j + sw) * N["pitch"] + (N["nx"] + i + col0)
                elif side == 1 and i >= S["nx"] - sw:
                    dst = N["base"] + c * N["plane"] + (j + sw) * N["pitch"] + (i - S["nx"] + col0)
                elif side == 2 and j < sw:
                    dst = N["base"] + c * N["plane"] + (N["ny"] + j + sw) * N["pitch"] + (i + col0)
                elif side == 3 and j >= S["ny"] - sw:
                    dst = N["base"] + c * N["plane"] + (j - S["ny"] + sw) * N["pitch"] + (i + col0)
                else:
                    continue
                assert dst not in out, "two points write one ghost cell"
                out[dst] = (b, c, i, j)
    return out


@pytest.mark.parametrize("order", [2, 4, 6])
@pytest.mark.parametrize("grid", [(37, 29, 2, 3), (40, 40, 4, 4), (65, 33, 3, 2), (27, 60, 1, 5), (30, 30, 1, 1)],
                         ids=["37x29_2x3", "40x40_4x4", "65x33_3x2", "27x60_1x5", "30x30_1x1"])
def test_fused_exchange_writes_what_the_halo_kernel_writes(order, grid):
    NX, NY, px, py = grid
    if NX // px < CW_OF[order] or NY // py < CW_OF[order]:
        pytest.skip("subdomains narrower than a closure block are rejected by sbp_decomp_create")
    sw = (W_OF[order] - 1) // 2
    col0 = (sw + 1) // 2 * 2
    subs, _ = _layout(NX, NY, px, py, sw, col0)
    assert _fused_writes(subs, px, py, sw, col0) == _halo_writes(subs, px, py, sw, col0)
