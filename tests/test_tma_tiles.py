"""Tile copies of the TMA-staged D_eo (k_dslash_tma, tile_segment and
tma_tile in milc_qcd_gb300/csrc): the copy list of every tile, restated here
line for line, stays inside the link planes and the tile's shared memory,
starts and ends on 16-byte boundaries, adds up to the tile's 1152 bytes per
site, and puts into slot i (slot hb - h0 along x) exactly the link that site
h0 + i reads for each direction and kind.  This is the CPU check run before
the kernel's first launch; the GPU tests compare its solves with the oracle."""
import pytest


def site_coords(g, par, h):
    nx, ny, nz, nt = g
    q = 2 * h; xe = q % nx; r = q // nx
    y = r % ny; r //= ny; z = r % nz; t = r // nz
    x = xe + ((xe + y + z + t + par) & 1)
    return x, y, z, t

def cb_index(g, x, y, z, t):
    nx, ny, nz, nt = g
    return (x + nx * (y + ny * (z + nz * t))) >> 1

def tma_tile(g, G):
    nx, ny, nz, nt = g
    if nx % 4 or ny < 4 or nz < 4 or nt < 4 or G < 1 or G > 16: return None
    nx2 = nx // 2
    for r in range(ny, 0, -1):
        if ny % r: continue
        t = r * nx2
        if t * G > 256 or (t * G) % 32: continue
        return t, r
    return None

def tile_segment(g, T, R, h0, l, seg):
    nx, ny, nz, nt = g
    mu, kind = l >> 2, l & 3
    s = 0 if kind < 2 else (1 if kind == 2 else 3)
    nx2 = nx >> 1
    row = h0 // nx2; y0 = row % ny; pz = row // ny; z = pz % nz; t = pz // nz
    if s == 0 or mu == 0:
        return None if seg else (h0, 0, T)
    if mu == 1:
        yr = y0 - s
        if yr < 0: yr += ny
        n1 = min(R, ny - yr); pbase = pz * ny * nx2
        if seg == 0: return (pbase + yr * nx2, 0, n1 * nx2)
        if n1 == R: return None
        return (pbase, n1 * nx2, (R - n1) * nx2)
    if seg: return None
    if mu == 2:
        zz = z - s
        if zz < 0: zz += nz
        src0 = ((t * nz + zz) * ny + y0) * nx2
    else:
        tt = t - s
        if tt < 0: tt += nt
        src0 = ((tt * nz + z) * ny + y0) * nx2
    return (src0, 0, T)

def check(g, G, par):
    nx, ny, nz, nt = g
    Vh = nx * ny * nz * nt // 2
    tt = tma_tile(g, G)
    if tt is None: return "no tile"
    T, R = tt
    assert Vh % T == 0 and Vh % 2 == 0
    opar = 1 - par
    for b in range(Vh // T):
        h0 = b * T
        slots = {}
        total = 0
        for c in range(160):
            l, q, seg = c // 10, (c % 10) >> 1, c & 1
            sg = tile_segment(g, T, R, h0, l, seg)
            if sg is None: continue
            src0, loc0, cnt = sg
            mu, kind = l >> 2, l & 3
            sp = par if kind < 2 else opar
            assert 0 <= src0 and src0 + cnt <= Vh, (g, b, l, sg)
            reg = l * 72 * T
            if q < 4:
                src_b = (((sp * 4 + mu) * 4 + q) * Vh + src0) * 16; dst_b = reg + q * 16 * T + 16 * loc0; nb = cnt * 16
                assert dst_b + nb <= reg + 64 * T
            else:
                src_b = ((sp * 4 + mu) * Vh + src0) * 8; dst_b = reg + 64 * T + 8 * loc0; nb = cnt * 8
                assert dst_b + nb <= reg + 72 * T
            assert src_b % 16 == 0 and dst_b % 16 == 0 and nb % 16 == 0, (g, l, q, sg)
            assert dst_b + nb <= T * 1152
            total += nb
            for j in range(cnt):
                key = (l, q, loc0 + j)
                assert key not in slots
                slots[key] = src0 + j
        assert total == T * 1152, (total, T * 1152)
        for i in range(T):
            h = h0 + i
            x, y, z, t = site_coords(g, par, h)
            L = [nx, ny, nz, nt]
            for mu in range(4):
                c = [x, y, z, t]
                def nb(d):
                    cc = list(c); cc[mu] = (cc[mu] + d) % L[mu]; return cb_index(g, *cc)
                hb1, hb3 = nb(-1), nb(-3)
                jb1 = hb1 - h0 if mu == 0 else i
                jb3 = hb3 - h0 if mu == 0 else i
                for kind, j, want in ((0, i, h), (1, i, h), (2, jb1, hb1), (3, jb3, hb3)):
                    assert 0 <= j < T, (g, mu, kind, j)
                    for q in range(5):
                        assert slots[(4 * mu + kind, q, j)] == want, (g, b, i, mu, kind, q, slots[(4 * mu + kind, q, j)], want)
    return "ok T=%d R=%d" % (T, R)



@pytest.mark.parametrize("dims", [(4, 4, 4, 8), (8, 8, 8, 8), (8, 12, 8, 8), (12, 8, 8, 8), (16, 16, 16, 16)])
@pytest.mark.parametrize("G", [2, 4, 8, 16])
@pytest.mark.parametrize("par", [0, 1])
def test_tile_copies(dims, G, par):
    out = check(dims, G, par)
    assert out.startswith("ok") or out == "no tile"


def test_tile_choice():
    assert tma_tile((32, 32, 32, 64), 8) == (32, 2)
    assert tma_tile((32, 32, 32, 64), 16) == (16, 1)
    assert tma_tile((48, 48, 48, 96), 8) == (24, 1)
    assert tma_tile((6, 6, 6, 6), 8) is None       # nx/2 odd: rows not 16-byte aligned
    assert tma_tile((4, 4, 4, 8), 2) is None        # a whole warp needs more rows than ny holds
