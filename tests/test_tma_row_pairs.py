"""The two-step smoother's TMA row-pair layout, checked on the CPU.

k_cheb_pair (simcoflow3d_gb300/csrc/k_solver.cu) stages each FP32 array of a
level through a tensor map that views it as (2 sy, (n1+2)/2, n2+2) floats:
row pairs, so that every global stride is a multiple of 16 bytes.  A tile
arrives as two boxes per array, one over the even rows (x = i) and one over
the odd rows (x = sy + i) of its row pairs, each box's first x rounded down
to a multiple of 4 floats.  This test restates the box origins and the
per-thread shared-memory offsets (c2_idx) in Python, fills the boxes the way
the copy engine does (coordinates outside the tensor read as 0), and checks
that every read of every interior first-step cell lands on the intended
element, for row lengths of both residues mod 4 and odd n1."""
import pytest

TX, TY = 32, 8
EX, EY = TX + 2, TY + 2
WA, WE = 36, 40
HA, HN, HX = TY // 2 + 1, TY // 2 + 2, TY // 2 + 3


def _round32(v):
    return (v + 31) // 32 * 32


BA, BE, BN, BX = _round32(WA * HA), _round32(WE * HA), _round32(WA * HN), _round32(WE * HX)
GB, GD, GT, GP = 0, 2 * BA, 4 * BA, 6 * BA
GE = 8 * BA
GN = GE + 2 * BE
GX = GN + 2 * BN
SLOT = GX + 2 * BX


def _fill(n0, n1, bx, by):
    """Shared-memory slot contents as the copy engine writes them: offset ->
    (i, j) of the element, or None where the box lies outside the tensor."""
    sy = n0 + 2
    npairs = (n1 + 2) // 2
    slot = {}

    def box(base, w, h, x0, y0):
        for r in range(h):
            for col in range(w):
                x, y = x0 + col, y0 + r
                off = base + r * w + col
                assert off not in slot
                if 0 <= x < 2 * sy and 0 <= y < npairs:
                    odd = x >= sy
                    slot[off] = (x - sy if odd else x, 2 * y + (1 if odd else 0))
                else:
                    slot[off] = None

    ya, yn = by // 2, by // 2 - 1
    for p in range(2):
        xa = (p * sy + bx) & ~3
        xe = (p * sy + bx - 1) & ~3
        assert xa % 4 == 0 and xe % 4 == 0          # TMA: x times 4 bytes a multiple of 16
        for g in (GB, GD, GT, GP):
            box(g + p * BA, WA, HA, xa, ya)
        box(GE + p * BE, WE, HA, xe, ya)
        box(GN + p * BN, WA, HN, xa, yn)
        box(GX + p * BX, WE, HX, xe, yn)
    return slot


def _idx(ex, ey, sha, she):
    p, q = ey & 1, (ey & 1) ^ 1
    return {
        "a": p * BA + (ey >> 1) * WA + ex + sha[p],
        "e": GE + p * BE + (ey >> 1) * WE + ex + she[p],
        "n": GN + p * BN + ((ey + 2) >> 1) * WA + ex + sha[p],
        "s": GN + q * BN + ((ey + 1) >> 1) * WA + ex + sha[q],
        "x": GX + p * BX + ((ey + 2) >> 1) * WE + ex + she[p],
        "xn": GX + q * BX + ((ey + 3) >> 1) * WE + ex + she[q],
        "xs": GX + q * BX + ((ey + 1) >> 1) * WE + ex + she[q],
    }


def _cells():
    """The 34 x 10 first-step cells: each thread's own column and the halo
    ring handed out as the kernel does."""
    cells = [(tx + 1, ty + 1) for ty in range(TY) for tx in range(TX)]
    nh = EX * EY - TX * TY
    for tid in range(TX * TY):
        if tid < EX:
            cells.append((tid, 0))
        elif tid < 2 * EX:
            cells.append((tid - EX, EY - 1))
        elif tid < 2 * EX + TY:
            cells.append((0, tid - 2 * EX + 1))
        elif tid < nh:
            cells.append((EX - 1, tid - 2 * EX - TY + 1))
    assert len(set(cells)) == EX * EY
    return cells


@pytest.mark.parametrize("n0,n1", [(70, 45), (68, 46), (256, 256), (64, 64), (34, 9), (2, 2)])
def test_every_first_step_read_lands_on_its_element(n0, n1):
    sy = n0 + 2
    assert n0 % 2 == 0 and (sy * (n1 + 2)) % 4 == 0   # the kernel's shape condition
    assert SLOT % 32 == 0 and all(b % 32 == 0 for b in (BA, BE, BN, BX))   # 128-byte boxes
    for bx in range(0, n0, TX):
        for by in range(0, n1, TY):
            slot = _fill(n0, n1, bx, by)
            sha = [(p * sy + bx) & 3 for p in range(2)]
            she = [p * sy + bx - ((p * sy + bx - 1) & ~3) for p in range(2)]
            for ex, ey in _cells():
                i, j = bx + ex, by + ey
                if not (1 <= i <= n0 and 1 <= j <= n1):
                    continue
                t = _idx(ex, ey, sha, she)
                want = [(GB + t["a"], (i, j)), (GD + t["a"], (i, j)), (GT + t["a"], (i, j)),
                        (GP + t["a"], (i, j)), (t["e"], (i, j)), (t["e"] - 1, (i - 1, j)),
                        (t["n"], (i, j)), (t["s"], (i, j - 1)), (t["x"], (i, j)), (t["x"] + 1, (i + 1, j)),
                        (t["x"] - 1, (i - 1, j)), (t["xn"], (i, j + 1)), (t["xs"], (i, j - 1))]
                for off, ij in want:
                    assert 0 <= off < SLOT
                    if ij[1] <= 2 * ((n1 + 2) // 2) - 1:
                        assert slot[off] == ij, (n0, n1, bx, by, ex, ey, off, slot[off], ij)
                    else:   # the unpaired last ghost row of an odd n1 reads as 0
                        assert slot[off] is None


def test_shapes_outside_the_row_pair_view():
    # odd n0 (a row pair is not 16-byte aligned), or sy = 2 mod 4 with an odd
    # number of ghosted rows (the plane stride is not): one-step launches
    for n0, n1 in [(69, 44), (68, 45)]:
        sy = n0 + 2
        assert not (n0 % 2 == 0 and (sy * (n1 + 2)) % 4 == 0)
    # sy = 0 mod 4 takes any n1
    assert all((72 * (n1 + 2)) % 4 == 0 for n1 in range(1, 40))
