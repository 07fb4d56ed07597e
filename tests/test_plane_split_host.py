"""Host model of the plane kernel's split units (ypass2_split in
csrc/msf_fused.cu), no GPU: unit u takes slot (k1 = u / (n2/2),
l = u % (n2/2)); slots with l = 0 are the edge units (line 0 for k1 < B/2,
line n2/2 otherwise), the others interior units paired with (-k1, -l).

The kernel clears every plane slot right after reading it, which is only
correct if each (item k1, kz line) is read by exactly one unit; the half
spectrum's outputs must also each be written once."""
import pytest

SPLIT2 = {16: (4, 4), 32: (8, 4), 64: (8, 8), 128: (16, 8), 256: (16, 16), 512: (32, 16)}   # P -> (B, A)
PLANES = [(32, 32), (64, 32), (128, 32), (256, 32), (512, 32), (32, 64), (64, 64), (128, 64), (256, 64), (512, 64),
          (32, 128), (64, 128), (128, 128), (256, 128), (32, 256), (64, 256), (128, 256)]


def threads(n1, n2):
    """PlaneShape::NT."""
    return 512 if n2 * (n1 // 2) >= 4096 else 256


def units(n1, n2):
    B, A = SPLIT2[n1 // 2]
    H = n2 // 2
    NT = threads(n1, n2)
    rot = H % 64 == 0 and NT % H == 0   # odd passes rotated by 32 within each k1 block
    for u in range(B * H):
        kk = u // H
        ll = (u + ((u // NT) & 1) * 32) % H if rot else u % H
        if ll == 0:
            l = lp = 0 if kk < B // 2 else n2 // 2
            k1 = kk % (B // 2)
            k1p = B - k1 if k1 else B // 2
            yield u, True, (k1, l), (k1p, lp)
        else:
            yield u, False, (kk, ll), ((B - kk) & (B - 1), n2 - ll)


@pytest.mark.parametrize("n1,n2", PLANES)
def test_every_item_read_once(n1, n2):
    B, A = SPLIT2[n1 // 2]
    seen = set()
    for _, _, a, b in units(n1, n2):
        assert a != b
        for it in (a, b):
            assert it not in seen
            seen.add(it)
    assert seen == {(k1, l) for k1 in range(B) for l in range(n2)}


@pytest.mark.parametrize("n1,n2", PLANES)
def test_every_output_written_once(n1, n2):
    """Outputs (q, k), k = 0 .. n2/2, q = 0 .. n1-1 (both halves q and q + P)."""
    B, A = SPLIT2[n1 // 2]
    P = n1 // 2
    out = []
    for _, edge, (k1, l), (k1p, lp) in units(n1, n2):
        if edge and k1 == 0:
            out += [(B * k2, l) for k2 in range(A)] + [(B // 2 + B * k2, l) for k2 in range(A)]
        elif k1 == 0:
            out += [(B * k2, l) for k2 in range(A)]
        else:
            out += [(k1 + B * k2, l) for k2 in range(A)]
            if edge:
                out += [(k1p + B * k2, l) for k2 in range(A)]
    full = [(q, k) for q, k in out] + [(q + P, k) for q, k in out]
    assert sorted(full) == sorted((q, k) for q in range(n1) for k in range(n2 // 2 + 1))


def test_twiddle_index_uniform_per_warp():
    """k1 (and so the twiddle index) is the same for 32 consecutive units
    whenever n2/2 is a multiple of 32."""
    for n1, n2 in PLANES:
        if (n2 // 2) % 32:
            continue
        us = list(units(n1, n2))
        for w in range(0, len(us), 32):
            assert len({u // (n2 // 2) for u, *_ in us[w:w + 32]}) == 1


@pytest.mark.parametrize("n1,n2", [(256, 128), (128, 128), (64, 256)])
def test_edge_units_spread_over_warps(n1, n2):
    """With the odd passes rotated, no warp holds more edge units than the
    passes it makes need: at the headline shape (two passes) one per warp."""
    NT = threads(n1, n2)
    per_warp = {}
    for u, edge, *_ in units(n1, n2):
        if edge:
            w = (u % NT) // 32
            per_warp[w] = per_warp.get(w, 0) + 1
    B, _ = SPLIT2[n1 // 2]
    assert max(per_warp.values()) == -(-B // (NT // 32))
    if (n1, n2) == (256, 128):
        assert sorted(per_warp) == list(range(16)) and set(per_warp.values()) == {1}
