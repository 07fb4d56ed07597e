"""Host model of the x pass's pass-2 reads (k_xpower_tma in
csrc/msf_xtma.cu), no GPU.

A tile holds n0 rows of W complex values (8 bytes each); in pass 2 a warp's
lane (k1, l) reads sample n1 of its item at row A k1 + n1, column l.  With
rows narrower than 128 bytes the 32 / W k1 rows of a warp sit A W 8 bytes
apart, on the same banks, so each k1 group reads its samples cyclically
shifted by g = k1 mod RG rows (RG = rows per 128 bytes).  The shift must
bring every warp load to two wavefronts (256 bytes: the least there is)
and leave the power |X[k]|^2 of the group's DFT unchanged."""
import numpy as np
import pytest

A, B = 16, 16      # Split2<256>: the 256-point x FFT as 16 x 16


def rg(W):
    rw = 128 // (W * 8)
    return min(rw, A) if rw > 1 else 1


def wavefronts(word_addrs):
    """Shared-memory wavefronts of one warp access: the most distinct
    4-byte words any of the 32 banks must deliver."""
    per_bank = {}
    for w in word_addrs:
        per_bank.setdefault(w % 32, set()).add(w)
    return max(len(v) for v in per_bank.values())


def warp_words(W, warp, n1, shift=True):
    words = []
    for lane in range(32):
        it = 32 * warp + lane
        l, k1 = it % W, it // W
        g = k1 % rg(W) if shift else 0
        row = A * k1 + (n1 + g) % A
        f2 = row * W + l                       # float2 index in the tile
        words += [2 * f2, 2 * f2 + 1]
    return words


@pytest.mark.parametrize("W", [8, 16, 32])
def test_pass2_reads_take_two_wavefronts(W):
    warps = B * W // 32
    for warp in range(warps):
        for n1 in range(A):
            assert wavefronts(warp_words(W, warp, n1)) == 2, (W, warp, n1)


def test_unshifted_eight_column_reads_conflict():
    """Without the shift the four k1 rows of a warp share 16 banks: four
    wavefronts per load, twice the least."""
    assert max(wavefronts(warp_words(8, w, n1, shift=False)) for w in range(4) for n1 in range(A)) == 4


def test_power_is_invariant_under_the_shift():
    rng = np.random.default_rng(5)
    x = rng.standard_normal(A) + 1j * rng.standard_normal(A)
    p = np.abs(np.fft.fft(x)) ** 2
    for g in range(A):
        q = np.abs(np.fft.fft(np.roll(x, -g))) ** 2      # sample (n1 + g) mod A at position n1
        np.testing.assert_allclose(q, p, rtol=1e-12, atol=1e-12 * p.max())


def test_only_the_last_rg_minus_one_loads_wrap():
    """The kernel selects the wrapped address only for n1 + RG - 1 >= A."""
    for W in (8, 16, 32):
        R = rg(W)
        for g in range(R):
            for n1 in range(A):
                wraps = n1 + g >= A
                assert not wraps or n1 + R - 1 >= A
