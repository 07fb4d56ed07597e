"""Host model of the bulk-copied z sweep's block partition (k_zs_bulk in
csrc/msf_smooth.cu), no GPU.

A CTA of G row pairs owns the n = nrows * n2 contiguous ints of its rows,
starting at int index `first` of an int32 grid whose base is 16-byte
aligned.  It places block int i at raw[off + i] (off = first mod 4), moves
the hn < 4 ints before the first 16-byte aligned int and the tn < 4 after
the aligned interior by plain loads, and the nb-int interior by one bulk
copy, which needs both ends 16-byte aligned and a size that is a multiple of
16 bytes.  Every int must be moved exactly once and nothing outside the
block (or past the shared-memory array) touched."""
import pytest

SMOOTH = [16, 18, 20, 24, 25, 27, 30, 32, 36, 40, 45, 48, 50, 54, 60, 64, 72, 75, 80, 81, 90, 96, 100, 108,
          120, 125, 128, 135, 144, 150, 160, 162, 180, 192, 200, 216, 225, 240, 243, 250, 256, 512]


def bulk_rows(n2):
    return 32 if n2 <= 128 else (16 if n2 <= 256 else 8)


def partition(first, n):
    off = first & 3
    hn = min(4 - off if off else 0, n)
    nb = (n - hn) & ~3
    tn = n - hn - nb
    return off, hn, nb, tn


@pytest.mark.parametrize("n2", SMOOTH)
def test_blocks_partition_exactly_and_align(n2):
    G = bulk_rows(n2)
    cap = 2 * G * n2 + 4                       # raw ints in shared memory
    for n0n1 in (1, 2, 3, 7, 2 * G - 1, 2 * G, 2 * G + 1, 5 * G + 3):
        V = n0n1 * n2
        rows = n0n1
        pairs = (rows + 1) // 2
        for frame in range(5):                 # frame offsets of every residue mod 4
            for blk in range(-(-pairs // G)):
                r0 = 2 * blk * G
                nrows = min(2 * G, rows - r0)
                assert nrows >= 1
                first = frame * V + r0 * n2
                n = nrows * n2
                off, hn, nb, tn = partition(first, n)
                assert hn + nb + tn == n and 0 <= hn < 4 and 0 <= tn < 4 and nb % 4 == 0
                if nb:
                    assert (first + hn) % 4 == 0            # global source: 16-byte aligned
                    assert (off + hn) % 4 == 0              # shared destination: 16-byte aligned
                    assert nb * 4 <= (1 << 20) - 1          # one mbarrier phase's transaction count
                # the block fits the raw array; the transposed reads
                # raw[off + r n2 + z], r < nrows, stay inside it
                assert off + n <= cap


def test_raw_array_starts_aligned():
    """The raw array follows the line buffer (n2 (G+1) float2) and the
    twiddles (n2 float2): a 16-byte multiple whenever G is even."""
    for n2 in SMOOTH:
        G = bulk_rows(n2)
        assert G % 2 == 0 and (n2 * (G + 2) * 8) % 16 == 0


def test_shared_memory_fits_three_or_four_ctas():
    for n2 in SMOOTH:
        G = bulk_rows(n2)
        smem = n2 * (G + 2) * 8 + (2 * G * n2 + 4) * 4
        assert smem + 1024 <= 233472 // 3, n2       # 228 KB per SM, 1 KB reserved per CTA
