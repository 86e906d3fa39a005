"""CPU check of the index arithmetic the Wolff kernel relies on.

The square-lattice Wolff growth takes the row of a queued site, floor(k / hy),
as the high word of k * ceil(2^32 / hy) (mcs_wolff.cuh, wolff_mdiv /
wolff_links) whenever the lattice has at most 2^16 sites.  This checks that
identity on every k < 2^16 at the boundaries of each quotient, for every
half-width 1 < hy <= 2^15.
"""


def _row(k, hy):
    m = ((1 << 32) + hy - 1) // hy
    return (k * m) >> 32


def test_multiply_high_row_is_exact_below_2_16():
    for hy in range(2, (1 << 15) + 1):
        for q in range(0, ((1 << 16) - 1) // hy + 1):
            for k in (q * hy, q * hy + hy - 1):
                if k < (1 << 16):
                    assert _row(k, hy) == k // hy, (hy, k)
        assert _row((1 << 16) - 1, hy) == ((1 << 16) - 1) // hy
