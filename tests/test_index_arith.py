"""Integer identities the kernels rely on, checked exhaustively on the CPU."""
import os
import re

CSRC = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "asmooth_gb300",
                    "csrc")


def test_deposit_reciprocal_division():
    """k_deposit_items splits a cell number c of a pair's box into (x, y, z) with
    floor(c / d) = (c * ceil(2^15 / d)) >> 15; exact for every c below the tile's
    cell count and every d up to a tile face."""
    src = open(os.path.join(CSRC, "asg_deposit.cu")).read()
    ts = int(re.search(r"constexpr int TS = (\d+);", src).group(1))
    assert "#define ASG_M15(d) ((32768 + (d) - 1) / (d))" in src
    for d in range(1, ts * ts + 1):
        m = (32768 + d - 1) // d
        for c in range(ts ** 3):
            assert (c * m) >> 15 == c // d, (c, d)
        assert (ts ** 3 - 1) * m < 2 ** 31  # no overflow of the int product


def test_dens_fixed_point_chunks():
    """k_dens_scatter sums 32 lanes' 64-bit terms (below 2^44) as two 32-bit
    warp reductions of 22-bit chunks: neither chunk sum can overflow."""
    src = open(os.path.join(CSRC, "asg_knn.cu")).read()
    assert "f & 0x3fffffull" in src and "f >> 22" in src
    lo_max, hi_max = 2 ** 22 - 1, (2 ** 44 - 1) >> 22
    assert 32 * lo_max < 2 ** 32 and 32 * hi_max < 2 ** 32
