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


def test_dens_fixed_point_sums():
    """k_dens_scatter counts a weight w as w * 2^(FIX_BITS - e_j), below
    2^(FIX_BITS + 4) (w <= 8 hinv_j^3 < 2^(e_j + 3), one rounding); a lane sums
    at most the 32 queries of a bundle per bucket as a double-float, rounds hi
    and lo to integers and adds them to acc[j] with one atomic: neither the
    per-bucket sum nor acc can overflow before a receiver collects
    2^(60 - FIX_BITS) terms."""
    src = open(os.path.join(CSRC, "asg_knn.cu")).read()
    fix = int(re.search(r"constexpr int FIX_BITS = (\d+);", src).group(1))
    assert "two_sum_acc_nonneg(sh, sl, __fmul_rn(w, sc));" in src
    assert "__float2ll_rn(sh) + __float2ll_rn(sl)" in src
    term = 2 ** (fix + 4)
    assert 32 * term < 2 ** 63
    assert 2 ** (60 - fix) * term <= 2 ** 64 and 2 ** (60 - fix) >= 2 ** 20
