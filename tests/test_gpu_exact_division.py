"""The exact FP64 WENO5 kernels divide by 3 and 6 with an FMA-corrected
multiplication by the rounded reciprocal instead of a division.  The result must
be the IEEE quotient bit for bit; the kernel parity tests cover it on the golden
fixtures, this test on 2^28 pseudo-random inputs (every exponent, NaN and
infinity included, plus 2^27 in the range the schemes meet)."""
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("seed", [1, 2])
def test_division_by_3_and_6_matches_ieee(gb, seed):
    assert gb.check_exact_division(1 << 27, seed=seed) == 0
