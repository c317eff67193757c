"""The tracking loop replaces some FP64 operations by exact equivalents that
run on other pipes (the FP64 pipe is the loop's bottleneck): the facet
screen's double-to-float conversion on the integer pipe, the mean-free-path
update's division by a correctly rounded reciprocal and two corrections
(Markstein), IEEE comparisons on bit patterns, and the random-number sample
2^-64 (double)seed assembled on the integer pipe.  Every one must give the
FP64 operation's bits; the parity tests check the whole loop, this checks the
pieces on many operands, hard cases included (qsg_check_arithmetic)."""
import pytest

from quicksilver_gb300 import _native as N

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("seed", [1, 0x5eed5eed])
def test_replacements_match_fp64(gpu, seed):
    assert N.check_arithmetic(1 << 24, seed=seed) == (0, 0, 0, 0)


def test_check_arithmetic_arguments(gpu):
    with pytest.raises(N.QsgError) as ei:
        N.check_arithmetic(16, device=N.device_count())
    assert ei.value.code == N.QSG_ERR_INVALID
    assert N.check_arithmetic(0) == (0, 0, 0, 0)


def test_fp64_issue_rate_is_measured(gpu):
    """The FP64 roof the bench reports the tracking kernel against: a few
    times 1e10 FP64 warp instructions per second on a GB300-class part (one
    per ~20 cycles per SM); anything far outside means the probe is broken."""
    rate = N.measure_fp64_rate()
    assert 1e9 < rate < 1e12
    with pytest.raises(N.QsgError):
        N.measure_fp64_rate(device=N.device_count())
