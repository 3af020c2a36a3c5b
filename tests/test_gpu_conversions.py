"""The batched kernel converts between 32.32 fixed point and float on the
hardware converters; they must give the integer restatements' bits
(shy_math.h: shy_q32 = llrintf(v * 2^32), shy_unq = (float)((double)q * 2^-32))
over every float with |v| < 2^31 and 2^31 + 2^27 int64 values, including
those past 2^53 that take the restatement itself.  The device kernels' erf
(float-float, shy_erff_ff) must give the FP64 evaluation's bits (shy_erff)
for every one of the 2^32 floats, and the batched kernel's float evaporation
division (shy_evap_div_ff) the integer restatement's (shy_evap_div) for every
positive float at the default evaporation rate and three others, as must the
exact mode's volume evaporation (shy_evap_mul_ff); the edge height
(shy_minus_0002) must give the double expression's for every float."""
import pytest


@pytest.mark.gpu
def test_hardware_conversions_match_integer_restatements(shy):
    assert shy.check_conversions() == (0, 0, 0, 0, 0)


def test_check_conversions_rejects_null(shy):
    # the argument check runs before any device work
    assert shy.lib().shy_check_conversions(None) == -1
