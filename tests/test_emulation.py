"""The integer-only roundings the batched GPU kernels use in place of FP64
(shy_math.h: shy_q32, shy_unq, shy_evap_div) against the floating-point
expressions they replace.  The full check (stride 1) covers every float and
was run when the routines were written; the suite runs a strided subset."""
import os
import subprocess

ORACLE = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle")


def test_integer_roundings_match_fp64(po):
    exe = os.path.join(ORACLE, "emulation_check")
    assert os.path.exists(exe)
    for evap in ("0.001", "0.01", "0.0005"):
        r = subprocess.run([exe, evap, "61"], capture_output=True, text=True, timeout=300)
        assert r.returncode == 0, r.stdout + r.stderr
        assert "total mismatches 0" in r.stdout


def test_integer_roundings_spot_values(po):
    L = po.lib()
    import ctypes as C
    L.orc_q32_int.argtypes = [C.c_float]
    L.orc_q32_int.restype = C.c_int64
    L.orc_unq_int.argtypes = [C.c_int64]
    L.orc_unq_int.restype = C.c_float
    L.orc_evap_div_int.argtypes = [C.c_float, C.c_float]
    L.orc_evap_div_int.restype = C.c_float
    assert L.orc_q32_int(1.0) == 1 << 32
    assert L.orc_q32_int(-0.5) == -(1 << 31)
    assert L.orc_q32_int(2.0 ** -33) == 0          # half: ties to even
    assert L.orc_q32_int(3 * 2.0 ** -33) == 2
    assert L.orc_unq_int(1 << 32) == 1.0
    assert L.orc_unq_int(-(3 << 30)) == -0.75
    s = C.c_float(0.3).value
    want = C.c_float(s / (1.0 - C.c_float(0.001).value)).value
    assert L.orc_evap_div_int(s, 0.001) == want
