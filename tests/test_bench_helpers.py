"""Host-side figures of bench.py (no GPU)."""

import math

import bench


def test_fft_flop_fraction_of_the_1d_solve():
    r = bench.fft_flop_fraction(128, 1, 200, 1.0)
    # 12 real transforms of 2.5 n log2 n flops per step: 30 log2 n flops per DOF*step
    assert r["fft_flops_per_dof_step"] == 30 * 7
    assert math.isclose(r["achieved_tflops"], 210 * 128 * 200 / 1e-3 / 1e12)
    assert math.isclose(r["peak_tflops"], 152 * 128 * 2 * 2.07e3 / 1e6)
    assert math.isclose(r["frac"], r["achieved_tflops"] / r["peak_tflops"])
