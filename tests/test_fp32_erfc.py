"""The FP32 path's erfc (Moments<float>::erfc_pos in csrc/mhd_kernels.cuh):
Numerical Recipes' Chebyshev fit "erfcc" (Press et al., 2nd ed., sec. 6.2),
whose published fractional error is below 1.2e-7 for every argument.  The
coefficients are read from the shipped source and checked against scipy's
erfc -- no GPU; the device evaluation itself is covered by the FP32 error
budget of the GPU suite."""
import re
from pathlib import Path

import numpy as np
import pytest

special = pytest.importorskip("scipy.special")

SRC = (Path(__file__).resolve().parents[1] / "mhd3d_mpi_fortran_gb300" / "csrc" / "mhd_kernels.cuh").read_text()


def shipped_coefficients():
    body = re.search(r"float erfc_pos\(float z\) \{(.*?)\n  \}", SRC, re.S).group(1)
    first = re.search(r"fmaf\(t, ([-0-9.]+)f, ([-0-9.]+)f\)", body)
    rest = re.findall(r"q = fmaf\(t, q, ([-0-9.]+)f\)", body)
    return [float(first.group(1)), float(first.group(2))] + [float(c) for c in rest]


def erfcc(z, coef, dtype=np.float64):
    z = np.asarray(z, dtype=dtype)
    t = dtype(1.0) / (dtype(0.5) * z + dtype(1.0))
    q = dtype(coef[0]) * t + dtype(coef[1])
    for c in coef[2:]:
        q = t * q + dtype(c)
    return t * np.exp(-z * z + q)


def test_the_coefficients_are_the_ten_of_erfcc():
    c = shipped_coefficients()
    assert len(c) == 10
    assert c[-1] == pytest.approx(-1.26551223) and c[0] == pytest.approx(0.17087277)


def test_fractional_error_within_the_published_bound():
    z = np.concatenate([np.linspace(0.0, 4.0, 40001), np.linspace(4.0, 9.0, 5001)])
    ref = special.erfc(z)
    err = np.abs(erfcc(z, shipped_coefficients()) / ref - 1.0)
    assert err.max() < 1.2e-7, err.max()


def test_single_precision_evaluation_stays_near_float32_rounding():
    """Evaluated in float32 the fractional error grows with z, where the
    rounding of the exponent's argument -z^2 + q is magnified by exp (1.5e-5
    near z = 9, on values of order 1e-35); where erfc is of order one it stays
    below 1e-6, and the absolute error (float32 rounding of the ten-term sum)
    stays below 5e-7 everywhere."""
    z = np.linspace(0.0, 9.0, 20001)
    ref = special.erfc(z)
    got = erfcc(z.astype(np.float32), shipped_coefficients(), np.float32).astype(np.float64)
    near = z <= 2.0
    assert np.abs(got[near] / ref[near] - 1.0).max() < 1e-6
    assert np.abs(got - ref).max() < 5e-7


def test_half_erfc_sign_handling():
    """half_erfc returns 0.5 erfc(-x) (left) or 0.5 erfc(x) (right) from
    erfc(|x|), using 1 - h on the far side: the identity erfc(-x) = 2 - erfc(x)."""
    c = shipped_coefficients()
    x = np.linspace(-6.0, 6.0, 2401)
    h = 0.5 * erfcc(np.abs(x), c)
    left = np.where(x <= 0, h, 1.0 - h)
    right = np.where(x >= 0, h, 1.0 - h)
    assert np.abs(left - 0.5 * special.erfc(-x)).max() < 1e-7
    assert np.abs(right - 0.5 * special.erfc(x)).max() < 1e-7
