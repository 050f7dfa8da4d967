"""Oracle regression against the committed fixtures in tests/golden/
(generated by tests/golden/make_golden.py from the oracle; the reference has no
golden vectors of its own)."""
import sys
from pathlib import Path

import numpy as np
import pytest

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE / "golden"))
import make_golden  # noqa: E402

CASES = make_golden.cases()


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_oracle_matches_golden(case):
    name, kind, kw, steps = case
    ref = np.load(HERE / "golden" / f"{name}.npz")
    got = make_golden.run(name, kind, kw, steps)
    for k in ref.files:
        # libm exp/erfc may differ by an ulp between hosts (x86_64 / aarch64)
        np.testing.assert_allclose(got[k], ref[k], rtol=1e-11, atol=1e-13, err_msg=k)


def _numpy_run(kind, kw, steps):
    """make_golden.run with the independent numpy restatement in place of the
    C++ oracle (the same states, parameters and interior slices)."""
    from mhd3d_mpi_fortran_gb300 import ics
    from mhd3d_mpi_fortran_gb300.abi import Params
    from oracle.mhd_numpy import NumpyMHD
    s = make_golden.state_of(kind)
    g = s.grid
    tau = 2e-3 if kind == "tube" else 0.5 * ics.cfl_dt(s)
    n = NumpyMHD(Params(g.nx0, g.ny0, g.nz0, tau=tau, **kw), s)
    for _ in range(steps):
        n.step()
    f, ng = n.state(), g.ng
    if kind == "tube":
        return {k: f[k][ng + 1, ng + 1, ng:ng + g.nz0] for k in ("rho", "p", "vz", "bx")}
    ext = {"bi": (1, 0, 0), "bj": (0, 1, 0), "bk": (0, 0, 1)}
    return {k: f[k][ng:ng + g.nx0 + ext.get(k, (0, 0, 0))[0], ng:ng + g.ny0 + ext.get(k, (0, 0, 0))[1],
                    ng:ng + g.nz0 + ext.get(k, (0, 0, 0))[2]] for k in make_golden.FIELDS}


NUMPY_CASES = CASES


@pytest.mark.parametrize("case", NUMPY_CASES, ids=[c[0] for c in NUMPY_CASES])
def test_independent_restatement_reproduces_golden(case):
    """The committed fixtures (made by the C++ oracle) are reproduced by the
    numpy restatement written separately from the Fortran."""
    name, kind, kw, steps = case
    ref = np.load(HERE / "golden" / f"{name}.npz")
    got = _numpy_run(kind, kw, steps)
    for k in ref.files:
        np.testing.assert_allclose(got[k], ref[k], rtol=1e-11, atol=1e-13, err_msg=k)
