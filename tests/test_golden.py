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
