"""The export fixtures (tests/golden/export_*.npz) against the reference's own
writers (src/VTKDatExport.cpp through oracle/_ref): regenerated here, they
must reproduce the committed bytes. Skipped where the reference library is not
built (it needs the reference sources)."""
import os
import sys

import numpy as np
import pytest

from conftest import GOLDEN

sys.path.insert(0, GOLDEN)


def test_export_fixtures_match_reference(tmp_path, oracle_lib):
    O = oracle_lib
    if not O.RefSolver.available():
        pytest.skip("oracle/_ref not built (reference sources absent)")
    import make_golden as M

    for name, spec in M.EXPORT_CASES.items():
        want = np.load(os.path.join(GOLDEN, f"{name}.npz"))
        out = tmp_path / name
        out.mkdir()
        # regenerate into a scratch copy and compare every array
        saved = M.HERE
        try:
            M.HERE = str(out)
            M.run_export_case(name, spec, str(out))
        finally:
            M.HERE = saved
        got = np.load(out / f"{name}.npz")
        assert sorted(got.files) == sorted(want.files)
        for k in want.files:
            np.testing.assert_array_equal(got[k], want[k], err_msg=f"{name}/{k}")
