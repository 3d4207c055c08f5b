"""The checked build (RT_CHECKED: every queue position and path index of the wavefront kernels checked
against the path capacity, out-of-range ones flagged instead of accessed) runs the textured, two-level
and plain scenes through single renders, ray casts and a batch without raising its error flag, and gives
the same results as the normal build — the bounds-check pass that stands in for a memory checker."""
import os
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = Path(__file__).resolve().parent


def test_checked_build_matches_and_stays_in_bounds(tmp_path):
    sys.path.insert(0, str(HERE.parent / "reina-vk_gb300"))
    import build

    normal = build.build()
    checked = build.build_checked()
    results = []
    for lib, name in ((normal, "normal"), (checked, "checked")):
        out = tmp_path / f"{name}.npz"
        env = dict(os.environ, REINA_GB300_LIB=str(lib))
        res = subprocess.run([sys.executable, str(HERE / "checked_run.py"), str(out)], env=env, capture_output=True,
                             text=True, timeout=900)
        assert res.returncode == 0, res.stderr[-2000:]
        results.append(np.load(out))
    a, b = results
    assert set(a.files) == set(b.files)
    for k in a.files:
        if k.endswith("_hits"):
            assert np.array_equal(a[k], b[k]), k
        else:
            x, y = a[k].astype(np.float64), b[k].astype(np.float64)
            ok = (np.abs(x - y) <= 1e-5 * np.abs(y) + 1e-7) | (np.isnan(x) & np.isnan(y))
            assert ok.all(axis=-1).mean() >= 0.999, k
