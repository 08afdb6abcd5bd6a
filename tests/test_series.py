"""WorkPIV.calcul_series (the pipelined series API) gives the results of
WorkPIV.calcul, pair by pair and in order."""

import numpy as np
import pytest

from fluidimage_gb300 import WorkPIV, workloads


@pytest.mark.gpu
def test_series_matches_calcul():
    (im0, im1), _ = workloads.config2_images(shape=(512, 512))
    params = workloads.config2_params(WorkPIV.create_default_params())
    work = WorkPIV(params)
    pairs = [(im0, im1), (np.roll(im0, 37, axis=1), np.roll(im1, 37, axis=1)), (im0, im1)]
    singles = [work.calcul({"arrays": p, "names": ("a", "b")}) for p in pairs]
    series = list(work.calcul_series({"arrays": p, "names": ("a", "b")} for p in pairs))
    assert len(series) == len(pairs)
    for a, b in zip(singles, series):
        for pa, pb in zip(a.passes, b.passes):
            np.testing.assert_array_equal(pa.deltaxs, pb.deltaxs)
            np.testing.assert_array_equal(pa.deltays, pb.deltays)
            assert pa.errors == pb.errors
        np.testing.assert_array_equal(a.passes[-1].deltaxs_final, b.passes[-1].deltaxs_final)
        np.testing.assert_array_equal(a.passes[-1].deltays_smooth, b.passes[-1].deltays_smooth)


@pytest.mark.gpu
def test_series_cold_start_matches_calcul():
    """calcul_series as the first call of a fresh process (no TPS table built yet):
    the per-device tables are complete before any stream reads them."""
    import subprocess
    import sys
    from pathlib import Path

    code = r"""
import numpy as np
from fluidimage_gb300 import WorkPIV, workloads
(im0, im1), _ = workloads.config2_images(shape=(512, 512))
params = workloads.config2_params(WorkPIV.create_default_params())
pairs = [(np.roll(im0, 13 * k, axis=1), np.roll(im1, 13 * k, axis=1)) for k in range(4)]
series = list(WorkPIV(params).calcul_series({"arrays": p, "names": ("a", "b")} for p in pairs))
work = WorkPIV(params)
for p, b in zip(pairs, series):
    a = work.calcul({"arrays": p, "names": ("a", "b")})
    np.testing.assert_array_equal(a.passes[-1].deltaxs_final, b.passes[-1].deltaxs_final)
    np.testing.assert_array_equal(a.passes[-1].deltays, b.passes[-1].deltays)
print("ok")
"""
    root = Path(__file__).resolve().parents[1]
    out = subprocess.run([sys.executable, "-c", code], cwd=root, capture_output=True,
                         text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    assert out.stdout.strip().endswith("ok")
