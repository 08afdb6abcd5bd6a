"""Two passes of synthetic PIV results with every attribute a results file holds
(built with the classes given, so that this package's and upstream's objects hold
the same values).  Test infrastructure only."""

from __future__ import annotations

import numpy as np


def build(heavy_cls, multi_cls, couple, params):
    rng = np.random.default_rng(7)

    def f32(n):
        return rng.normal(size=n).astype(np.float32)

    results = multi_cls()
    n0, n1 = 12, 30
    r0 = heavy_cls(
        deltaxs=f32(n0), deltays=f32(n0), xs=24.0 + 16.0 * (np.arange(n0) % 4),
        ys=24.0 + 16.0 * (np.arange(n0) // 4),
        errors={3: "Correlation peak touching boundary.",
                7: "diff neighbour too large (diff2 = 5.25)",
                9: "correl < correl_min"},
        correls_max=rng.random(n0).astype(np.float32), correls=[None] * n0,
        couple=couple, params=params, secondary_peaks=[None] * n0)
    r0.deltaxs_wrong = {3: np.float32(1.5), 7: np.float32(-2.25), 9: np.float32(0.125)}
    r0.deltays_wrong = {3: np.float32(0.5), 7: np.float32(3.0), 9: np.float32(-1.0)}
    r0.deltaxs_approx = rng.normal(size=n1)
    r0.deltays_approx = rng.normal(size=n1)
    r0.ixvecs_approx = 12.0 + 8.0 * (np.arange(n1) % 6)
    r0.iyvecs_approx = 12.0 + 8.0 * (np.arange(n1) // 6)
    r0.deltaxs_tps = [rng.normal(size=15), rng.normal(size=18)]
    r0.deltays_tps = [rng.normal(size=15), rng.normal(size=18)]
    results.append(r0)
    r1 = heavy_cls(
        deltaxs=f32(n1), deltays=f32(n1), xs=rng.normal(size=n1) + 40.0,
        ys=rng.normal(size=n1) + 40.0, errors={}, correls_max=rng.random(n1).astype(np.float32),
        correls=[None] * n1, couple=couple, params=params, secondary_peaks=[None] * n1)
    r1.deltaxs_wrong, r1.deltays_wrong = {}, {}
    r1.xs_smooth = (12.0 + 8.0 * (np.arange(n1) % 6)).astype(np.float32)
    r1.ys_smooth = (12.0 + 8.0 * (np.arange(n1) // 6)).astype(np.float32)
    r1.deltaxs_smooth = rng.normal(size=n1)
    r1.deltays_smooth = rng.normal(size=n1)
    r1.deltaxs_final = rng.normal(size=n1)
    r1.deltays_final = rng.normal(size=n1)
    r1.ixvecs_final = r0.ixvecs_approx.copy()
    r1.iyvecs_final = r0.iyvecs_approx.copy()
    r1.deltaxs_tps = [rng.normal(size=33)]
    r1.deltays_tps = [rng.normal(size=33)]
    results.append(r1)
    return results
