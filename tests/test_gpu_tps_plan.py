"""The TPS plan (compaction of the valid vectors in index order and the subdomain
layout of ThinPlateSplineSubdom.__init__, thin_plate_spline_subdom.py:38-91) from
fi_tps_plan_make, one block for small passes and the multi-block form for large
ones, against numpy's compaction and the oracle's layout: the centres, values and
selection exactly, the header (count, subdomain grid, smoothing, extremes, buffers)
exactly."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [500, 4000, 4097, 65025, 300001])
def test_plan_matches_numpy_and_oracle(n):
    import torch

    from fluidimage_gb300 import _lib as L
    from oracle import piv as O

    rng = np.random.default_rng(n)
    side = int(np.ceil(np.sqrt(n)))
    xs = (8.0 * (np.arange(n) % side) + 16.0 + 0.5 * rng.integers(0, 3, n)).astype(np.float32)
    ys = (8.0 * (np.arange(n) // side) + 16.0).astype(np.float32)
    dx = rng.normal(0, 2, n).astype(np.float32)
    dy = rng.normal(0, 2, n).astype(np.float32)
    dx[rng.random(n) < 0.07] = np.nan
    dy[rng.random(n) < 0.03] = np.nan
    dev = torch.device("cuda")
    t = lambda a: torch.as_tensor(a, device=dev)  # noqa: E731
    plan = torch.empty(L.TPS_PLAN_BYTES, dtype=torch.uint8, device=dev)
    cx = torch.empty(n, dtype=torch.float64, device=dev)
    cy = torch.empty(n, dtype=torch.float64, device=dev)
    ux = torch.empty(n, dtype=torch.float32, device=dev)
    uy = torch.empty(n, dtype=torch.float32, device=dev)
    sel = torch.empty(n, dtype=torch.int32, device=dev)
    tx, ty, tdx, tdy = t(xs), t(ys), t(dx), t(dy)
    L.check(L.load().fi_tps_plan_make(L.ptr(tx), L.ptr(ty), L.ptr(tdx), L.ptr(tdy), n, 200, 0.5,
                                      20.0, L.ptr(plan), L.ptr(cx), L.ptr(cy), L.ptr(ux),
                                      L.ptr(uy), L.ptr(sel), None), "fi_tps_plan_make")
    torch.cuda.synchronize()
    hdr = L.TpsPlan.from_buffer_copy(plan.cpu().numpy().tobytes())
    valid = ~(np.isnan(dx) | np.isnan(dy))
    nv = int(valid.sum())
    assert hdr.status == 0 and hdr.num_centers == nv
    np.testing.assert_array_equal(sel.cpu().numpy()[:nv], np.nonzero(valid)[0])
    np.testing.assert_array_equal(cx.cpu().numpy()[:nv], xs[valid].astype(np.float64))
    np.testing.assert_array_equal(cy.cpu().numpy()[:nv], ys[valid].astype(np.float64))
    np.testing.assert_array_equal(ux.cpu().numpy()[:nv], dx[valid])
    np.testing.assert_array_equal(uy.cpu().numpy()[:nv], dy[valid])
    centers = np.vstack([ys[valid].astype(np.float64), xs[valid].astype(np.float64)])
    tps = O.TPSSubdom(centers, 200, 0.5)
    assert (hdr.nb_subdomx, hdr.nb_subdomy) == (tps.nb_subdomx, tps.nb_subdomy)
    assert hdr.smoothing == tps.smoothing_coef
    assert (hdr.x_min, hdr.x_max) == (centers[1].min(), centers[1].max())
    assert (hdr.y_min, hdr.y_max) == (centers[0].min(), centers[0].max())
    np.testing.assert_array_equal(hdr.x_min - hdr.buffer_x, tps.lim_min_x[0])
    np.testing.assert_array_equal(hdr.y_min - hdr.buffer_y, tps.lim_min_y[0])
