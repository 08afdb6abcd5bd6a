"""fi_griddata (the griddata path of apply_interp, calcul/interpolate/griddata.py:11-27)
against scipy's griddata ('linear', then 'nearest' where NaN) on perturbed window
grids with holes.  Points the kernel flags (cells of cocircular centres, where
several Delaunay triangulations exist and scipy follows Qhull's, or equidistant
nearest centres) are counted and left out; elsewhere the values agree to 1e-9."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _case(seed, nx=21, ny=17, step=16, holes=0.1, half=True, hole_block=None):
    rng = np.random.default_rng(seed)
    ixvecs = 8 + step * np.arange(nx)
    iyvecs = 8 + step * np.arange(ny)
    gx, gy = np.meshgrid(ixvecs, iyvecs)
    gx, gy = gx.ravel().astype(float), gy.ravel().astype(float)
    if half:
        gx += 0.5 * rng.integers(0, 2, gx.size)
        gy += 0.5 * rng.integers(0, 2, gy.size)
    valid = rng.random(gx.size) >= holes
    if hole_block is not None:
        (r0, r1), (c0, c1) = hole_block
        m = np.zeros((ny, nx), bool)
        m[r0:r1, c0:c1] = True
        valid &= ~m.ravel()
    sel = np.nonzero(valid)[0].astype(np.int32)
    vals_x = rng.normal(0, 3, sel.size).astype(np.float32)
    vals_y = rng.normal(0, 3, sel.size).astype(np.float32)
    qx = np.arange(0, ixvecs[-1] + 12, step // 2)
    qy = np.arange(0, iyvecs[-1] + 12, step // 2)
    return ixvecs, iyvecs, gx[sel], gy[sel], sel, vals_x, vals_y, qx, qy


def _scipy(cx, cy, v, qx, qy):
    from scipy import interpolate

    g0, g1 = np.meshgrid(qx, qy)
    pts = np.stack([cx, cy], 1)
    out = interpolate.griddata(pts, v, (g0, g1), "linear")
    nan = np.isnan(out)
    out[nan] = interpolate.griddata(pts, v, (g0, g1), "nearest")[nan]
    return out.ravel()


def _gpu(ixvecs, iyvecs, cx, cy, sel, vx, vy, qx, qy):
    import torch

    from fluidimage_gb300 import _lib as L

    lib = L.load()
    dev = torch.device("cuda")
    g0, g1 = np.meshgrid(qx, qy)
    t = lambda a, dt: torch.as_tensor(np.ascontiguousarray(a, dtype=dt), device=dev)
    tcx, tcy = t(cx, np.float64), t(cy, np.float64)
    tvx, tvy = t(vx, np.float32), t(vy, np.float32)
    tsel = t(sel, np.int32)
    tix, tiy = t(ixvecs, np.int32), t(iyvecs, np.int32)
    tpx, tpy = t(g0.ravel(), np.float64), t(g1.ravel(), np.float64)
    n = tpx.numel()
    nscr = int(lib.fi_griddata_scratch_ints(ixvecs.size, iyvecs.size))
    scratch = torch.empty(nscr, dtype=torch.int32, device=dev)
    ox = torch.empty(n, dtype=torch.float64, device=dev)
    oy = torch.empty(n, dtype=torch.float64, device=dev)
    rx = torch.empty(n, dtype=torch.int32, device=dev)
    ry = torch.empty(n, dtype=torch.int32, device=dev)
    flags = torch.empty(n, dtype=torch.uint8, device=dev)
    status = torch.empty(1, dtype=torch.int32, device=dev)
    L.check(lib.fi_griddata(L.ptr(tcx), L.ptr(tcy), L.ptr(tvx), L.ptr(tvy), L.ptr(tsel),
                            int(sel.size), L.ptr(tix), ixvecs.size, L.ptr(tiy), iyvecs.size,
                            L.ptr(tpx), L.ptr(tpy), n, L.ptr(scratch), L.ptr(ox), L.ptr(oy),
                            L.ptr(rx), L.ptr(ry), L.ptr(flags), L.ptr(status),
                            L.stream_handle()), "fi_griddata")
    torch.cuda.synchronize()
    return (ox.cpu().numpy(), oy.cpu().numpy(), rx.cpu().numpy(), ry.cpu().numpy(),
            flags.cpu().numpy(), int(status.item()))


@pytest.mark.parametrize("seed,half,holes,block", [
    (1, True, 0.1, None), (2, True, 0.0, None), (3, False, 0.05, None),
    (4, True, 0.2, ((5, 11), (7, 14))), (5, False, 0.0, ((0, 4), (0, 5))),
    (6, True, 0.05, ((2, 16), (3, 18)))])
def test_griddata_matches_scipy(seed, half, holes, block):
    ixvecs, iyvecs, cx, cy, sel, vx, vy, qx, qy = _case(seed, half=half, holes=holes,
                                                        hole_block=block)
    ox, oy, rx, ry, flags, status = _gpu(ixvecs, iyvecs, cx, cy, sel, vx, vy, qx, qy)
    assert status == 0
    wx = _scipy(cx, cy, vx.astype(np.float64), qx, qy)
    wy = _scipy(cx, cy, vy.astype(np.float64), qx, qy)
    ok = flags == 0
    print(f"seed {seed}: {int((~ok).sum())} of {ok.size} points flagged")
    assert ok.mean() > 0.5
    np.testing.assert_allclose(ox[ok], wx[ok], rtol=0, atol=1e-9)
    np.testing.assert_allclose(oy[ok], wy[ok], rtol=0, atol=1e-9)
    np.testing.assert_array_equal(rx, np.rint(ox).astype(np.int32))
    np.testing.assert_array_equal(ry, np.rint(oy).astype(np.int32))
    # flagged points hold one of the valid values: inside [min, max] of the data
    assert np.all(np.isfinite(ox)) and np.all(np.isfinite(oy))
