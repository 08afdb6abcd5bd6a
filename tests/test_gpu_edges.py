"""Edge cases of a pass against the oracle: constant images (every window flat:
zero planes, norm 0, correls_max 0, the peak at the last maximum of an all-zero
plane), images with constant regions (flat and textured windows side by side), a
single window per image, and images of one window plus a ragged border.  The GPU
pass (after WorkFIX) equals the oracle's pass followed by the oracle's WorkFIX: same
errors, same NaN pattern, displacements within 5e-3 px, correls_max within 2e-5
relative."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL_PX = 5e-3


def _pass(im0, im1, n, overlap, dtype):
    import torch

    from fluidimage_gb300 import WorkPIV

    params = WorkPIV.create_default_params()
    params.piv0.shape_crop_im0 = n
    params.piv0.grid.overlap = overlap
    params.multipass.number = 1
    params.fix.threshold_diff_neighbour = None
    params.fix.correl_min = float("-inf")
    res = WorkPIV(params, interp_last=False).calcul(
        {"arrays": (im0.astype(dtype), im1.astype(dtype)), "names": ("a", "b")})
    torch.cuda.synchronize()
    return res.passes[0]


def _compare(got, want):
    from oracle import piv as O

    O.fix(want, correl_min=float("-inf"), threshold_diff_neighbour=None)
    a = np.asarray(got.deltaxs, np.float64)
    b = np.asarray(want.deltaxs, np.float64)
    assert a.shape == b.shape
    assert np.array_equal(np.isnan(a), np.isnan(b))
    ok = ~np.isnan(b)
    if ok.any():
        assert np.abs(a[ok] - b[ok]).max() <= TOL_PX
        assert np.abs(np.asarray(got.deltays)[ok] - want.deltays[ok]).max() <= TOL_PX
        np.testing.assert_allclose(np.asarray(got.correls_max)[ok], want.correls_max[ok],
                                   rtol=2e-5, atol=1e-7)
    assert dict(got.errors) == want.errors


def _images(kind, shape, seed=5):
    from fluidimage_gb300 import synthetic

    model = synthetic.ParticleModel(density=0.05, noise=2.0, dtype="uint8")
    im0, im1 = synthetic.make_pair(shape, synthetic.uniform_shift(2.3, -1.4), model, seed=seed)
    im0, im1 = im0.astype(np.float64), im1.astype(np.float64)
    if kind == "constant":
        im0[:] = 37.0
        im1[:] = 37.0
    elif kind == "constant_im1":
        im1[:] = 12.0
    elif kind == "flat_regions":
        im0[:, : shape[1] // 3] = 50.0
        im1[:, : shape[1] // 3] = 50.0
        im0[shape[0] // 2:, shape[1] // 2:] = 0.0
    return im0, im1


@pytest.mark.parametrize("dtype", ["uint8", "uint16", "float32"])
@pytest.mark.parametrize("kind", ["constant", "constant_im1", "flat_regions"])
def test_flat_windows_match_oracle(kind, dtype):
    from oracle import piv as O

    im0, im1 = _images(kind, (128, 160))
    n = 32
    got = _pass(im0, im1, n, 0.5, dtype)
    want = O.piv_pass(im0.astype(dtype), im1.astype(dtype), (n, n), 0.5)
    _compare(got, want)


@pytest.mark.parametrize("shape, n", [((35, 41), 32), ((33, 33), 32), ((40, 33), 32),
                                      ((64, 70), 48), ((30, 50), 24), ((17, 18), 16)])
def test_small_grids_and_ragged_borders_match_oracle(shape, n):
    """Grids of 1 x 1, 1 x 2 and 2 x 1 vectors and ragged borders, WorkFIX without the
    neighbour test (upstream's neighbour mean needs 2 x 2, see below)."""
    from oracle import piv as O

    im0, im1 = _images("particles", shape, seed=9)
    got = _pass(im0, im1, n, 0.5, "uint16")
    want = O.piv_pass(im0.astype("uint16"), im1.astype("uint16"), (n, n), 0.5)
    assert np.asarray(got.deltaxs).size >= 1
    _compare(got, want)


@pytest.mark.parametrize("shape, n", [((32, 32), 32), ((16, 16), 16), ((24, 30), 24)])
def test_empty_grid_raises_index_error_like_upstream(shape, n):
    """An image the size of the window has an empty grid: upstream's
    _prepare_with_image fails with an IndexError (singlepass.py:128-133); so does the
    oracle, and the work raises an IndexError too (GridError)."""
    from fluidimage_gb300 import WorkPIV
    from oracle import piv as O

    im0, im1 = _images("particles", shape, seed=9)
    with pytest.raises(IndexError):
        O.make_grid(shape, (n, n), 0.5)
    params = WorkPIV.create_default_params()
    params.piv0.shape_crop_im0 = n
    params.multipass.number = 1
    with pytest.raises(IndexError):
        WorkPIV(params).calcul({"arrays": (im0.astype("uint16"), im1.astype("uint16")),
                                "names": ("a", "b")})


def test_neighbour_test_on_a_one_row_grid_raises_index_error_like_upstream():
    """WorkFIX's neighbour mean on a grid of one row fails with an IndexError upstream
    (mean_neighbors.py:5-125); the oracle and the work do the same."""
    from fluidimage_gb300 import WorkPIV
    from oracle import piv as O

    im0, im1 = _images("particles", (35, 41), seed=9)
    want = O.piv_pass(im0.astype("uint16"), im1.astype("uint16"), (32, 32), 0.5)
    with pytest.raises(IndexError):
        O.fix(want, correl_min=0.2, threshold_diff_neighbour=2.0)
    params = WorkPIV.create_default_params()
    params.piv0.shape_crop_im0 = 32
    params.multipass.number = 1
    params.fix.threshold_diff_neighbour = 2.0
    with pytest.raises(IndexError):
        WorkPIV(params, interp_last=False).calcul(
            {"arrays": (im0.astype("uint16"), im1.astype("uint16")), "names": ("a", "b")})
