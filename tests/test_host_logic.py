"""Host-side logic (parameters only, no GPU): grids, masks, pass shapes, error
strings, parameter tree, synthetic images."""

import numpy as np
import pytest

import goldens
from fluidimage_gb300 import WorkPIV, engine, synthetic
from oracle import piv as O


@pytest.mark.parametrize("imshape", [(512, 512), (2048, 2048), (768, 1024), (2160, 4096),
                                     (160, 192), (101, 77)])
@pytest.mark.parametrize("n,overlap", [(16, 0.5), (24, 0.75), (32, 0.5), (48, 0.5),
                                       (64, 0.75), (32, -3)])
def test_grid_matches_oracle(imshape, n, overlap):
    if n > min(imshape):
        pytest.skip("window larger than image")
    gx, gy = engine.make_grid(imshape, (n, n), overlap)
    ox, oy = O.make_grid(imshape, (n, n), overlap)
    np.testing.assert_array_equal(gx, ox)
    np.testing.assert_array_equal(gy, oy)


@pytest.mark.parametrize("imshape,n,overlap,count", [
    ((512, 512), 32, 0.5, 961),
    ((2048, 2048), 64, 0.5, 3969),
    ((2048, 2048), 32, 0.5, 16129),
    ((2048, 2048), 16, 0.5, 65025),
    ((4096, 4096), 32, 0.75, 259081),
    ((2160, 4096), 16, 0.75, 548277),
])
def test_window_counts_of_the_benchmark_configs(imshape, n, overlap, count):
    gx, gy = engine.make_grid(imshape, (n, n), overlap)
    assert gx.size * gy.size == count


@pytest.mark.parametrize("n", [16, 24, 32, 48, 64])
@pytest.mark.parametrize("dmax", [None, "50%", 5.0, 3, 0.5])
def test_displacement_mask_matches_oracle(n, dmax):
    d = engine.parse_displacement_max(dmax, (n, n))
    mask, box = engine.displacement_mask(n, d)
    omask, b0, b1 = O.displacement_mask((n, n), d)
    if mask is None:
        assert omask is None
    else:
        np.testing.assert_array_equal(mask, omask)
    assert box == (b0[0], b0[1], b1[0], b1[1])


def test_pass_shapes():
    assert engine.pass_shapes(64, 3, 2) == [(64, 64), (32, 32), (16, 16)]
    assert engine.pass_shapes(48, 2, [2]) == [(48, 48), (24, 24)]
    assert engine.pass_shapes((64, 32), 2, 2) == O.pass_shapes((64, 32), 2, 2)
    with pytest.raises(ValueError):
        engine.pass_shapes(64, 3, [2])


def test_default_params_match_upstream():
    params = WorkPIV.create_default_params()
    for path, value in goldens.DEFAULTS.items():
        obj = params
        for part in path.split("."):
            obj = getattr(obj, part)
        if path == "piv0.method_correl":
            assert obj == "gb300"
        else:
            assert obj == value, path
    with pytest.raises(AttributeError):
        params.piv0.shape_crop = 32


def test_unknown_correlation_method_rejected():
    params = WorkPIV.create_default_params()
    params.piv0.method_correl = "scipy.signal"
    with pytest.raises(ValueError, match="method_correl"):
        WorkPIV(params)


def test_error_dict_strings():
    err = np.array([0, 1, 2, 3, 4, 0, 0, 1], dtype=np.uint8)
    flags = np.array([0, 0, 0, 0, 0, 1, 4, 1], dtype=np.uint8)
    diff2 = np.array([0, 0, 0, 0, 0, 0, 6.25, 0], dtype=np.float32)
    d = engine.error_dict(err, flags, diff2, 2)
    assert d == {
        1: "Correlation peak touching boundary.",
        2: "Correlation peak touching nan.",
        3: "wrong subpix",
        4: "Bad im_crop shape.",
        5: "correl < correl_min",
        6: "diff neighbour too large (diff = 2.50)",
        7: "Correlation peak touching boundary. + correl < correl_min",
    }


def test_error_strings_cover_golden_vocabulary():
    """Every error string recorded from upstream can be produced by error_dict."""
    produced = set(engine.ERROR_STRINGS.values()) | {
        "correl < correl_min", "delta2 < displacement_max2", "diff neighbour too large"}
    for name in goldens.fixture_names():
        z = goldens.load(name)
        for ip in range(int(z["nb_passes"])):
            for s in goldens.errors(z, ip).values():
                for part in s.split(" (diff")[0].split(" + "):
                    assert part in produced, part


def test_synthetic_pairs_are_deterministic():
    model = synthetic.ParticleModel(density=0.05, noise=2.0, dtype="uint8")
    a = synthetic.make_pair((64, 80), synthetic.uniform_shift(1.5, -2.0), model, seed=3)
    b = synthetic.make_pair((64, 80), synthetic.uniform_shift(1.5, -2.0), model, seed=3)
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1], b[1])
    assert a[0].dtype == np.uint8 and a[0].shape == (64, 80)
    f = synthetic.oseen_vortex((2048, 2048), d_max=8.0, rc=200.0)
    r = np.linspace(1, 1500, 20000)
    dx, dy = f(1023.5 + r, np.full_like(r, 1023.5))
    assert abs(np.hypot(dx, dy).max() - 8.0) < 1e-3


@pytest.mark.parametrize("sigma", [0.8, 1.0, 1.5, 2.0, 3.0])
def test_gaussian_weights_match_scipy(sigma):
    """The host-side kernel of ``preproc.gaussian_filter`` is scipy.ndimage's
    (``_gaussian_kernel1d`` reversed, radius ``int(4 sigma + 0.5)``), bit for bit."""
    from scipy.ndimage import _filters

    from fluidimage_gb300 import preproc as P

    w, radius = P._gauss_weights(sigma)
    assert radius == int(4.0 * sigma + 0.5)
    want = _filters._gaussian_kernel1d(sigma, 0, radius)[::-1]
    np.testing.assert_array_equal(w, want)
