"""Record golden vectors by running the upstream fluidimage PIV code itself.

Run from the repository root (needs the upstream sources, not needed afterwards):

    FLUIDIMAGE_REFERENCE_SRC=<upstream checkout>/src PYTHONDONTWRITEBYTECODE=1 \
        python tests/golden/make_golden.py [case ...]

Each case writes ``tests/golden/<case>.npz`` holding the input images, the
parameters (JSON) and the upstream outputs of ``WorkPIV.calcul`` (every pass:
displacements, positions, peak values, errors, interpolated fields) or of the
per-window correlation plugin ``CorrelFFTNumpy``.  Upstream runs with
``method_correl = "np.fft"`` in pure-Python transonic mode (see refharness.py).
"""

from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(HERE))
sys.path.insert(0, str(ROOT))

import refharness  # noqa: E402

refharness.install()

from fluidimage.calcul.correl import CorrelFFTNumpy  # noqa: E402
from fluidimage.calcul.errors import PIVError  # noqa: E402
from fluidimage.works.piv import WorkPIV  # noqa: E402

from fluidimage_gb300 import synthetic  # noqa: E402

PASS_KEYS = [
    "deltaxs", "deltays", "xs", "ys", "correls_max", "deltaxs_input", "deltays_input",
    "deltaxs_approx", "deltays_approx", "ixvecs_approx", "iyvecs_approx",
    "deltaxs_final", "deltays_final", "ixvecs_final", "iyvecs_final",
    "deltaxs_smooth", "deltays_smooth", "xs_smooth", "ys_smooth",
]


def _encode_dict(prefix, d, out):
    keys = np.array(sorted(d.keys()), dtype=np.int64)
    out[prefix + "_keys"] = keys
    vals = [d[int(k)] for k in keys]
    if vals and isinstance(vals[0], str):
        out[prefix + "_vals"] = np.array(vals, dtype=str) if vals else np.array([], dtype=str)
    else:
        out[prefix + "_vals"] = np.array(vals, dtype=np.float64)


def run_workpiv(name, im0, im1, settings, keep_planes=False):
    params = WorkPIV.create_default_params()
    params.piv0.method_correl = "np.fft"
    for path, value in settings.items():
        obj = params
        parts = path.split(".")
        for p in parts[:-1]:
            obj = getattr(obj, p)
        setattr(obj, parts[-1], value)
    work = WorkPIV(params)
    result = work.calcul({"arrays": (im0, im1), "names": ("im0", "im1")})
    out = {
        "im0": im0,
        "im1": im1,
        "settings": np.array(json.dumps(settings)),
        "numpy_version": np.array(np.__version__),
        "nb_passes": np.array(len(result.passes)),
    }
    for ip, r in enumerate(result.passes):
        work_piv = work.works_piv[ip]
        out[f"p{ip}_ixvecs"] = np.asarray(work_piv.ixvecs)
        out[f"p{ip}_iyvecs"] = np.asarray(work_piv.iyvecs)
        out[f"p{ip}_shape_crop"] = np.asarray(work_piv.shape_crop_im0)
        for key in PASS_KEYS:
            if hasattr(r, key):
                out[f"p{ip}_{key}"] = np.asarray(getattr(r, key))
        _encode_dict(f"p{ip}_errors", r.errors, out)
        for key in ("deltaxs_wrong", "deltays_wrong"):
            if hasattr(r, key):
                _encode_dict(f"p{ip}_{key}", getattr(r, key), out)
        sec = getattr(r, "secondary_peaks", None)
        if sec is not None and any(o is not None for o in sec):
            counts = np.array([-1 if o is None else len(o) for o in sec], dtype=np.int64)
            flat = [p for o in sec if o for p in o]
            out[f"p{ip}_secondary_counts"] = counts
            out[f"p{ip}_secondary_peaks"] = np.array(
                [[float(a), float(b), float(c)] for a, b, c in flat], dtype=np.float64
            ).reshape(-1, 3)
        rep = getattr(r, "replaced_vectors", None)
        if rep is not None:
            keys = np.array(sorted(rep), dtype=np.int64)
            out[f"p{ip}_replaced_keys"] = keys
            out[f"p{ip}_replaced_vals"] = np.array(
                [[float(v) for v in rep[int(k)]] for k in keys], dtype=np.float64
            ).reshape(-1, 3)
        if keep_planes:
            n0, n1 = work_piv.shape_crop_im0
            planes = np.full((len(r.correls), n0, n1), np.nan, dtype=np.float32)
            for i, c in enumerate(r.correls):
                if c is not None:
                    planes[i] = c
            out[f"p{ip}_planes"] = planes
    np.savez_compressed(HERE / f"{name}.npz", **out)
    print(f"wrote {name}.npz")


def case_correl_window():
    """Per-window plugin: planes, norms, peaks and subpix of CorrelFFTNumpy."""
    out = {"numpy_version": np.array(np.__version__)}
    rng_cases = [
        ("sq32", (32, 32), (3.3, 5.8), None),
        ("sq32_dmax", (32, 32), (3.3, 5.8), "50%"),
        ("sq16", (16, 16), (-2.4, 1.6), None),
        ("sq64", (64, 64), (7.7, -4.2), None),
        ("sq24", (24, 24), (2.6, -3.1), None),
        ("sq48", (48, 48), (-5.3, 4.4), None),
        ("sq48_dmax", (48, 48), (-5.3, 4.4), 9.0),
        ("sq12", (12, 12), (1.6, -2.2), None),
        ("sq8", (8, 8), (1.2, 0.7), None),
    ]
    for icase, (tag, shape, shift, dmax) in enumerate(rng_cases):
        model = synthetic.ParticleModel(density=0.06, noise=2.0, dtype="uint8")
        big0, big1 = synthetic.make_pair((shape[0] + 40, shape[1] + 40),
                                         synthetic.uniform_shift(*shift), model,
                                         seed=100 + icase, as_float32=True)
        im0 = np.ascontiguousarray(big0[20:20 + shape[0], 20:20 + shape[1]])
        im1 = np.ascontiguousarray(big1[20:20 + shape[0], 20:20 + shape[1]])
        correl = CorrelFFTNumpy(shape, shape, method_subpix="2d_gaussian2",
                                nsubpix=None, displacement_max=dmax)
        for pair_tag, (a, b) in (("same", (im0, im0)), ("shift", (im0, im1))):
            key = f"{tag}_{pair_tag}"
            plane, norm = correl(a, b)
            out[key + "_im0"] = a
            out[key + "_im1"] = b
            out[key + "_plane"] = plane.copy()
            out[key + "_norm"] = np.array(norm)
            try:
                dx, dy, cmax, _ = correl.compute_displacements_from_correl(plane, norm)
                err = ""
            except PIVError as e:
                dx, dy, cmax = e.results
                err = e.explanation
            out[key + "_peak"] = np.array([dx, dy, cmax], dtype=np.float64)
            out[key + "_err"] = np.array(err)
            out[key + "_plane_after"] = plane
            if not err:
                sdx, sdy = correl.apply_subpix(dx, dy, plane)
                out[key + "_subpix"] = np.array([sdx, sdy], dtype=np.float64)
            out[key + "_dmax"] = np.array(json.dumps(dmax))
    np.savez_compressed(HERE / "correl_window.npz", **out)
    print("wrote correl_window.npz")


def case_single_pass_c1():
    """512x512 float32-from-uint8, shift (3.3, -1.7), 32 px windows, overlap 0.5."""
    model = synthetic.ParticleModel(density=0.05, diameter=(2.0, 3.0),
                                    intensity=(128, 255), noise=2.0, dtype="uint8")
    im0, im1 = synthetic.make_pair((512, 512), synthetic.uniform_shift(3.3, -1.7),
                                   model, seed=1000, as_float32=True)
    run_workpiv("single_pass_c1", im0, im1, {
        "piv0.shape_crop_im0": 32, "piv0.grid.overlap": 0.5,
        "piv0.method_subpix": "2d_gaussian2", "multipass.number": 1,
        "fix.threshold_diff_neighbour": None, "fix.correl_min": float("-inf"),
    })


def case_multipass_small():
    """Config-2 recipe on a 384x384 uint16 Oseen pair: 64->32->16, TPS every pass."""
    model = synthetic.ParticleModel(density=0.05, diameter=(2.0, 3.0),
                                    intensity=(1000, 4000), noise=20.0, dtype="uint16")
    field = synthetic.oseen_vortex((384, 384), d_max=8.0, rc=60.0)
    im0, im1 = synthetic.make_pair((384, 384), field, model, seed=2000)
    run_workpiv("multipass_small", im0, im1, {
        "piv0.shape_crop_im0": 64, "piv0.grid.overlap": 0.5,
        "multipass.number": 3, "multipass.coeff_zoom": 2, "multipass.use_tps": True,
        "multipass.subdom_size": 200, "multipass.smoothing_coef": 0.5,
        "fix.threshold_diff_neighbour": 2,
    })


def case_dmax():
    """displacement_max='50%' mask, two passes with TPS, uint8 sinusoid field."""
    model = synthetic.ParticleModel(density=0.05, noise=2.0, dtype="uint8")
    im0, im1 = synthetic.make_pair((256, 256), synthetic.sinusoid(4.0, 256.0), model,
                                   seed=3000)
    run_workpiv("dmax_two_pass", im0, im1, {
        "piv0.shape_crop_im0": 32, "piv0.grid.overlap": 0.5,
        "piv0.displacement_max": "50%",
        "multipass.number": 2, "multipass.use_tps": True,
        "multipass.subdom_size": 100, "multipass.smoothing_coef": 2.0,
        "fix.displacement_max": 10, "fix.threshold_diff_neighbour": 3,
    }, keep_planes=True)


def case_edges():
    """Peaks beyond the window (boundary errors, second chance), a blank region
    (zero-variance windows) and image borders, 16 px windows, single pass."""
    model = synthetic.ParticleModel(density=0.04, noise=3.0, dtype="uint8")
    im0, im1 = synthetic.make_pair((160, 192), synthetic.uniform_shift(6.6, -7.3), model,
                                   seed=4000)
    im0[40:100, 60:130] = 17
    im1[40:100, 60:130] = 17
    run_workpiv("edges_single_pass", im0, im1, {
        "piv0.shape_crop_im0": 16, "piv0.grid.overlap": 0.5,
        "multipass.number": 1, "multipass.use_tps": False,
        "fix.threshold_diff_neighbour": None,
    }, keep_planes=True)


def case_griddata():
    """Two passes with the default ``use_tps='last'`` (griddata between passes)."""
    model = synthetic.ParticleModel(density=0.05, noise=2.0, dtype="uint8")
    im0, im1 = synthetic.make_pair((256, 256), synthetic.uniform_shift(-2.2, 3.6), model,
                                   seed=5000)
    run_workpiv("griddata_two_pass", im0, im1, {
        "piv0.shape_crop_im0": 32, "piv0.grid.overlap": 0.5,
        "multipass.number": 2, "multipass.use_tps": "last",
    })


def case_griddata_oseen():
    """Config-2 recipe on a 384x384 uint16 Oseen pair with use_tps=False: griddata
    between the three passes and at the end (the setting of most upstream examples)."""
    model = synthetic.ParticleModel(density=0.05, diameter=(2.0, 3.0), intensity=(1000, 4000),
                                    noise=20.0, dtype="uint16", max_value=4095)
    field = synthetic.oseen_vortex((384, 384), d_max=6.0, rc=60.0)
    im0, im1 = synthetic.make_pair((384, 384), field, model, seed=7000)
    run_workpiv("griddata_oseen_three_pass", im0, im1, {
        "piv0.shape_crop_im0": 64, "piv0.grid.overlap": 0.5,
        "multipass.number": 3, "multipass.coeff_zoom": 2, "multipass.use_tps": False,
        "fix.threshold_diff_neighbour": 2,
    })


def case_secondary_peaks():
    """nb_peaks_to_search=3 with WorkFIX secondary-peak replacement, two passes with
    TPS (32 -> 16 px windows): two particle populations moving by (3, 1) and
    (-4, 2) px share a band of the image, so windows there hold competing peaks.
    fix.displacement_max = 60 keeps upstream's unsquared check of the replacement
    (|d|^2 > displacement_max) from rejecting every peak."""
    shape, band = (192, 256), (60, 130)
    ma = synthetic.ParticleModel(density=0.05, noise=2.0, dtype="uint8")
    a0, a1 = synthetic.make_pair(shape, synthetic.uniform_shift(3.0, 1.0), ma, seed=6000)
    mb = synthetic.ParticleModel(density=0.05, noise=0.0, dtype="uint8")
    b0, b1 = synthetic.make_pair(shape, synthetic.uniform_shift(-4.0, 2.0), mb, seed=6001)
    m = np.zeros(shape)
    m[band[0]:band[1]] = 1.0
    im0 = np.clip(a0 + m * b0, 0, 255).astype(np.uint8)
    im1 = np.clip(a1 + m * b1, 0, 255).astype(np.uint8)
    run_workpiv("secondary_peaks_two_pass", im0, im1, {
        "piv0.shape_crop_im0": 32, "piv0.grid.overlap": 0.5,
        "piv0.nb_peaks_to_search": 3,
        "multipass.number": 2, "multipass.use_tps": True,
        "multipass.subdom_size": 100, "multipass.smoothing_coef": 2.0,
        "fix.threshold_diff_neighbour": 3.0, "fix.correl_min": 0.1,
        "fix.displacement_max": 60,
    }, keep_planes=True)


def case_subpix_methods():
    """The other subpixel methods in one pass each: '2d_gaussian', 'centroid' with
    nsubpix=2 (close-boundary errors near the plane edges), 'no_subpix'."""
    model = synthetic.ParticleModel(density=0.05, noise=3.0, dtype="uint8")
    field = synthetic.oseen_vortex((128, 160), d_max=6.0, rc=40.0)
    im0, im1 = synthetic.make_pair((128, 160), field, model, seed=7000)
    for tag, method, nsub in (("gaussian", "2d_gaussian", None),
                              ("centroid2", "centroid", 2),
                              ("none", "no_subpix", None)):
        run_workpiv(f"subpix_{tag}_single", im0, im1, {
            "piv0.shape_crop_im0": 16, "piv0.grid.overlap": 0.5,
            "piv0.method_subpix": method, "piv0.nsubpix": nsub,
            "multipass.number": 1, "multipass.use_tps": False,
            "fix.threshold_diff_neighbour": None,
        }, keep_planes=True)


def case_window_48_24():
    """Upstream's default first window (shape_crop_im0 = 48) in two passes, 48 -> 24
    px (the radix-3 FFT sizes), overlap 0.5, TPS between passes and at the end, on a
    320x320 uint16 12-bit Oseen pair."""
    model = synthetic.ParticleModel(density=0.05, diameter=(2.0, 3.0), intensity=(1000, 4000),
                                    noise=20.0, dtype="uint16", max_value=4095)
    field = synthetic.oseen_vortex((320, 320), d_max=6.0, rc=50.0)
    im0, im1 = synthetic.make_pair((320, 320), field, model, seed=9000)
    run_workpiv("multipass_48_24", im0, im1, {
        "piv0.shape_crop_im0": 48, "piv0.grid.overlap": 0.5,
        "multipass.number": 2, "multipass.coeff_zoom": 2, "multipass.use_tps": True,
        "multipass.subdom_size": 200, "multipass.smoothing_coef": 0.5,
        "fix.threshold_diff_neighbour": 2,
    })


def case_overlap_075():
    """Overlap 0.75: 24 px windows in one pass (step 6 px) with the final TPS, and 64
    -> 32 px windows in two passes (the overlap of the batched workloads), uint8."""
    model = synthetic.ParticleModel(density=0.05, noise=2.0, dtype="uint8")
    im0, im1 = synthetic.make_pair((160, 192), synthetic.sinusoid(3.0, 160.0), model,
                                   seed=9100)
    run_workpiv("single_pass_24_ov75", im0, im1, {
        "piv0.shape_crop_im0": 24, "piv0.grid.overlap": 0.75,
        "multipass.number": 1, "multipass.use_tps": "last",
        "multipass.subdom_size": 150, "multipass.smoothing_coef": 1.0,
        "fix.threshold_diff_neighbour": 3,
    })
    field = synthetic.oseen_vortex((256, 256), d_max=5.0, rc=50.0)
    im0, im1 = synthetic.make_pair((256, 256), field, model, seed=9200)
    run_workpiv("multipass_64_32_ov75", im0, im1, {
        "piv0.shape_crop_im0": 64, "piv0.grid.overlap": 0.75,
        "multipass.number": 2, "multipass.coeff_zoom": 2, "multipass.use_tps": True,
        "multipass.subdom_size": 200, "multipass.smoothing_coef": 0.5,
        "fix.threshold_diff_neighbour": 2,
    })


PREPROC_CASES = [
    # (name, function, image key, kwargs)
    ("minima_u8_w7", "sliding_minima", "u8", dict(window_size=7)),
    ("minima_u8_5x9_nearest", "sliding_minima", "u8", dict(window_size=(5, 9),
                                                            boundary_condition="nearest")),
    ("minima_u8_w4_constant", "sliding_minima", "u8", dict(window_size=4, weight=0.7,
                                                           boundary_condition="constant")),
    ("median_u8_w5_mirror", "sliding_median", "u8", dict(window_size=5,
                                                         boundary_condition="mirror")),
    ("median_u16_w6", "sliding_median", "u16", dict(window_size=6)),
    ("percentile_u8_w6_wrap", "sliding_percentile", "u8", dict(percentile=10.0, window_size=6,
                                                               boundary_condition="wrap")),
    ("minima_f32_w5_half", "sliding_minima", "f32", dict(window_size=5, weight=0.5)),
    ("minima_u8_int_weight", "sliding_minima", "u8", dict(window_size=3, weight=1)),
    ("temporal_minima_u8", "temporal_minima", "u8", dict()),
    ("temporal_median_u16_333", "temporal_median", "u16", dict(window_shape=(3, 3, 3))),
    ("temporal_percentile_u8_3", "temporal_percentile", "u8", dict(percentile=20.0,
                                                                   window_shape=3)),
    ("threshold_u8", "global_threshold", "u8", dict(minima=10, maxima=200)),
    ("threshold_u16_default", "global_threshold", "u16", dict(minima=50)),
    ("tanh_u8", "rescale_intensity_tanh", "u8", dict()),
    ("tanh_u16_thr", "rescale_intensity_tanh", "u16", dict(threshold=900.0)),
    ("sharpen_u8", "sharpen", "u8", dict()),
    ("sharpen_u16_s2", "sharpen", "u16", dict(sigma1=2.0, sigma2=0.8, alpha=10.0)),
    ("sharpen_f32", "sharpen", "f32", dict(sigma1=1.5, sigma2=1.0, alpha=5.0)),
]


def case_preproc():
    """The upstream preprocessing tools (works/preproc/_toolbox_py.py) on stacks of
    5 small particle images with a background gradient (uint8, uint16, float32)."""
    import importlib
    import types

    import fluidimage.works

    # the package __init__ needs image I/O helpers absent here: load the toolbox
    # module under a bare package entry instead
    pkg = "fluidimage.works.preproc"
    if pkg not in sys.modules:
        mod = types.ModuleType(pkg)
        mod.__path__ = [str(Path(fluidimage.works.__file__).parent / "preproc")]
        sys.modules[pkg] = mod
    tools = importlib.import_module(pkg + "._toolbox_py")

    rng = np.random.default_rng(8000)
    model8 = synthetic.ParticleModel(density=0.05, noise=3.0, dtype="uint8")
    shape = (48, 64)
    frames = []
    for k in range(5):
        a, _ = synthetic.make_pair(shape, synthetic.uniform_shift(1.0, 0.5), model8,
                                   seed=8000 + k)
        frames.append(a)
    bg = (np.arange(shape[1])[None, :] * 0.5 + np.arange(shape[0])[:, None] * 0.3)
    u8 = np.clip(np.array(frames, dtype=np.float64) * 0.6 + bg[None] + 10, 0, 255).astype(np.uint8)
    u16 = (u8.astype(np.uint16) * 16 + rng.integers(0, 16, u8.shape)).astype(np.uint16)
    f32 = (u8.astype(np.float32) / 7.0).astype(np.float32)
    images = {"u8": u8, "u16": u16, "f32": f32}
    out = {"img_" + k: v for k, v in images.items()}
    out["numpy_version"] = np.array(np.__version__)
    for name, fn, key, kwargs in PREPROC_CASES:
        res = getattr(tools, fn)(img=images[key].copy(), **kwargs)
        out["out_" + name] = np.asarray(res)
        out["args_" + name] = np.array(json.dumps({"function": fn, "image": key,
                                                   "kwargs": kwargs}))
    np.savez_compressed(HERE / "preproc.npz", **out)
    print("wrote preproc.npz")


def case_minimal_piv_oseen():
    """The configuration of upstream's own test_minimal_piv (works/piv/test_piv.py:16-34)
    on its Oseen sample pair (image_samples/Oseen/Images/Oseen_center_01/02.tif, 8-bit
    TIFF, read with this package's image reader since PIL is absent here): 32 -> 16 px
    windows at overlap -3 (windows 96 px apart in the first pass), two peaks searched,
    TPS between the passes on a grid of 3 x 2 vectors, fix.displacement_max 3."""
    from fluidimage_gb300.images import imread

    import os

    samples = Path(os.environ[refharness.SRC_ENV]).parent / "image_samples" / "Oseen" / "Images"
    im0 = imread(samples / "Oseen_center_01.tif")
    im1 = imread(samples / "Oseen_center_02.tif")
    run_workpiv("minimal_piv_oseen", im0, im1, {
        "piv0.shape_crop_im0": 32, "piv0.grid.overlap": -3,
        "piv0.nb_peaks_to_search": 2,
        "multipass.number": 2, "multipass.use_tps": True,
        "fix.displacement_max": 3, "fix.threshold_diff_neighbour": 2,
    })


def case_small_windows():
    """Windows of 12 and 8 px: upstream's default parameters with three passes (48 ->
    24 -> 12 px, use_tps 'last': griddata between the passes, TPS at the end) on a
    288x320 uint16 12-bit Oseen pair, and 16 -> 8 px with TPS between the passes on a
    160x192 uint8 pair moving by under 2 px."""
    model = synthetic.ParticleModel(density=0.05, diameter=(2.0, 3.0), intensity=(1000, 4000),
                                    noise=20.0, dtype="uint16", max_value=4095)
    field = synthetic.oseen_vortex((288, 320), d_max=5.0, rc=50.0)
    im0, im1 = synthetic.make_pair((288, 320), field, model, seed=9100)
    run_workpiv("multipass_48_24_12", im0, im1, {"multipass.number": 3})
    model8 = synthetic.ParticleModel(density=0.06, noise=2.0, dtype="uint8")
    im0, im1 = synthetic.make_pair((160, 192), synthetic.sinusoid(1.6, 96.0), model8, seed=9101)
    run_workpiv("multipass_16_8", im0, im1, {
        "piv0.shape_crop_im0": 16, "piv0.grid.overlap": 0.5,
        "multipass.number": 2, "multipass.use_tps": True,
        "multipass.subdom_size": 100, "multipass.smoothing_coef": 1.0,
        "fix.threshold_diff_neighbour": 2,
    })


CASES = {
    "correl_window": case_correl_window,
    "single_pass_c1": case_single_pass_c1,
    "multipass_small": case_multipass_small,
    "dmax_two_pass": case_dmax,
    "edges_single_pass": case_edges,
    "griddata_two_pass": case_griddata,
    "griddata_oseen_three_pass": case_griddata_oseen,
    "secondary_peaks_two_pass": case_secondary_peaks,
    "subpix_methods": case_subpix_methods,
    "multipass_48_24": case_window_48_24,
    "overlap_075": case_overlap_075,
    "preproc": case_preproc,
    "minimal_piv_oseen": case_minimal_piv_oseen,
    "small_windows": case_small_windows,
}

if __name__ == "__main__":
    names = sys.argv[1:] or list(CASES)
    for name in names:
        CASES[name]()
