"""Tensor-core DFT correlation pass (fi_piv_pass_tc) on the GPU.

Each precision form against the FP64 oracle (complex128 FFTs, float64 planes and
fit) and against upstream's float32 results (golden fixtures):

* planes: max |c - c64| / max |c64| per window within the form's bound
  (bf16 x1 1e-2, bf16 3-term 2e-5, fp16 3-term 2e-6; the CPU emulation of the
  kernel predicts ~2e-3, ~3e-6, ~1.2e-7);
* integer peaks: equal to upstream's outside the form's near-ties (flagged by the
  kernel: the top two plane values within 3e-2 / 1e-4 / 1e-5 relative), counted;
* displacements: within 0.005 px of upstream and of the FP64 oracle for the two
  3-term forms outside near-ties; the single-term form's error is printed.
"""

import numpy as np
import pytest

import goldens

pytestmark = pytest.mark.gpu

FORMS = ["bf16x1", "bf16x3", "fp16x3"]
PLANE_BOUND = {"bf16x1": 1e-2, "bf16x3": 2e-5, "fp16x3": 2e-6}
TOL_PX = 5e-3


def _work(params, form, **kw):
    from fluidimage_gb300 import WorkPIV

    params.piv0.method_correl = f"gb300_tc_{form}"
    return WorkPIV(params, **kw)


def _calcul(work, im0, im1):
    import torch

    res = work.calcul({"arrays": (im0, im1), "names": ("im0", "im1")})
    torch.cuda.synchronize()
    return res


@pytest.mark.parametrize("form", FORMS)
def test_tc_planes_vs_fp64(form):
    from fluidimage_gb300 import WorkPIV, workloads
    from oracle import accuracy as A

    (im0, im1), _ = workloads.config1_images()
    params = workloads.config1_params(WorkPIV.create_default_params())
    ref = A.fp64_multipass(im0, im1, params, keep_planes=True)
    res = _calcul(_work(params, form, keep_correls=True), im0, im1)
    planes = A.plane_relative_error(res.passes[0].correls, ref[0].planes)
    acc = A.summary(res.passes, ref)
    print(form, "planes vs FP64:", planes, "displacements vs FP64:", acc)
    assert planes["windows"] > 900
    assert planes["max"] <= PLANE_BOUND[form]
    if form != "bf16x1":
        assert acc["max_px"] <= TOL_PX


@pytest.mark.parametrize("form", FORMS)
def test_tc_single_pass_matches_reference(form):
    """The config-1 golden (512^2, 32 px, overlap 0.5): upstream's integer peaks,
    errors and displacements outside near-ties."""
    z = goldens.load("single_pass_c1")
    from fluidimage_gb300 import WorkPIV

    params = WorkPIV.create_default_params()
    for path, value in goldens.settings(z).items():
        obj = params
        parts = path.split(".")
        for part in parts[:-1]:
            obj = getattr(obj, part)
        setattr(obj, parts[-1], value)
    res = _calcul(_work(params, form), z["im0"], z["im1"])
    r = res.passes[0]
    tie = r.near_tie_flags != 0
    gdx, gdy = z["p0_deltaxs"], z["p0_deltays"]
    nt = ~tie
    np.testing.assert_array_equal(np.isnan(r.deltaxs)[nt], np.isnan(gdx)[nt])
    ok = ~np.isnan(gdx) & nt
    d = np.abs(np.concatenate([r.deltaxs[ok] - gdx[ok], r.deltays[ok] - gdy[ok]]))
    # integer peak = round of the displacement's integer part: compare the peaks
    # through the subpixel offsets being below one pixel
    print(form, {"max_px": float(d.max()), "median_px": float(np.median(d)),
                 "near_ties": int(tie.sum())})
    assert tie.sum() <= 0.05 * tie.size
    assert (d < 1.0).all(), "an integer peak differs from upstream's outside near-ties"
    if form != "bf16x1":
        assert d.max() <= TOL_PX
    np.testing.assert_allclose(r.correls_max[ok], z["p0_correls_max"][ok],
                               rtol=PLANE_BOUND[form] * 10 + 1e-5, atol=1e-5)


@pytest.mark.parametrize("form", ["bf16x3", "fp16x3"])
def test_tc_in_multipass_matches_reference(form):
    """Config-2 recipe on a 384^2 golden (64 -> 32 -> 16 px): the 32 px pass, with
    shifted windows, runs on the tensor cores; the other passes on the FP32 FFT."""
    import test_gpu_parity as P

    z = goldens.load("multipass_small")
    params = P._params(z)
    res = _calcul(_work(params, form), z["im0"], z["im1"])
    report = []
    prev = None
    for ip, r in enumerate(res.passes):
        if ip == 1:
            tie = r.near_tie_flags != 0
            gdx = z["p1_deltaxs"]
            ok = ~np.isnan(gdx) & ~tie & ~np.isnan(r.deltaxs)
            d = np.abs(r.deltaxs[ok] - gdx[ok])
            report.append({"pass": 1, "max_px": float(d.max()), "near_ties": int(tie.sum())})
            assert d.max() <= TOL_PX
        else:
            P._compare_pass(z, ip, r, report, prev)
        prev = r
    print(form, report)


@pytest.mark.parametrize("form", ["bf16x3", "fp16x3"])
def test_tc_sinusoid_overlap_075_vs_fp64(form):
    """A crop of the precision-sweep workload (uint16 12-bit, density 0.06, diameter
    2.5 px, sinusoidal displacement of 5 px, 32 px windows at overlap 0.75) against
    the FP64 oracle and the FP32 FFT pass."""
    from fluidimage_gb300 import WorkPIV, workloads
    from oracle import accuracy as A

    (im0, im1), _ = workloads.config4_images(shape=(512, 512))
    params = workloads.config4_params(WorkPIV.create_default_params())
    ref = A.fp64_multipass(im0, im1, params)
    res = _calcul(_work(params, form), im0, im1)
    params.piv0.method_correl = "gb300"
    res32 = _calcul(WorkPIV(params), im0, im1)
    acc = A.summary(res.passes, ref)
    acc32 = A.summary(res32.passes, ref)
    print(form, "vs FP64:", acc, "FP32 FFT vs FP64:", acc32)
    assert acc["compared"] > 0.9 * res.passes[0].deltaxs.size
    assert acc["max_px"] <= TOL_PX
