"""Full-size workloads on the GPU, checked stage by stage against the CPU oracle.

At 2048x2048 the whole oracle pipeline takes minutes, so each stage is checked
conditionally: the oracle recomputes a stage from the GPU's own inputs to that
stage (the same fixed field, the same integer window shifts).  Tolerances:

* correlation passes: integer peaks exact except near-ties (counted), vectors
  within 5e-3 px, median difference below 1e-4 px;
* TPS (float64 both sides; the GPU solves the subdomain systems in mixed
  precision to FP64 accuracy): interpolated field within 1e-8 px of the oracle's
  FP64 LU solution;
* ground truth: RMS error of the final field against the imposed Oseen vortex
  below 0.3 px (interior vectors; 16 px windows with TPS smoothing on a vortex
  whose displacement varies by ~0.6 px across a window).
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def config2_run():
    import torch

    from fluidimage_gb300 import WorkPIV, workloads

    (im0, im1), field = workloads.config2_images(pair=0)
    params = workloads.config2_params(WorkPIV.create_default_params())
    work = WorkPIV(params)
    t0 = torch.from_numpy(im0.view(np.int16)).cuda()
    t1 = torch.from_numpy(im1.view(np.int16)).cuda()
    outs = work.calcul_device(t0, t1)
    res = work.results_to_host(outs)
    return im0, im1, field, params, res


def test_config2_shapes(config2_run):
    im0, im1, field, params, res = config2_run
    assert [r.deltaxs.size for r in res.passes] == [3969, 16129, 65025]
    assert res.passes[-1].deltaxs_final.shape == (65025,)


def test_config2_pass0_matches_oracle(config2_run):
    from oracle import piv as O

    im0, im1, field, params, res = config2_run
    r = res.passes[0]
    o = O.piv_pass(im0, im1, (64, 64), 0.5, apply_subpix=False)
    _check_pass(r, o, params)


@pytest.mark.parametrize("ip,n", [(1, 32), (2, 16)])
def test_config2_shifted_passes_match_oracle(config2_run, ip, n):
    from oracle import piv as O

    im0, im1, field, params, res = config2_run
    r = res.passes[ip]
    o = O.piv_pass(im0, im1, (n, n), 0.5, dxin=r.deltaxs_input, dyin=r.deltays_input,
                   apply_subpix=(ip == 2))
    _check_pass(r, o, params)


def _check_pass(r, o, params):
    from oracle import piv as O

    raw_ok = o.err == 0
    # the GPU result r is after WorkFIX; compare where both kept the vector
    keep = ~np.isnan(r.deltaxs)
    both = keep & raw_ok
    d = np.abs(np.concatenate([r.deltaxs[both] - o.deltaxs[both],
                               r.deltays[both] - o.deltays[both]]))
    ties = getattr(r, "near_ties", 0)
    assert np.count_nonzero(d > 5e-3) <= ties
    assert np.median(d) < 1e-4
    # WorkFIX on the oracle's raw pass reproduces the GPU's kept vectors
    O.fix(o, params.fix.correl_min, params.fix.threshold_diff_neighbour,
          params.fix.displacement_max)
    mism = np.count_nonzero(np.isnan(o.deltaxs) != np.isnan(r.deltaxs))
    assert mism <= 2 * ties + 2, mism
    np.testing.assert_array_equal(np.asarray(r.xs, float), np.asarray(o.xs, float))


@pytest.mark.parametrize("ip", [0, 1])
def test_config2_tps_between_passes_matches_oracle(config2_run, ip):
    """TPS of pass ip's fixed field onto the next grid, recomputed by the oracle."""
    from oracle import piv as O

    im0, im1, field, params, res = config2_run
    r = res.passes[ip]
    nxt = res.passes[ip + 1]
    ns = type("R", (), {})()
    ns.deltaxs, ns.deltays = r.deltaxs.copy(), r.deltays.copy()
    ns.xs, ns.ys = np.asarray(r.xs), np.asarray(r.ys)
    gx = np.unique(r.ixvecs_approx)
    gy = np.unique(r.iyvecs_approx)
    O.apply_interp(ns, (gx, gy), params.multipass)
    err = max(np.abs(r.deltaxs_approx - ns.deltaxs_approx).max(),
              np.abs(r.deltays_approx - ns.deltays_approx).max())
    print(f"TPS pass {ip} -> next grid: max |GPU - FP64 LU| = {err:.3e} px")
    np.testing.assert_allclose(r.deltaxs_approx, ns.deltaxs_approx, rtol=0, atol=1e-8)
    np.testing.assert_allclose(r.deltays_approx, ns.deltays_approx, rtol=0, atol=1e-8)
    np.testing.assert_array_equal(nxt.deltaxs_input, np.round(ns.deltaxs_approx).astype("int32"))


def test_config2_final_field_accuracy(config2_run):
    im0, im1, field, params, res = config2_run
    r = res.passes[-1]
    tx, ty = field(r.ixvecs_final.astype(float), r.iyvecs_final.astype(float))
    inner = ((r.ixvecs_final > 64) & (r.ixvecs_final < 2048 - 64)
             & (r.iyvecs_final > 64) & (r.iyvecs_final < 2048 - 64))
    err = np.hypot(r.deltaxs_final - tx, r.deltays_final - ty)[inner]
    rms = float(np.sqrt(np.mean(err**2)))
    print(f"config2 final field RMS error vs ground truth: {rms:.4f} px")
    assert rms < 0.3
    valid = ~np.isnan(r.deltaxs)
    assert valid.mean() > 0.95
