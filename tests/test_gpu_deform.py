"""Image deformation and the hand-written adjoint of deform-and-correlate on the GPU.

* warp: within the range of the float64 numpy oracle over sample positions moved
  by two float32 ulps of the image size (the rounding of the float32 positions,
  which steep particle edges turn into up to ~0.1 counts);
* soft-argmax read-out r of every 32 x 32 window: within 1e-4 px of the float64
  torch reference on the same deformed image;
* gradients with respect to the nodes and to im1, central scheme (im0 by -d/2, im1
  by +d/2) and im1-only scheme: the pure-torch autograd reference (float64) within
  1e-3 of the gradient's norm; against FP64 central finite differences with
  h = 1e-3 px within 5 % (the piecewise-linear sampling makes differences over h
  include pixels that cross an integer position) and with h = 1e-5 px within 1e-3;
* refinement: 20 Adam steps lower the RMS error against the imposed field;
* deformation-mode multipass: a deformed pass equals the oracle's pass on the
  oracle's deformation of both images by the same field (im0 by -d/2, im1 by
  +d/2), and lowers the RMS error against the imposed field below the
  window-shift mode's.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _case(H=256, W=320, B=2, seed=0):
    import torch

    from fluidimage_gb300 import deform, synthetic

    model = synthetic.ParticleModel(density=0.06, diameter=(2.0, 3.0), intensity=(1000, 4000),
                                    noise=20.0, dtype="uint16", max_value=4095)
    ims0, ims1, fields = [], [], []
    for b in range(B):
        field = synthetic.oseen_vortex((H, W), d_max=5.0, rc=60.0)
        im0, im1 = synthetic.make_pair((H, W), field, model, seed=seed + b)
        ims0.append(im0.astype(np.float32))
        ims1.append(im1.astype(np.float32))
        fields.append(field)
    xn, yn = deform.node_grid(H, W)
    truth = []
    for field in fields:
        gx, gy = np.meshgrid(xn.astype(np.float64), yn.astype(np.float64))
        u, v = field(gx, gy)
        truth.append(np.stack([u, v]))
    truth = np.array(truth, dtype=np.float32)
    rng = np.random.default_rng(seed)
    init = (truth + 0.3 * rng.standard_normal(truth.shape)).astype(np.float32)
    dev = torch.device("cuda")
    t = lambda a: torch.as_tensor(np.ascontiguousarray(a), device=dev)  # noqa: E731
    return (t(np.array(ims0)), t(np.array(ims1)), t(init), t(truth), t(xn), t(yn))


def test_warp_matches_oracle():
    import torch

    from fluidimage_gb300 import deform
    from oracle import deform as OD

    im0, im1, nodes, truth, xn, yn = _case(B=1)
    f, gx, gy, im = (nodes[0].cpu().numpy().astype(np.float64), xn.cpu().numpy(),
                     yn.cpu().numpy(), im1[0].cpu().numpy())
    eps = 2 * float(np.spacing(np.float32(max(im.shape))))
    for scale in (1.0, 0.5, -0.5):
        got = deform.warp(nodes, xn, yn, im1, scale)
        torch.cuda.synchronize()
        outs = [OD.warp(f + np.array([du, dv])[:, None, None], gx, gy, im, scale)
                for du in (-eps, 0.0, eps) for dv in (-eps, 0.0, eps)]
        lo, hi = np.min(outs, axis=0) - 1e-3, np.max(outs, axis=0) + 1e-3
        as_u16 = deform.warp(nodes, xn, yn, im1.to(torch.int32).to(torch.int16), scale)
        for g in (got[0], as_u16[0]):
            g = g.cpu().numpy()  # float32 image, then uint16 (int16 storage): same samples
            bad = (g < lo) | (g > hi)
            assert not bad.any(), (scale, int(bad.sum()), float(np.abs(g - outs[4]).max()))


def test_readout_matches_torch_reference():
    import torch

    import deform_reference as R
    from fluidimage_gb300 import deform

    im0, im1, nodes, truth, xn, yn = _case()
    im1w = deform.warp(nodes, xn, yn, im1)
    r, cz, cpk = deform.windows(im0, im1w, 0.1)
    want = R.windows_r(im0.double(), im1w.double(), 0.1)
    err = (r.double() - want).abs().max().item()
    print("soft-argmax r vs float64 torch:", err, "px")
    assert err <= 1e-4
    assert (cpk >= cz).all()


def _grads_gpu(nodes, im0, im1, xn, yn, symmetric):
    from fluidimage_gb300 import deform

    p = nodes.clone().requires_grad_(True)
    q = im1.clone().requires_grad_(True)
    r = deform.DeformCorrelate.apply(p, im0, q, xn, yn, 0.1, symmetric)
    loss = (r * r).sum(dim=-1).mean()
    loss.backward()
    return loss.item(), p.grad, q.grad


@pytest.mark.parametrize("symmetric", [True, False], ids=["central", "im1_only"])
def test_adjoint_matches_autograd_and_finite_differences(symmetric):
    import torch

    import deform_reference as R

    im0, im1, nodes, truth, xn, yn = _case()
    loss, g_nodes, g_im1 = _grads_gpu(nodes, im0, im1, xn, yn, symmetric)
    # pure-torch autograd reference, float64
    p = nodes.double().clone().requires_grad_(True)
    q = im1.double().clone().requires_grad_(True)
    ref_loss = R.loss(p, im0.double(), q, xn, yn, symmetric=symmetric)
    ref_loss.backward()
    rel_n = ((g_nodes.double() - p.grad).norm() / p.grad.norm()).item()
    rel_i = ((g_im1.double() - q.grad).norm() / q.grad.norm()).item()
    print("loss", loss, ref_loss.item(), "relative gradient error: nodes", rel_n, "im1", rel_i)
    assert abs(loss - ref_loss.item()) <= 1e-4 * abs(ref_loss.item()) + 1e-7
    assert rel_n <= 1e-3
    assert rel_i <= 1e-3
    # FP64 central differences of the reference loss
    base = nodes.double()
    worst = {}
    for h, rel in ((1e-3, 5e-2), (1e-5, 1e-3)):
        for (b, c, i, j) in [(0, 0, 2, 3), (1, 1, 4, 5), (0, 1, 6, 8), (1, 0, 1, 7)]:
            a = base.clone()
            m = base.clone()
            a[b, c, i, j] += h
            m[b, c, i, j] -= h
            fd = (R.loss(a, im0.double(), im1.double(), xn, yn, symmetric=symmetric)
                  - R.loss(m, im0.double(), im1.double(), xn, yn, symmetric=symmetric)
                  ).item() / (2 * h)
            g = g_nodes[b, c, i, j].item()
            scale = max(abs(fd), 1e-2 * g_nodes.abs().max().item())
            worst[h] = max(worst.get(h, 0.0), abs(g - fd) / scale)
            assert abs(g - fd) <= rel * scale, (h, b, c, i, j, g, fd)
    print("worst relative difference to central differences:", worst)
    del torch


def test_refinement_lowers_error():
    import torch

    from fluidimage_gb300 import deform

    im0, im1, nodes, truth, xn, yn = _case()
    inner = (slice(None), slice(None), slice(1, -1), slice(1, -1))
    before = ((nodes - truth)[inner] ** 2).mean().sqrt().item()
    out, losses = deform.refine(nodes, im0, im1, xn, yn, steps=20, lr=0.05, history=True)
    torch.cuda.synchronize()
    after = ((out - truth)[inner] ** 2).mean().sqrt().item()
    print("RMS error vs imposed field: before", before, "after", after, "losses", losses[:3],
          losses[-3:])
    assert losses[-1] < losses[0]
    assert after < before


def test_deformed_multipass_matches_oracle_and_truth():
    import torch

    from fluidimage_gb300 import WorkPIV, synthetic, workloads
    from oracle import deform as OD
    from oracle import piv as O

    model = synthetic.ParticleModel(density=0.05, diameter=(2.0, 3.0), intensity=(1000, 4000),
                                    noise=20.0, dtype="uint16", max_value=4095)
    field = synthetic.oseen_vortex((512, 512), d_max=8.0, rc=60.0)
    im0, im1 = synthetic.make_pair((512, 512), field, model, seed=77)
    params = workloads.config2_params(WorkPIV.create_default_params())
    res_def = WorkPIV(params, deform=True).calcul({"arrays": (im0, im1), "names": ("a", "b")})
    res_shift = WorkPIV(params).calcul({"arrays": (im0, im1), "names": ("a", "b")})
    torch.cuda.synchronize()
    # the last pass against the oracle: the same field, the oracle's float64 warp
    prev, last = res_def.passes[-2], res_def.passes[-1]
    nx, ny = np.unique(prev.ixvecs_approx).size, np.unique(prev.iyvecs_approx).size
    nodes = np.stack([prev.deltaxs_approx.reshape(ny, nx), prev.deltays_approx.reshape(ny, nx)])
    xn = np.unique(prev.ixvecs_approx).astype(np.float32)
    yn = np.unique(prev.iyvecs_approx).astype(np.float32)
    nodes32 = nodes.astype(np.float32)
    w0 = OD.warp(nodes32, xn, yn, im0.astype(np.float64), -0.5).astype(np.float32)
    w1 = OD.warp(nodes32, xn, yn, im1.astype(np.float64), 0.5).astype(np.float32)
    o = O.piv_pass(w0, w1, (16, 16), 0.5, apply_subpix=True)
    want_x = o.deltaxs + nodes32[0].ravel()
    raw = np.asarray(last.deltaxs)
    ok = ~np.isnan(raw) & ~np.isnan(want_x) & (np.asarray(last.near_tie_flags) == 0)
    d = np.abs(raw[ok] - want_x[ok])
    print("deformed pass vs oracle: max", d.max(), "median", np.median(d))
    assert np.median(d) < 1e-3
    assert np.mean(d < 5e-3) > 0.99

    def rms(r):
        gx, gy = r.ixvecs_final.astype(float), r.iyvecs_final.astype(float)
        tx, ty = field(gx, gy)
        inner = (gx > 32) & (gx < 480) & (gy > 32) & (gy < 480)
        e = np.hypot(r.deltaxs_final - tx, r.deltays_final - ty)[inner]
        return float(np.sqrt(np.mean(e ** 2)))

    e_def, e_shift = rms(res_def.passes[-1]), rms(res_shift.passes[-1])
    print("RMS error vs imposed field: deformation", e_def, "window shift", e_shift)
    assert e_def < e_shift


def test_deformed_multipass_with_tensor_core_pass():
    """Deformation mode with the 32 px passes on the tensor cores (fp16 3-term): the
    deformed images are float32, which the tensor-core pass takes like integer
    images; the final field stays within 5e-3 px of the FP32 FFT form's."""
    import torch

    from fluidimage_gb300 import WorkPIV, synthetic, workloads

    model = synthetic.ParticleModel(density=0.05, diameter=(2.0, 3.0), intensity=(1000, 4000),
                                    noise=20.0, dtype="uint16", max_value=4095)
    field = synthetic.oseen_vortex((512, 512), d_max=6.0, rc=60.0)
    im0, im1 = synthetic.make_pair((512, 512), field, model, seed=78)
    params = workloads.config2_params(WorkPIV.create_default_params())
    ref = WorkPIV(params, deform=True).calcul({"arrays": (im0, im1), "names": ("a", "b")})
    params_tc = workloads.config2_params(WorkPIV.create_default_params())
    params_tc.piv0.method_correl = "gb300_tc_fp16x3"
    got = WorkPIV(params_tc, deform=True).calcul({"arrays": (im0, im1), "names": ("a", "b")})
    torch.cuda.synchronize()
    a, b = ref.passes[-1], got.passes[-1]
    d = np.hypot(a.deltaxs_final - b.deltaxs_final, a.deltays_final - b.deltays_final)
    print("deformed multipass, tensor-core vs FFT 32 px pass: max", d.max(), "median",
          np.median(d))
    assert np.median(d) < 1e-4
    assert np.mean(d < 5e-3) > 0.99
