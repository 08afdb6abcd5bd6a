"""The two CPU restatements of the deformation agree (numpy oracle and the torch
autograd reference), and the torch reference's gradient equals FP64 central finite
differences on a small case: the references the GPU adjoint is checked against are
themselves consistent.  The bilinear sampling is piecewise linear in the field, so
differences over h = 1e-3 px include the kinks of the pixels that cross an integer
position inside the stencil (a few percent on a 96 x 128 image); over h = 1e-5 px
they agree to 1e-4."""

import numpy as np
import pytest
import torch

import deform_reference as R
from oracle import deform as OD


def _case(seed=0, H=96, W=128):
    from fluidimage_gb300 import synthetic

    model = synthetic.ParticleModel(density=0.06, noise=2.0, dtype="uint8")
    im0, im1 = synthetic.make_pair((H, W), synthetic.uniform_shift(2.3, -1.6), model, seed=seed)
    xn = (16.0 + 32.0 * np.arange(W // 32)).astype(np.float32)
    yn = (16.0 + 32.0 * np.arange(H // 32)).astype(np.float32)
    rng = np.random.default_rng(seed)
    nodes = np.stack([2.3 + 0.4 * rng.standard_normal((yn.size, xn.size)),
                      -1.6 + 0.4 * rng.standard_normal((yn.size, xn.size))])
    return im0.astype(np.float64), im1.astype(np.float64), nodes, xn, yn


@pytest.mark.parametrize("scale", [1.0, 0.5, -0.5])
def test_torch_reference_warp_equals_numpy_oracle(scale):
    im0, im1, nodes, xn, yn = _case()
    got = R.warp(torch.as_tensor(nodes)[None], torch.as_tensor(xn), torch.as_tensor(yn),
                 torch.as_tensor(im1)[None], scale)[0].numpy()
    np.testing.assert_allclose(got, OD.warp(nodes, xn, yn, im1, scale), rtol=0, atol=1e-9)


@pytest.mark.parametrize("symmetric", [True, False], ids=["central", "im1_only"])
def test_torch_reference_gradient_equals_central_differences(symmetric):
    im0, im1, nodes, xn, yn = _case(seed=3)
    t0 = torch.as_tensor(im0)[None]
    t1 = torch.as_tensor(im1)[None]
    txn, tyn = torch.as_tensor(xn), torch.as_tensor(yn)
    p = torch.as_tensor(nodes)[None].clone().requires_grad_(True)
    R.loss(p, t0, t1, txn, tyn, symmetric=symmetric).backward()
    g = p.grad[0].numpy()
    for h, rel in ((1e-3, 5e-2), (1e-5, 1e-4)):
        for c, i, j in [(0, 0, 0), (1, 1, 2), (0, 2, 3), (1, 2, 1)]:
            a = torch.as_tensor(nodes)[None].clone()
            b = a.clone()
            a[0, c, i, j] += h
            b[0, c, i, j] -= h
            fd = (R.loss(a, t0, t1, txn, tyn, symmetric=symmetric)
                  - R.loss(b, t0, t1, txn, tyn, symmetric=symmetric)).item() / (2 * h)
            assert abs(fd - g[c, i, j]) <= rel * max(abs(fd), 1e-3), (h, c, i, j, fd, g[c, i, j])
