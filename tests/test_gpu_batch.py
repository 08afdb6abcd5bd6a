"""Batched single-pass PIV (PIVBatch): pairs of mixed image sizes, dtypes, window
sizes (8-64 px) and overlaps in one batch give the results of WorkPIV on each
pair alone, with direct launches, after autotuning and through a CUDA graph replay.
The per-window code is the same, compiled into another kernel, so float32 rounding
may differ by an ulp: validity, error strings and vector positions must be equal,
displacements within 1e-5 px and correls_max within 1e-5 relative outside the
windows flagged as near-ties."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _jobs():
    from fluidimage_gb300 import WorkPIV, synthetic

    specs = [  # (shape, dtype, window, overlap, field)
        ((160, 224), "uint8", 16, 0.5, synthetic.uniform_shift(2.2, -1.4)),
        ((256, 192), "uint16", 24, 0.75, synthetic.uniform_shift(-3.1, 2.6)),
        ((200, 200), "uint16", 32, 0.5, synthetic.oseen_vortex((200, 200), d_max=5.0, rc=40.0)),
        ((288, 320), "uint8", 48, 0.75, synthetic.uniform_shift(4.4, 1.9)),
        ((256, 256), "float32", 64, 0.5, synthetic.uniform_shift(-5.2, -2.7)),
        ((192, 160), "uint16", 16, 0.75, synthetic.sinusoid(3.0, 160.0)),
        ((320, 256), "uint8", 32, 0.75, synthetic.uniform_shift(1.3, 5.1)),
        ((96, 128), "uint8", 12, 0.5, synthetic.uniform_shift(1.4, -0.8)),
        ((80, 112), "uint16", 8, 0.5, synthetic.uniform_shift(-0.7, 1.2)),
    ]
    jobs = []
    for k, (shape, dtype, n, ov, field) in enumerate(specs):
        if dtype == "uint16":
            model = synthetic.ParticleModel(density=0.05, intensity=(1000, 4000), noise=20.0,
                                            dtype="uint16", max_value=4095)
        else:
            model = synthetic.ParticleModel(density=0.05, noise=2.0, dtype="uint8")
        im0, im1 = synthetic.make_pair(shape, field, model, seed=500 + k,
                                       as_float32=(dtype == "float32"))
        params = WorkPIV.create_default_params()
        params.piv0.shape_crop_im0 = n
        params.piv0.grid.overlap = ov
        params.fix.threshold_diff_neighbour = 3 if k % 2 else None
        jobs.append((im0, im1, params))
    return jobs


def _check(got, want):
    assert len(got) == len(want)
    for r, w in zip(got, want):
        nt = (w.near_tie_flags == 0) & (r.near_tie_flags == 0)
        np.testing.assert_array_equal(np.isnan(r.deltaxs)[nt], np.isnan(w.deltaxs)[nt])
        ok = nt & ~np.isnan(w.deltaxs)
        np.testing.assert_allclose(r.deltaxs[ok], w.deltaxs[ok], rtol=0, atol=1e-5)
        np.testing.assert_allclose(r.deltays[ok], w.deltays[ok], rtol=0, atol=1e-5)
        okc = nt & ~np.isnan(w.correls_max)
        np.testing.assert_allclose(r.correls_max[okc], w.correls_max[okc], rtol=1e-5, atol=1e-6)
        np.testing.assert_array_equal(np.asarray(r.xs), np.asarray(w.xs))
        skip = set(np.nonzero(~nt)[0].tolist())
        assert {k: v for k, v in r.errors.items() if k not in skip} == \
            {k: v for k, v in w.errors.items() if k not in skip}


def test_batch_matches_workpiv():
    import torch

    from fluidimage_gb300 import PIVBatch, WorkPIV

    jobs = _jobs()
    want = [WorkPIV(p, interp_last=False).calcul({"arrays": (a, b), "names": ("a", "b")}).passes[0]
            for a, b, p in jobs]
    batch = PIVBatch(jobs)
    assert set(batch.groups) == {8, 12, 16, 24, 32, 48, 64}
    batch.run()
    torch.cuda.synchronize()
    _check(batch.results(), want)
    # autotuned configuration, then a CUDA graph replayed twice on zeroed outputs
    choice = batch.autotune(reps=1)
    assert set(choice) == set(batch.groups)
    batch.capture()
    for _ in range(2):
        for job in batch.jobs:
            job.out.deltaxs_raw.zero_()
            job.out.deltaxs.zero_()
        batch.run()
        torch.cuda.synchronize()
        _check(batch.results(), want)
