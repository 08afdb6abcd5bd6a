"""The CPU oracle against golden vectors recorded from the upstream PIV code.

These pin the oracle: every output of ``oracle.piv.multipass`` must equal what the
upstream ``WorkPIV.calcul`` produced on the same images (bit for bit: same numpy
FFT, same float32 peak/subpixel arithmetic, same float64 TPS).
"""

import numpy as np
import pytest

import goldens
from oracle import piv as O

PASS_ARRAYS = ["deltaxs", "deltays", "xs", "ys", "correls_max"]
INTERP_ARRAYS = [
    "deltaxs_approx", "deltays_approx", "deltaxs_final", "deltays_final",
    "deltaxs_smooth", "deltays_smooth", "xs_smooth", "ys_smooth",
    "deltaxs_input", "deltays_input",
]


def _eq(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    assert a.shape == b.shape
    np.testing.assert_array_equal(a, b)


@pytest.fixture(scope="module", params=goldens.fixture_names())
def golden_run(request):
    z = goldens.load(request.param)
    params = goldens.params_namespace(z)
    keep = any(k.endswith("_planes") for k in z.files)
    return z, O.multipass(z["im0"], z["im1"], params, keep_planes=keep)


def test_pass_outputs_bit_exact(golden_run):
    z, results = golden_run
    assert len(results) == int(z["nb_passes"])
    for ip, r in enumerate(results):
        _eq(r.ixvecs, z[f"p{ip}_ixvecs"])
        _eq(r.iyvecs, z[f"p{ip}_iyvecs"])
        for key in PASS_ARRAYS:
            _eq(getattr(r, key), z[f"p{ip}_{key}"])
        assert r.errors == goldens.errors(z, ip)
        for key in ("deltaxs_wrong", "deltays_wrong"):
            if f"p{ip}_{key}_keys" in z.files:
                got = {k: float(v) for k, v in getattr(r, key).items()}
                want = goldens.errors(z, ip, key)
                assert got.keys() == want.keys()
                np.testing.assert_array_equal(
                    [got[k] for k in sorted(got)], [want[k] for k in sorted(want)]
                )


def test_interpolated_fields_bit_exact(golden_run):
    z, results = golden_run
    for ip, r in enumerate(results):
        for key in INTERP_ARRAYS:
            if f"p{ip}_{key}" in z.files:
                _eq(getattr(r, key), z[f"p{ip}_{key}"])


def test_planes_bit_exact(golden_run):
    z, results = golden_run
    for ip, r in enumerate(results):
        if f"p{ip}_planes" in z.files:
            np.testing.assert_array_equal(r.planes, z[f"p{ip}_planes"])


def test_correl_window_plugin():
    """Per-window ``CorrelFFTNumpy`` contract: plane, norm, peak, subpix."""
    z = goldens.load("correl_window")
    tags = sorted({k.rsplit("_", 1)[0] for k in z.files if k.endswith("_plane")})
    assert tags
    for tag in tags:
        im0 = z[tag + "_im0"][None]
        im1 = z[tag + "_im1"][None]
        planes, norms = O.correl_fft(im0, im1)
        np.testing.assert_array_equal(planes[0], z[tag + "_plane"])
        assert norms[0] == float(z[tag + "_norm"])
        dmax = O.parse_displacement_max(
            __import__("json").loads(str(z[tag + "_dmax"])), planes.shape[1:]
        )
        dx, dy, cmax, err, i0, i1 = O.displacements_from_correl(
            planes, norms, planes.shape[1:], dmax
        )
        peak = z[tag + "_peak"]
        assert (dx[0], dy[0]) == (peak[0], peak[1])
        assert np.float32(cmax[0]) == np.float32(peak[2])
        want_err = str(z[tag + "_err"])
        assert O.ERROR_STRINGS.get(int(err[0]), "") == want_err
        np.testing.assert_array_equal(planes[0], z[tag + "_plane_after"])
        if tag + "_subpix" in z.files:
            sdx, sdy, wrong = O.subpix_2d_gaussian2(planes, i0, i1, planes.shape[1:])
            assert not wrong[0]
            np.testing.assert_allclose([sdx[0], sdy[0]], z[tag + "_subpix"], rtol=0,
                                       atol=1e-6)


@pytest.mark.parametrize("shape", [(24, 32), (21, 32), (12, 13), (7, 9)])
def test_like_fftshift_known_answer(shape):
    """Upstream ``calcul/test_correl.py:233-245``: exact equality with fftshift(a[::-1, ::-1])."""
    n0, n1 = shape
    a = np.reshape(np.arange(n0 * n1, dtype=np.float32), (n0, n1))
    np.testing.assert_array_equal(
        O.like_fftshift(a), np.ascontiguousarray(np.fft.fftshift(a[::-1, ::-1]))
    )


def test_correl_known_answers():
    """Upstream ``calcul/test_correl.py:67-111``: zero displacement within 1e-3 with
    ``correl_max == 1``; a (3.3, 5.8) px shift found within 0.8 px."""
    from fluidimage_gb300 import synthetic

    model = synthetic.ParticleModel(density=0.08, noise=0.0, dtype="uint8")
    big0, big1 = synthetic.make_pair((72, 72), synthetic.uniform_shift(3.3, 5.8), model,
                                     seed=7, as_float32=True)
    im0 = big0[20:52, 20:52][None].copy()
    im1 = big1[20:52, 20:52][None].copy()
    for a, b, want in ((im0, im0, (0.0, 0.0)), (im0, im1, (3.3, 5.8))):
        planes, norms = O.correl_fft(a, b)
        dx, dy, cmax, err, i0, i1 = O.displacements_from_correl(planes, norms, (32, 32), 16.0)
        assert err[0] == 0
        sdx, sdy, _ = O.subpix_2d_gaussian2(planes, i0, i1, (32, 32))
        tol = 1e-3 if want == (0.0, 0.0) else 0.8
        assert abs(sdx[0] - want[0]) < tol and abs(sdy[0] - want[1]) < tol
        if want == (0.0, 0.0):
            assert np.isclose(cmax[0], 1.0)


def test_fft_energy_parseval():
    """Upstream ``calcul/test_fft.py:8-40``: Parseval energy bookkeeping of the oracle."""
    rng = np.random.default_rng(0)
    w = rng.random((3, 24, 20)).astype(np.float32)
    planes, norms = O.correl_fft(w, w)
    wc = w - w.mean(axis=(1, 2), keepdims=True)
    np.testing.assert_allclose(norms, (wc.astype(np.float64) ** 2).sum(axis=(1, 2)),
                               rtol=5e-5)
    np.testing.assert_allclose(planes.max(axis=(1, 2)) / norms, 1.0, rtol=5e-5)


def test_secondary_peaks_and_replacements_bit_exact(golden_run):
    """nb_peaks_to_search >= 2: the other peaks of every window and the vectors
    WorkFIX replaced by one of them (with their old values)."""
    z, results = golden_run
    for ip, r in enumerate(results):
        if f"p{ip}_secondary_counts" in z.files:
            counts = np.array([-1 if o is None else len(o) for o in r.secondary_peaks])
            _eq(counts, z[f"p{ip}_secondary_counts"])
            flat = [p for o in r.secondary_peaks if o for p in o]
            _eq(np.array(flat, dtype=np.float64).reshape(-1, 3), z[f"p{ip}_secondary_peaks"])
        if f"p{ip}_replaced_keys" in z.files:
            rep = getattr(r, "replaced_vectors", {})
            _eq(sorted(rep), z[f"p{ip}_replaced_keys"])
            _eq([[float(v) for v in rep[k]] for k in sorted(rep)], z[f"p{ip}_replaced_vals"])
        else:
            assert not getattr(r, "replaced_vectors", {})


def test_new_fixtures_exercise_the_options():
    """The secondary-peak fixture replaces vectors in both passes; the subpixel
    fixtures hit close-boundary and wrong-subpix errors."""
    z = goldens.load("secondary_peaks_two_pass")
    assert z["p0_replaced_keys"].size > 0 and z["p1_replaced_keys"].size > 0
    z = goldens.load("subpix_centroid2_single")
    vals = [str(v) for v in z["p0_errors_vals"]]
    assert "close boundary" in vals and "wrong subpix" in vals
