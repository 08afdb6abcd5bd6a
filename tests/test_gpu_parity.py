"""GPU parity against golden vectors recorded from the upstream PIV code.

Tolerances (the reference computes float32 FFTs with numpy's pocketfft, the
GPU float32 FFTs in registers, so planes differ by float32 rounding):

* integer peak positions: exact, except on windows flagged as near-ties, which are
  counted and reported: the top two plane values within 1e-6 relative (the "last
  maximum" then depends on float rounding), or two values of the 3x3 subpixel crop
  at its minimum (the '2d_gaussian2' 1e-8 floor then depends on float rounding);
* displacements: within 5e-3 px of the reference (the stated bar), and in
  practice within 1e-4 px;
* correls_max: within 2e-5 relative;
* TPS-interpolated fields (float64 on both sides, inputs differing by float32
  rounding): within 1e-3 px; the rounded window shifts must match exactly;
* error dictionaries: same keys and strings (the "(diff = x.xx)" number may
  differ by 0.01 when the upstream value sits on a rounding boundary).
"""

import numpy as np
import pytest

import goldens

pytestmark = pytest.mark.gpu

TOL_PX = 5e-3
TOL_PX_TYPICAL = 1e-4


def _params(z):
    from fluidimage_gb300 import WorkPIV

    params = WorkPIV.create_default_params()
    for path, value in goldens.settings(z).items():
        obj = params
        parts = path.split(".")
        for part in parts[:-1]:
            obj = getattr(obj, part)
        setattr(obj, parts[-1], value)
    params.piv0.method_correl = "gb300"
    return params


def _run(name, **kw):
    import torch

    from fluidimage_gb300 import WorkPIV

    z = goldens.load(name)
    params = _params(z)
    keep = any(k.endswith("_planes") for k in z.files)
    work = WorkPIV(params, keep_correls=keep, **kw)
    res = work.calcul({"arrays": (z["im0"], z["im1"]), "names": ("im0", "im1")})
    torch.cuda.synchronize()
    return z, res


def _same_errors(got, want, skip=()):
    skip = set(skip)
    gk = set(got) - skip
    wk = set(want) - skip
    assert gk == wk, (gk ^ wk)
    for k in wk:
        g, w = got[k], want[k]
        if g == w:
            continue
        gs, ws = g.split(" (diff = "), w.split(" (diff = ")
        assert gs[0] == ws[0] and len(gs) == len(ws) == 2, (k, g, w)
        assert abs(float(gs[1][:-1]) - float(ws[1][:-1])) <= 0.0100001, (k, g, w)


def _griddata_of(r, key):
    """The oracle's ``griddata`` (scipy, linear then nearest) of the pass's own
    vectors onto the grid of field ``key`` (``..._approx`` or ``..._final``)."""
    from oracle import piv as O

    kind = key.split("_")[1]
    gx = np.asarray(getattr(r, "ixvecs_" + kind))
    gy = np.asarray(getattr(r, "iyvecs_" + kind))
    sel = ~(np.isnan(r.deltaxs) | np.isnan(r.deltays))
    comp = r.deltaxs if key.startswith("deltaxs") else r.deltays
    centers = np.vstack([np.asarray(r.xs, float)[sel], np.asarray(r.ys, float)[sel]])
    return O.griddata(centers, np.asarray(comp, np.float64)[sel], np.unique(gx),
                      np.unique(gy))


def _interp_of(r, key, z):
    """The oracle's apply_interp (FP64 TPS, or scipy's griddata, as the parameters
    say) of the pass's own vectors onto the grid of field ``key``."""
    from types import SimpleNamespace

    from oracle import piv as O

    last = not key.endswith("_approx")
    kind = "final" if last else "approx"
    gx = np.unique(np.asarray(getattr(r, "ixvecs_" + kind)))
    gy = np.unique(np.asarray(getattr(r, "iyvecs_" + kind)))
    # float64 positions like upstream's (xs = (ixs0 + ixs1) / 2.0, half-integers)
    ns = SimpleNamespace(xs=np.asarray(r.xs, np.float64), ys=np.asarray(r.ys, np.float64),
                         deltaxs=np.asarray(r.deltaxs), deltays=np.asarray(r.deltays))
    O.apply_interp(ns, (gx, gy), goldens.params_namespace(z).multipass, last=last)
    return np.asarray(getattr(ns, key))


def _compare_pass(z, ip, r, report, prev=None):
    """Strict comparison outside the flagged near-tie vectors (counted).  A vector
    whose window shift came from an ambiguous griddata point of the previous pass
    (several Delaunay triangulations; upstream follows Qhull's), or from a triangle
    holding such a vector, and differs from upstream's shift is counted with them."""
    gdx = z[f"p{ip}_deltaxs"]
    gdy = z[f"p{ip}_deltays"]
    tie = r.near_tie_flags != 0
    amb = getattr(prev, "griddata_tie_flags_approx", None)
    if amb is not None:
        # a griddata value that is a half-integer (a grid point midway between two
        # vectors): the shift is np.round of it, and upstream's rounding then follows
        # the last-ulp error of scipy's barycentric transform, not the exact value
        amb = np.asarray(amb) != 0
        for comp in ("deltaxs_approx", "deltays_approx"):
            v = np.asarray(getattr(prev, comp), np.float64)
            amb = amb | (np.abs(np.abs(v - np.floor(v)) - 0.5) <= 4 * np.spacing(np.abs(v) + 1.0))
    if amb is not None and f"p{ip}_deltaxs_input" in z.files:
        moved = ((r.deltaxs_input != z[f"p{ip}_deltaxs_input"])
                 | (r.deltays_input != z[f"p{ip}_deltays_input"]))
        odd = moved & ~amb
        if odd.any():
            # an unambiguous point whose triangle holds a vector of the previous pass
            # that differs from upstream's (a near-tie, or itself moved): the shift
            # must be upstream's rule, round(griddata), applied to the GPU's vectors
            for comp in ("deltaxs", "deltays"):
                want = np.round(_griddata_of(prev, comp + "_approx")).astype(np.int32)
                np.testing.assert_array_equal(getattr(r, comp + "_input")[odd], want[odd],
                                              err_msg="a shift differs at an unambiguous point")
        tie = tie | moved
        report.append({"pass": ip, "shifts_from_ambiguous_griddata": int(moved.sum())})
    nt = ~tie
    np.testing.assert_array_equal(np.isnan(r.deltaxs)[nt], np.isnan(gdx)[nt])
    ok = ~np.isnan(gdx) & nt
    d = np.abs(np.concatenate([r.deltaxs[ok] - gdx[ok], r.deltays[ok] - gdy[ok]]))
    report.append({"pass": ip, "max_px": float(d.max(initial=0.0)),
                   "median_px": float(np.median(d)) if d.size else 0.0,
                   "near_ties": int(tie.sum())})
    assert (d <= TOL_PX).all(), f"pass {ip}: max |d - ref| = {d.max()} px"
    if d.size:
        assert np.median(d) < TOL_PX_TYPICAL
    cm = z[f"p{ip}_correls_max"]
    okc = ~np.isnan(cm) & nt
    np.testing.assert_allclose(r.correls_max[okc], cm[okc], rtol=2e-5, atol=2e-6)
    np.testing.assert_array_equal(np.asarray(r.xs, float)[nt], z[f"p{ip}_xs"][nt])
    np.testing.assert_array_equal(np.asarray(r.ys, float)[nt], z[f"p{ip}_ys"][nt])
    skip = set(np.nonzero(tie)[0].tolist())
    _same_errors(r.errors, goldens.errors(z, ip), skip)
    for key in ("deltaxs_input", "deltays_input"):
        if f"p{ip}_{key}" in z.files:
            np.testing.assert_array_equal(getattr(r, key)[nt], z[f"p{ip}_{key}"][nt])
    # interpolated fields; griddata points in cells of cocircular vectors (or with
    # equidistant nearest vectors) have several valid values (upstream's follows
    # Qhull's triangulation): they are counted and left out
    for key in ("deltaxs_approx", "deltays_approx", "deltaxs_final", "deltays_final",
                "deltaxs_smooth", "deltays_smooth"):
        if f"p{ip}_{key}" in z.files:
            got, want = getattr(r, key), z[f"p{ip}_{key}"]
            flags = getattr(r, "griddata_tie_flags_" + key.split("_")[1], None)
            sel = np.ones(want.shape, bool) if flags is None else flags == 0
            if not key.endswith("_approx"):  # on this pass's grid
                sel &= nt
            if flags is not None:
                report.append({"pass": ip, key + "_griddata_ties": int((~sel).sum())})
            if not bool(nt.all()):
                # a vector moved by an ambiguous shift (or a near-tie peak) changes
                # the interpolation around it (griddata's triangles, the TPS of its
                # subdomains): the GPU field is then checked against the oracle's
                # interpolation of the GPU's own vectors
                want = _interp_of(r, key, z)
                np.testing.assert_allclose(got[sel], want[sel], rtol=0, atol=1e-5,
                                           err_msg=key)
                continue
            np.testing.assert_allclose(got[sel], want[sel], rtol=0, atol=1e-3, err_msg=key)
    for key in ("ixvecs_approx", "iyvecs_approx", "ixvecs_final", "iyvecs_final",
                "xs_smooth", "ys_smooth"):
        if f"p{ip}_{key}" in z.files:
            m = nt if key.endswith("_smooth") else np.ones(z[f"p{ip}_{key}"].shape, bool)
            np.testing.assert_array_equal(getattr(r, key)[m], z[f"p{ip}_{key}"][m], err_msg=key)
    for key in ("deltaxs_wrong", "deltays_wrong"):
        if f"p{ip}_{key}_keys" in z.files:
            want = {k: v for k, v in goldens.errors(z, ip, key).items() if k not in skip}
            got = {k: v for k, v in getattr(r, key).items() if k not in skip}
            assert got.keys() == want.keys()
            np.testing.assert_allclose([got[k] for k in sorted(got)],
                                       [want[k] for k in sorted(want)], atol=TOL_PX)
    if f"p{ip}_secondary_counts" in z.files:
        _compare_secondary(z, ip, r, tie, report)


def _compare_secondary(z, ip, r, tie, report):
    """Secondary peaks (exact integer displacements, correl_max within float32
    rounding) and the vectors WorkFIX replaced, outside near-ties; a replacement
    also depends on the neighbours, so vectors next to a near-tie are left out."""
    counts = z[f"p{ip}_secondary_counts"]
    flat = z[f"p{ip}_secondary_peaks"]
    starts = np.concatenate([[0], np.cumsum(np.maximum(counts, 0))])
    for i, other in enumerate(r.secondary_peaks):
        if tie[i]:
            continue
        assert (other is None) == (counts[i] < 0), i
        if other is None:
            continue
        want = flat[starts[i]:starts[i + 1]]
        assert len(other) == len(want), (i, other, want)
        for (dx, dy, cm), (wdx, wdy, wcm) in zip(other, want):
            assert (dx, dy) == (int(wdx), int(wdy)), (i, other, want)
            np.testing.assert_allclose(cm, wcm, rtol=2e-5, atol=2e-6)
    grid = tie.reshape(-1)
    lay_ny = z[f"p{ip}_iyvecs"].size
    lay_nx = z[f"p{ip}_ixvecs"].size
    t2 = grid.reshape(lay_ny, lay_nx)
    near = np.zeros_like(t2)
    for a in (-1, 0, 1):
        for b in (-1, 0, 1):
            near |= np.roll(np.roll(t2, a, 0), b, 1)
    near = near.reshape(-1)
    rep = getattr(r, "replaced_vectors", {})
    keys = z[f"p{ip}_replaced_keys"] if f"p{ip}_replaced_keys" in z.files else np.zeros(0, int)
    vals = z[f"p{ip}_replaced_vals"] if f"p{ip}_replaced_keys" in z.files else np.zeros((0, 3))
    want = {int(k): v for k, v in zip(keys, vals) if not near[int(k)]}
    got = {k: v for k, v in rep.items() if not near[k]}
    assert got.keys() == want.keys(), (sorted(got), sorted(want))
    for k in want:
        np.testing.assert_allclose(np.asarray(got[k], float), want[k], atol=TOL_PX, rtol=2e-5)
    report.append({"pass": ip, "replaced": len(rep), "replaced_ref": int(keys.size)})


@pytest.mark.parametrize("name", ["single_pass_c1", "multipass_small", "dmax_two_pass",
                                  "edges_single_pass", "secondary_peaks_two_pass",
                                  "griddata_two_pass", "griddata_oseen_three_pass",
                                  "subpix_gaussian_single", "subpix_centroid2_single",
                                  "subpix_none_single", "multipass_48_24",
                                  "single_pass_24_ov75", "multipass_64_32_ov75",
                                  "minimal_piv_oseen", "multipass_48_24_12",
                                  "multipass_16_8"])
def test_workpiv_matches_reference(name):
    z, res = _run(name)
    assert len(res.passes) == int(z["nb_passes"])
    report = []
    prev = None
    for ip, r in enumerate(res.passes):
        _compare_pass(z, ip, r, report, prev)
        prev = r
    print(name, report)


@pytest.mark.parametrize("name", ["multipass_small", "multipass_48_24"])
def test_tps_lu_fallback_matches_reference(name, monkeypatch):
    """Every TPS subdomain through the FP64 LU kernel (the path of the subdomains the
    mixed-precision solver hands over: rank-deficient P, a non-positive pivot, no
    convergence, or more members than its shared-memory tiles hold), forced by a
    member limit of 0: same results as upstream, and every subdomain flagged."""
    from fluidimage_gb300 import engine

    monkeypatch.setattr(engine, "MP_MAX_MEMBERS", 0)
    z, res = _run(name, device="cuda")
    report = []
    prev = None
    for ip, r in enumerate(res.passes):
        _compare_pass(z, ip, r, report, prev)
        prev = r
    print(name, report)


def test_planes_match_reference():
    """Correlation planes (kept on request) equal upstream's within float32 rounding,
    including NaN boxes written by the second-chance search."""
    for name in ("dmax_two_pass", "edges_single_pass"):
        z, res = _run(name)
        for ip, r in enumerate(res.passes):
            if f"p{ip}_planes" not in z.files:
                continue
            want = z[f"p{ip}_planes"]
            for i, c in enumerate(r.correls):
                if c is None:
                    assert np.isnan(want[i]).all()
                    continue
                w = want[i]
                np.testing.assert_array_equal(np.isnan(c), np.isnan(w))
                scale = np.nanmax(np.abs(w)) or 1.0
                np.testing.assert_allclose(c[~np.isnan(w)] / scale, w[~np.isnan(w)] / scale,
                                           atol=2e-6)


def test_correl_plugin_per_window():
    """CorrelGB300 per-window contract against upstream CorrelFFTNumpy."""
    from fluidimage_gb300 import CorrelGB300, PIVError

    z = goldens.load("correl_window")
    tags = sorted({k.rsplit("_", 1)[0] for k in z.files if k.endswith("_plane")})
    for tag in tags:
        im0, im1 = z[tag + "_im0"], z[tag + "_im1"]
        import json

        dmax = json.loads(str(z[tag + "_dmax"]))
        c = CorrelGB300(im0.shape, im1.shape, displacement_max=dmax)
        plane, norm = c(im0, im1)
        want = z[tag + "_plane"]
        assert plane.dtype == np.float32 and plane.shape == want.shape
        np.testing.assert_allclose(plane / norm, want / float(z[tag + "_norm"]), atol=2e-6)
        assert norm == pytest.approx(float(z[tag + "_norm"]), rel=1e-5)
        peak = z[tag + "_peak"]
        err = str(z[tag + "_err"])
        try:
            dx, dy, cmax, other = c.compute_displacements_from_correl(plane, norm)
            got_err = ""
        except PIVError as e:
            dx, dy, cmax = e.results
            got_err = e.explanation
        assert got_err == err
        assert (dx, dy) == (peak[0], peak[1])
        assert cmax == pytest.approx(peak[2], rel=1e-5, abs=1e-6)
        np.testing.assert_array_equal(np.isnan(plane), np.isnan(z[tag + "_plane_after"]))
        if tag + "_subpix" in z.files:
            sdx, sdy = c.apply_subpix(dx, dy, plane)
            # identical windows give a symmetric 3x3 crop whose equal minima make the
            # '2d_gaussian2' 1e-8 floor depend on float rounding (a subpixel near-tie)
            iy, ix = c.iy0 - int(dy), c.ix0 - int(dx)
            crop = want[iy - 1:iy + 2, ix - 1:ix + 2].astype(np.float64)
            norm_crop = (crop - crop.min()) / (crop.max() - crop.min())
            tied = np.count_nonzero(norm_crop < 1e-5) >= 2
            tol = 5e-2 if tied else TOL_PX_TYPICAL
            np.testing.assert_allclose([sdx, sdy], z[tag + "_subpix"], atol=tol)


@pytest.mark.parametrize("order", ["rows", "shuffled"])
def test_members_index_range_matches_full_scan(order):
    """fi_tps_members restricted by fi_tps_y_bounds gives the same ordered members as
    the scan over every point, for row-ordered and for shuffled points (on and off
    the half-integer lattice)."""
    import torch

    from fluidimage_gb300 import _lib as L, engine

    lib = L.load()
    dev = torch.device("cuda")
    rng = np.random.default_rng(5)
    ny, nx = 70, 90
    ys, xs = np.meshgrid(np.arange(ny) * 8.0 + 4.0, np.arange(nx) * 8.0 + 4.0, indexing="ij")
    xs = (xs + rng.integers(0, 2, xs.shape) * 0.5).ravel()
    ys = (ys + rng.integers(0, 2, ys.shape) * 0.5).ravel()
    if order == "shuffled":
        perm = rng.permutation(xs.size)
        xs, ys = xs[perm], ys[perm]
    dx = rng.normal(0, 1, xs.size).astype(np.float32)
    dy = rng.normal(0, 1, xs.size).astype(np.float32)
    dx[rng.random(xs.size) < 0.05] = np.nan
    f32 = lambda a: torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).to(dev)  # noqa: E731
    tx, ty, tdx, tdy = f32(xs), f32(ys), f32(dx), f32(dy)
    n = xs.size
    plan = torch.empty(L.TPS_PLAN_BYTES, dtype=torch.uint8, device=dev)
    cx = torch.empty(n, dtype=torch.float64, device=dev)
    cy = torch.empty(n, dtype=torch.float64, device=dev)
    ux = torch.empty(n, dtype=torch.float32, device=dev)
    uy = torch.empty(n, dtype=torch.float32, device=dev)
    sel = torch.empty(n, dtype=torch.int32, device=dev)
    L.check(lib.fi_tps_plan_make(L.ptr(tx), L.ptr(ty), L.ptr(tdx), L.ptr(tdy), n, 200, 0.5, 20.0,
                                 L.ptr(plan), L.ptr(cx), L.ptr(cy), L.ptr(ux), L.ptr(uy),
                                 L.ptr(sel), None), "plan")
    hdr = L.TpsPlan.from_buffer_copy(plan.cpu().numpy().tobytes())
    nv, nsub = hdr.num_centers, hdr.nb_subdomx * hdr.nb_subdomy
    assert nsub > 20
    for lattice in (True, False):
        xy2, flag = engine.lattice_coords(cx, cy, nv) if lattice else (None, None)
        b0, b1 = engine.y_bounds(cy, nv)
        res = []
        for bounded in (False, True):
            cnt = torch.empty(nsub, dtype=torch.int32, device=dev)
            args = (L.ptr(xy2), L.ptr(flag)) if lattice else (None, None)
            bargs = (L.ptr(b0), L.ptr(b1)) if bounded else (None, None)
            L.check(lib.fi_tps_members(L.ptr(plan), nsub, L.ptr(cx), L.ptr(cy), nv, 0, L.ptr(cnt),
                                       None, None, None, *args, *bargs, None), "count")
            ch = cnt.cpu().numpy().astype(np.int64)
            off = torch.from_numpy(np.concatenate([[0], np.cumsum(ch)[:-1]])).to(dev)
            idx = torch.empty(int(ch.sum()), dtype=torch.int32, device=dev)
            coefs = torch.empty(int(ch.sum()), dtype=torch.float64, device=dev)
            L.check(lib.fi_tps_members(L.ptr(plan), nsub, L.ptr(cx), L.ptr(cy), nv, 1, None,
                                       L.ptr(off), L.ptr(idx), L.ptr(coefs), *args, *bargs, None),
                    "fill")
            torch.cuda.synchronize()
            res.append((ch, idx.cpu().numpy(), coefs.cpu().numpy()))
        np.testing.assert_array_equal(res[0][0], res[1][0])
        np.testing.assert_array_equal(res[0][1], res[1][1])
        np.testing.assert_array_equal(res[0][2], res[1][2])
        assert res[0][0].sum() > nv  # buffers overlap: points in several subdomains


@pytest.mark.parametrize("name", ["secondary_peaks_two_pass", "subpix_gaussian_single",
                                  "subpix_centroid2_single", "subpix_none_single"])
def test_correl_plugin_loop_vectors(name):
    """The per-window plugin driven like upstream's _loop_vectors on the first pass
    of a fixture (subpixel method, nsubpix, other peaks), against the oracle's pass
    (itself bit-exact to the fixture): same errors, other peaks and displacements."""
    from fluidimage_gb300 import CorrelGB300, PIVError
    from oracle import piv as O

    z = goldens.load(name)
    p = goldens.params_namespace(z)
    n = int(z["p0_shape_crop"][0])
    shape = (n, n)
    ref = O.piv_pass(z["im0"], z["im1"], shape, p.piv0.grid.overlap,
                     displacement_max=p.piv0.displacement_max, keep_planes=True,
                     method_subpix=p.piv0.method_subpix, nsubpix=p.piv0.nsubpix,
                     nb_peaks_to_search=p.piv0.nb_peaks_to_search)
    gx, gy = ref.ixvecs_grid, ref.iyvecs_grid
    im0pad, im1pad, npad = O.pad_images(z["im0"], z["im1"], shape)
    _, _, ix0p, iy0p, ix1p, iy1p = O.positions_first_pass(gx, gy, npad)
    w0, v0 = O.crop_windows(im0pad, ix0p, iy0p, shape)
    w1, v1 = O.crop_windows(im1pad, ix1p, iy1p, shape)
    c = CorrelGB300(shape, shape, method_subpix=p.piv0.method_subpix, nsubpix=p.piv0.nsubpix,
                    displacement_max=p.piv0.displacement_max,
                    particle_radius=p.piv0.particle_radius,
                    nb_peaks_to_search=p.piv0.nb_peaks_to_search)
    checked = 0
    for k in range(0, gx.size, 2):
        if not (v0[k] and v1[k]):
            continue
        plane, norm = c(w0[k], w1[k])
        top = np.sort(plane[np.isfinite(plane)].ravel())[-2:]
        if top[1] - top[0] <= 1e-6 * abs(top[1]):  # near-tie: the peak depends on rounding
            continue
        try:
            dx, dy, cmax, other = c.compute_displacements_from_correl(plane, norm)
        except PIVError as e:
            assert ref.err[k] in (O.ERR_BOUNDARY, O.ERR_NAN), (k, e.explanation)
            assert ref.secondary_peaks[k] is None
            continue
        want = ref.secondary_peaks[k]
        if p.piv0.nb_peaks_to_search > 1:
            assert len(other) == len(want), (k, other, want)
            for (a, b, cm), (wa, wb, wcm) in zip(other, want):
                assert (a, b) == (int(wa), int(wb))
                np.testing.assert_allclose(cm, wcm, rtol=2e-5, atol=2e-6)
        else:
            assert other is None
        try:
            sdx, sdy = c.apply_subpix(dx, dy, plane)
            got_err = 0
        except PIVError as e:
            got_err = {"wrong subpix": O.ERR_WRONG_SUBPIX,
                       "close boundary": O.ERR_CLOSE_BOUNDARY}[e.explanation]
            sdx, sdy = float(dx), float(dy)
        assert got_err == ref.err[k], k
        np.testing.assert_allclose([sdx, sdy], [ref.deltaxs[k], ref.deltays[k]], atol=TOL_PX)
        checked += 1
    assert checked > 20
