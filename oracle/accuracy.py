"""Error of a GPU PIV result against the FP64 oracle — TEST INFRASTRUCTURE ONLY.

The FP64 oracle is ``oracle.piv.multipass(..., dtype_complex=np.complex128)``:
the upstream algorithm (calcul/correl.py:671-685, calcul/subpix.py:16-61, the
WorkFIX and TPS steps) with complex128 FFTs, float64 planes and a float64
'2d_gaussian2' fit.  These helpers state a result's error against it:

* displacement error (px) of each pass, over the vectors that both kept, whose
  windows were cut at the same integer shift and that are not near-ties (those
  three exclusions are counted);
* the final interpolated field's error (px);
* the correlation planes' relative error (max |c - c64| / max |c64| per window).

Used by the tests and by the benchmark as the checker; nothing in the package
imports it.
"""

from __future__ import annotations

import numpy as np

from . import piv as O


def fp64_multipass(im0, im1, params, keep_planes=False):
    """The FP64 oracle's passes for a couple of images."""
    return O.multipass(im0, im1, params, dtype_complex=np.complex128, keep_planes=keep_planes)


def displacement_error(result, ref):
    """Error of one pass ``result`` (HeavyPIVResults-like: ``deltaxs``, ``deltays``,
    ``near_tie_flags``, optional ``deltaxs_input``) against the FP64 oracle pass
    ``ref``."""
    dx, dy = np.asarray(result.deltaxs, np.float64), np.asarray(result.deltays, np.float64)
    rx, ry = np.asarray(ref.deltaxs, np.float64), np.asarray(ref.deltays, np.float64)
    both = ~np.isnan(dx) & ~np.isnan(rx)
    ties = np.asarray(getattr(result, "near_tie_flags", np.zeros(dx.size, np.uint8))) != 0
    shift = np.zeros(dx.size, bool)
    if getattr(result, "deltaxs_input", None) is not None and ref.deltaxs_input is not None:
        shift = ((np.asarray(result.deltaxs_input) != np.asarray(ref.deltaxs_input))
                 | (np.asarray(result.deltays_input) != np.asarray(ref.deltays_input)))
    sel = both & ~ties & ~shift
    d = np.hypot(dx[sel] - rx[sel], dy[sel] - ry[sel])
    return {
        "max_px": float(d.max(initial=0.0)),
        "rms_px": float(np.sqrt(np.mean(d**2))) if d.size else 0.0,
        "compared": int(sel.sum()),
        "near_ties": int((both & ties).sum()),
        "other_shift": int((both & shift & ~ties).sum()),
    }


def final_field_error(result, ref):
    """Error (px) of the final interpolated field ``deltaxs_final``/``deltays_final``
    of the last pass against the FP64 oracle's."""
    if getattr(ref, "deltaxs_final", None) is None or getattr(result, "deltaxs_final", None) is None:
        return None
    d = np.hypot(np.asarray(result.deltaxs_final) - ref.deltaxs_final,
                 np.asarray(result.deltays_final) - ref.deltays_final)
    return {"max_px": float(np.nanmax(d)), "rms_px": float(np.sqrt(np.nanmean(d**2)))}


def plane_relative_error(planes, ref_planes):
    """Per-window ``max |c - c64| / max |c64|`` over the finite values of both
    (``planes``: sequence of n x n arrays or None; ``ref_planes``: [nvec, n, n])."""
    errs = []
    for i, c in enumerate(planes):
        if c is None:
            continue
        w = ref_planes[i]
        ok = np.isfinite(w) & np.isfinite(c)
        if not ok.any():
            continue
        scale = np.abs(w[ok]).max()
        if scale == 0:
            continue
        errs.append(np.abs(np.asarray(c, np.float64)[ok] - w[ok]).max() / scale)
    errs = np.asarray(errs)
    return {"max": float(errs.max(initial=0.0)),
            "median": float(np.median(errs)) if errs.size else 0.0,
            "windows": int(errs.size)}


def summary(results, refs):
    """Accuracy of a multipass result (list of passes) against the FP64 oracle's:
    the last pass's displacements and final field, plus every pass's displacement
    error."""
    last = displacement_error(results[-1], refs[-1])
    out = {"max_px": last["max_px"], "rms_px": last["rms_px"],
           "compared": last["compared"], "near_ties": last["near_ties"],
           "other_shift": last["other_shift"],
           "passes": [displacement_error(r, o) for r, o in zip(results, refs)]}
    fin = final_field_error(results[-1], refs[-1])
    if fin is not None:
        out["final_field_max_px"] = fin["max_px"]
        out["final_field_rms_px"] = fin["rms_px"]
    return out
