"""Helpers to load the golden fixtures recorded from the upstream PIV code."""

from __future__ import annotations

import json
from pathlib import Path
from types import SimpleNamespace

import numpy as np

GOLDEN_DIR = Path(__file__).resolve().parent / "golden"

DEFAULTS = {
    "piv0.shape_crop_im0": 48,
    "piv0.shape_crop_im1": None,
    "piv0.displacement_max": None,
    "piv0.method_correl": "fftw",
    "piv0.method_subpix": "2d_gaussian2",
    "piv0.nsubpix": None,
    "piv0.nb_peaks_to_search": 1,
    "piv0.particle_radius": 3,
    "piv0.grid.overlap": 0.5,
    "fix.correl_min": 0.2,
    "fix.threshold_diff_neighbour": 10,
    "fix.displacement_max": None,
    "multipass.number": 1,
    "multipass.coeff_zoom": 2,
    "multipass.use_tps": "last",
    "multipass.subdom_size": 200,
    "multipass.smoothing_coef": 5.0,
    "multipass.threshold_tps": 1.5,
}


def load(name):
    return np.load(GOLDEN_DIR / f"{name}.npz")


def settings(z):
    return json.loads(str(z["settings"]))


def params_namespace(z):
    """Upstream parameter tree (defaults + the fixture's settings) as namespaces."""
    values = dict(DEFAULTS)
    values.update(settings(z))
    root = SimpleNamespace()
    for path, value in values.items():
        obj = root
        parts = path.split(".")
        for p in parts[:-1]:
            if not hasattr(obj, p):
                setattr(obj, p, SimpleNamespace())
            obj = getattr(obj, p)
        setattr(obj, parts[-1], value)
    return root


def errors(z, ip, key="errors"):
    keys = z[f"p{ip}_{key}_keys"]
    vals = z[f"p{ip}_{key}_vals"]
    return {int(k): (str(v) if vals.dtype.kind in "US" else float(v)) for k, v in zip(keys, vals)}


def fixture_names():
    return sorted(p.stem for p in GOLDEN_DIR.glob("*.npz")
                  if p.stem not in ("correl_window", "preproc"))
