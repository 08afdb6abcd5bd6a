"""Run the upstream ``WorkPIV`` (the unmodified sources installed in
``baseline/_ref/src`` by ``tests/golden/install_reference.py``) with this package's
correlation plugin, ``params.piv0.method_correl = "gb300"``, on a golden case, and
save every pass's outputs.  Executed in a child process by
``tests/test_gpu_upstream.py`` so that the stand-in modules the upstream import
needs stay out of the test process.

Usage: ``python tests/upstream_run.py <src dir> <golden case> <out.npz>``.
"""

from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE / "golden"))
sys.path.insert(0, str(HERE.parent))

KEYS = ("deltaxs", "deltays", "xs", "ys", "correls_max", "deltaxs_final", "deltays_final")


def main(src, case, out):
    import refharness

    refharness.install(src)
    import fluidimage_gb300

    if not fluidimage_gb300.register_upstream():
        raise SystemExit("register_upstream() found no upstream fluidimage")
    from fluidimage.calcul.correl import correlation_classes
    from fluidimage.works.piv import WorkPIV

    assert correlation_classes["gb300"] is fluidimage_gb300.CorrelGB300
    z = np.load(HERE / "golden" / f"{case}.npz")
    params = WorkPIV.create_default_params()
    for path, value in json.loads(str(z["settings"])).items():
        obj = params
        parts = path.split(".")
        for p in parts[:-1]:
            obj = getattr(obj, p)
        setattr(obj, parts[-1], value)
    params.piv0.method_correl = "gb300"
    work = WorkPIV(params)
    result = work.calcul({"arrays": (z["im0"], z["im1"]), "names": ("im0", "im1")})
    res = {"nb_passes": np.array(len(result.passes)),
           "correl_class": np.array(type(work.works_piv[0].correl).__name__)}
    for ip, r in enumerate(result.passes):
        for key in KEYS:
            if hasattr(r, key):
                res[f"p{ip}_{key}"] = np.asarray(getattr(r, key))
        keys = sorted(int(k) for k in r.errors)
        res[f"p{ip}_errors_keys"] = np.array(keys, dtype=np.int64)
        res[f"p{ip}_errors_vals"] = np.array([str(r.errors[k]) for k in keys], dtype=str)
    np.savez(out, **res)


if __name__ == "__main__":
    if len(sys.argv) != 4:
        raise SystemExit(__doc__)
    main(*sys.argv[1:])
