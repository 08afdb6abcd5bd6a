"""GB300-native (sm_103a) PIV hot path with the fluidimage plugin and WorkPIV API.

* ``WorkPIV``: multipass PIV (window extraction, FFT cross-correlation, peak
  search, '2d_gaussian2' subpixel fit, WorkFIX, thin-plate-spline interpolation)
  with all windows of a pass in one kernel launch.
* ``CorrelGB300`` / ``correlation_classes``: the per-window correlation plugin
  (``params.piv0.method_correl = "gb300"``).
* ``WorkBOS``: background-oriented schlieren (PIV against a reference image kept
  on the GPU).
* ``PIVBatch``: single-pass PIV of many pairs of mixed image and window sizes in a
  few launches (one per window size, blocks fed by a device work queue),
  replayable as a CUDA graph.
* ``params.piv0.method_correl = "gb300_tc_fp16x3"`` (or ``_bf16x3``, ``_bf16x1``):
  32 px passes on the tensor cores (DFT as dense contractions).
* ``WorkPIV(params, deform=True)``: passes after the first on deformed images;
  ``deform``: the differentiable deform-and-correlate chain (hand-written adjoint)
  and its gradient refinement.
* ``preproc.WorkPreproc``: the preprocessing tools on the device.

Importing the package is cheap: the CUDA library is loaded on first use by
``fluidimage_gb300._lib`` and fails loudly when it is missing (no CPU fallback).
"""

__version__ = "0.1.0"

from .correl import CorrelGB300, correlation_classes, register_upstream  # noqa: E402
from .data_objects import ArrayCouple, HeavyPIVResults, MultipassPIVResults  # noqa: E402
from .errors import InterpError, PIVError  # noqa: E402
from .params import ParamContainer  # noqa: E402
from .piv import WorkPIV  # noqa: E402
from .bos import WorkBOS  # noqa: E402
from .batch import PIVBatch  # noqa: E402

__all__ = [
    "WorkPIV", "WorkBOS", "PIVBatch", "CorrelGB300", "correlation_classes", "register_upstream", "ArrayCouple",
    "HeavyPIVResults", "MultipassPIVResults", "PIVError", "InterpError", "ParamContainer",
]
