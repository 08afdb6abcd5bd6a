"""Batched single-pass PIV over many image pairs of mixed sizes on one GPU.

A series of couples is what a PIV topology feeds to its works, one couple per
process in the reference (topologies/piv.py:143-151 with the executors of
executors/multi_exec_async.py:114-158).  Here the couples of a batch, each with its
own image size, dtype, window size (8-64 px), overlap and parameters, run
together:

* the image minima of every pair in one launch (``fi_images_min_batch``);
* per window size present, one launch over the windows of every pair of that
  size, one block per work item, each block taking the next item from a device
  counter, largest windows first (``fi_piv_pass_batch``): the per-window
  computation of ``fi_piv_pass`` (works/piv/singlepass.py:262-361 per pair);
* WorkFIX (works/piv/fix.py:66-133) of every pair in two launches
  (``fi_fix_batch``).

The launches of a run contain no host synchronisation, so a run can be captured in
a CUDA graph and replayed (``capture``; ``run`` then replays it).  The windows per
work item (the block shape and its register budget) of each window size are picked
by ``autotune`` (CUDA-event timing of the candidates on the batch itself).

Each job is one pass of ``WorkPIV`` (``params.multipass.number == 1``) without the
final interpolation; results equal ``WorkPIV(params, interp_last=False).calcul``.
"""

from __future__ import annotations

from dataclasses import dataclass
from typing import List, Sequence

import numpy as np

from . import _lib as L
from .engine import PIVPipeline, _DTYPES
from .errors import GridError

#: autotuner choices, kept per (window size, log2 of the windows of that size)
_TUNED = {}


@dataclass
class _Job:
    params: object
    im0: object
    im1: object
    pipe: PIVPipeline
    out: object = None      # PassDevice
    args: object = None     # fi_piv_pass_args
    fix: object = None      # fi_fix_args


def _to_dev(a, dev):
    import torch

    from .piv import _to_device

    return a.to(dev).contiguous() if isinstance(a, torch.Tensor) else _to_device(a, dev)


class PIVBatch:
    """Single-pass PIV of ``jobs`` = [(im0, im1, params), ...] (host arrays or device
    tensors: uint8, uint16 as int16 storage, float32)."""

    def __init__(self, jobs: Sequence, device=None):
        import torch

        from .piv import _np_dtype

        self.device = torch.device(device if device is not None else "cuda")
        dev = self.device
        lib = L.load()
        self.jobs: List[_Job] = []
        pipes = {}
        for im0, im1, params in jobs:
            if params.multipass.number != 1:
                raise ValueError("PIVBatch runs single-pass works (params.multipass.number == 1)")
            if int(params.piv0.nb_peaks_to_search) != 1:
                raise NotImplementedError("PIVBatch: nb_peaks_to_search must be 1")
            if params.piv0.method_correl not in ("gb300", "np.fft", "fftw"):
                raise NotImplementedError(
                    "PIVBatch runs the FP32 FFT correlation (method_correl 'gb300', "
                    f"'np.fft' or 'fftw'), not {params.piv0.method_correl!r}")
            n = int(params.piv0.shape_crop_im0) if not isinstance(
                params.piv0.shape_crop_im0, (list, tuple)) else -1
            if n not in L.BATCH_WPB:
                raise NotImplementedError(
                    f"PIVBatch: windows of {params.piv0.shape_crop_im0} px (batched sizes: "
                    f"{sorted(L.BATCH_WPB)})")
            t0, t1 = _to_dev(im0, dev), _to_dev(im1, dev)
            key = (id(params), tuple(t0.shape), _np_dtype(t0))
            if key not in pipes:
                pipes[key] = PIVPipeline(params, tuple(t0.shape), _np_dtype(t0), device=dev,
                                         interp_last=False)
            self.jobs.append(_Job(params, t0, t1, pipes[key]))
        n_jobs = len(self.jobs)
        if n_jobs == 0:
            raise ValueError("empty batch")
        self.im_min = torch.empty((n_jobs, 2), dtype=torch.float32, device=dev)
        self.min_keys = torch.empty(2 * n_jobs, dtype=torch.int32, device=dev)
        for k, job in enumerate(self.jobs):
            lay = job.pipe.layouts[0]
            if (job.params.fix.threshold_diff_neighbour is not None
                    and (lay.ixvecs.size < 2 or lay.iyvecs.size < 2)):
                raise GridError(f"job {k}: WorkFIX's neighbour test needs a vector grid of at "
                                f"least 2 x 2 (this one is {lay.iyvecs.size} x {lay.ixvecs.size})")
            job.out, job.args = job.pipe.make_pass(lay, job.im0, job.im1, self.im_min[k],
                                                   None, None, _DTYPES[job.pipe.dtype])
            job.fix = job.pipe.make_fix(job.out, job.params.fix)
        # passes grouped by window size, the largest windows (longest items) launched
        # first, each group's passes by decreasing number of windows
        self.groups = {}
        for k, job in enumerate(self.jobs):
            self.groups.setdefault(job.pipe.layouts[0].n, []).append(k)
        for n in self.groups:
            self.groups[n].sort(key=lambda k: -self.jobs[k].pipe.layouts[0].nvec)
        self.order = sorted(self.groups, reverse=True)
        self.all_args = self._device_array([j.args for j in self.jobs], L.PivPassArgs)
        self.group_args = {n: self._device_array([self.jobs[k].args for k in ks], L.PivPassArgs)
                           for n, ks in self.groups.items()}
        self.counters = torch.zeros(len(self.groups), dtype=torch.int32, device=dev)
        self.fix_args = self._device_array([j.fix for j in self.jobs], L.FixArgs)
        nv = np.array([j.pipe.layouts[0].nvec for j in self.jobs], dtype=np.int64)
        starts = np.concatenate([[0], np.cumsum(nv)])
        if starts[-1] >= 2**31:
            raise ValueError("too many vectors in one batch")
        self.vec_start = torch.as_tensor(starts.astype(np.int32), device=dev)
        self.total_vectors = int(starts[-1])
        self.config = {}
        for n in self.groups:
            self._set_config(n, L.BATCH_WPB[n][0])
        self.graph = None

    # ------------------------------------------------------------------------------
    def _device_array(self, structs, cls):
        import torch

        arr = (cls * len(structs))(*structs)
        return torch.frombuffer(bytearray(bytes(arr)), dtype=torch.uint8).to(self.device)

    def _set_config(self, n, wpb):
        import torch

        lib = L.load()
        items = [lib.fi_piv_batch_items(n, self.jobs[k].pipe.layouts[0].nvec, wpb)
                 for k in self.groups[n]]
        starts = np.concatenate([[0], np.cumsum(items)]).astype(np.int32)
        self.config[n] = {"wpb": wpb, "item_start": torch.as_tensor(starts, device=self.device),
                          "items": int(starts[-1]),
                          "resident_blocks": int(lib.fi_piv_batch_max_blocks(n, wpb))}

    def _launch_group(self, gi, n, s):
        lib = L.load()
        cfg = self.config[n]
        L.check(lib.fi_piv_pass_batch(L.ptr(self.group_args[n]), L.ptr(cfg["item_start"]),
                                      len(self.groups[n]), n, cfg["wpb"], cfg["items"],
                                      L.ptr(self.counters[gi:gi + 1]), s), "fi_piv_pass_batch")

    def launches(self, stream=None):
        """Issue one run on ``stream`` (no host synchronisation): minima, one batch
        launch per window size, WorkFIX."""
        lib = L.load()
        s = L.stream_handle(stream)
        L.check(lib.fi_images_min_batch(L.ptr(self.all_args), len(self.jobs),
                                        L.ptr(self.min_keys), s), "fi_images_min_batch")
        for gi, n in enumerate(self.order):
            self._launch_group(gi, n, s)
        L.check(lib.fi_fix_batch(L.ptr(self.fix_args), L.ptr(self.vec_start), len(self.jobs),
                                 self.total_vectors, s), "fi_fix_batch")

    def run(self, stream=None):
        """One run: the captured graph when there is one, else the launches."""
        if self.graph is not None:
            self.graph.replay()
        else:
            self.launches(stream)

    def capture(self):
        """Capture a run in a CUDA graph; ``run`` then replays it."""
        import torch

        self.launches()  # first use: kernel attributes set outside the capture
        torch.cuda.synchronize()
        graph = torch.cuda.CUDAGraph()
        stream = torch.cuda.Stream(device=self.device)
        with torch.cuda.stream(stream):
            with torch.cuda.graph(graph, stream=stream):
                self.launches(stream)
        torch.cuda.synchronize()
        self.graph = graph
        return graph

    def autotune(self, reps=2):
        """Per window size, time the batch launch over its pairs for each windows-per-
        item candidate and keep the fastest; choices are cached per (window size,
        log2 of its windows)."""
        import torch

        choice = {}
        for gi, n in enumerate(self.order):
            nwin = sum(self.jobs[k].pipe.layouts[0].nvec for k in self.groups[n])
            key = (n, int(np.log2(max(nwin, 1))))
            if key in _TUNED:
                self._set_config(n, _TUNED[key])
                choice[n] = {"wpb": _TUNED[key], "cached": True}
                continue
            best = None
            for wpb in L.BATCH_WPB[n]:
                self._set_config(n, wpb)
                times = []
                for _ in range(reps + 1):
                    e0 = torch.cuda.Event(enable_timing=True)
                    e1 = torch.cuda.Event(enable_timing=True)
                    e0.record()
                    self._launch_group(gi, n, L.stream_handle())
                    e1.record()
                    torch.cuda.synchronize()
                    times.append(e0.elapsed_time(e1))
                ms = min(times[1:])
                if best is None or ms < best[0]:
                    best = (ms, wpb)
            ms, wpb = best
            _TUNED[key] = wpb
            self._set_config(n, wpb)
            choice[n] = {"wpb": wpb, "ms": ms, "cached": False,
                         "resident_blocks": self.config[n]["resident_blocks"]}
        self.graph = None  # a captured graph holds the old configuration
        return choice

    # ------------------------------------------------------------------------------
    def results(self):
        """Host ``HeavyPIVResults`` of every job, in job order."""
        from .piv import WorkPIV, _fetch

        works = [WorkPIV(j.params, device=self.device, interp_last=False) for j in self.jobs]
        wants = [w._device_results([j.out]) for w, j in zip(works, self.jobs)]
        got = iter(_fetch([t for want in wants for t in want.values()]))
        out = []
        for w, want, job in zip(works, wants, self.jobs):
            vals = {k: next(got) for k in want}
            out.append(w._host_results([job.out], None, vals).passes[0])
        return out
