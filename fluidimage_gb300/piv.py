"""``WorkPIV``: multipass PIV on one GB300, with the upstream work API.

Mirrors ``fluidimage.works.piv.WorkPIV`` (works/piv/multipass.py:17-190),
``FirstWorkPIV`` / ``WorkPIVFromDisplacement`` (works/piv/singlepass.py:566-870)
and ``WorkFIX`` (works/piv/fix.py:21-243): same parameter tree
(``create_default_params``), same ``calcul(couple)`` / ``calcul_from_arrays``
entry points, same ``MultipassPIVResults`` / ``HeavyPIVResults`` attributes.
All windows of a pass are processed by one kernel launch; the passes, the
false-vector removal and the TPS interpolation run on the GPU.
"""

from __future__ import annotations

import threading
import time

import numpy as np

from . import _lib
from .data_objects import ArrayCouple, HeavyPIVResults, MultipassPIVResults
from .engine import GridOutput, PIVPipeline, error_dict
from .errors import InterpError
from .params import ParamContainer

#: correlation tags computed by this backend (FFT cross-correlation semantics of
#: CorrelFFTNumpy / CorrelFFTW, calcul/correl.py:639-692): the FP32 FFT pass, and the
#: tensor-core DFT pass in one of its precision forms (32 px passes; passes of other
#: window sizes run the FP32 FFT pass)
TC_TAGS = {"gb300_tc_bf16x1": "bf16x1", "gb300_tc_bf16x3": "bf16x3",
           "gb300_tc_fp16x3": "fp16x3"}
FFT_TAGS = ("gb300", "np.fft", "fftw") + tuple(TC_TAGS)


def _complete_params_piv0(params):
    params._set_child("piv0", attribs={
        "shape_crop_im0": 48,
        "shape_crop_im1": None,
        "displacement_max": None,
        "displacement_mean": None,
        "method_correl": "gb300",
        "method_subpix": "2d_gaussian2",
        "nsubpix": None,
        "nb_peaks_to_search": 1,
        "particle_radius": 3,
    })
    params.piv0._set_child("grid", attribs={"overlap": 0.5, "from": "overlap"})
    params._set_child("mask", attribs={"strcrop": None})


def _complete_params_fix(params, tag="fix"):
    params._set_child(tag, attribs={
        "correl_min": 0.2,
        "threshold_diff_neighbour": 10,
        "displacement_max": None,
    })


def _complete_params_multipass(params):
    params._set_child("multipass", attribs={
        "number": 1,
        "coeff_zoom": 2,
        "use_tps": "last",
        "subdom_size": 200,
        "smoothing_coef": 5.0,
        "threshold_tps": 1.5,
    })


def _complete_params_series(params):
    params._set_child("series", attribs={
        "path": "",
        "str_subset": "pairs",
        "ind_start": "first",
        "ind_stop": None,
        "ind_step": 1,
    })


class LazyWeights:
    """Per-subdomain TPS weights (``deltaxs_tps``), copied to the host on first use."""

    def __init__(self, tps, comp):
        self._tps = tps
        self._comp = comp
        self._items = None

    def _load(self):
        if self._items is None:
            w = self._tps.weights.cpu().numpy()
            items = []
            for i, cnt in enumerate(self._tps.counts):
                n = int(cnt) + 3
                o = int(self._tps.w_offsets[i]) + self._comp * n
                items.append(w[o:o + n].copy())
            self._items = items
        return self._items

    def __len__(self):
        return self._tps.nb_subdom

    def __getitem__(self, i):
        return self._load()[i]

    def __iter__(self):
        return iter(self._load())


class WorkPIV:
    """Multipass PIV work (works/piv/multipass.py:17-190) on the GPU.

    Parameters
    ----------
    params : ParamContainer from :meth:`create_default_params`.
    keep_correls : store the correlation planes in ``HeavyPIVResults.correls``
        (upstream always stores them; here they cost a device-to-host copy).
    device : torch device (default ``cuda``).
    interp_last : compute the final interpolation (``deltaxs_final``...): TPS for
        ``use_tps`` True or ``'last'``, griddata for ``use_tps=False``, as upstream.
    deform : passes after the first deform im1 by the interpolated field of the
        previous pass (bilinear, ``fluidimage_gb300.deform.warp``) and measure the
        residual at unshifted windows, instead of shifting the windows by the
        rounded field (the reference's method; its to-do at singlepass.py:736-738).
    """

    @classmethod
    def _complete_params_with_default(cls, params):
        """Add this work's parameters to ``params`` (multipass.py:47-105): what a PIV
        topology calls on its ``WorkVelocimetry`` class (topologies/piv.py:58-76)."""
        _complete_params_series(params)
        _complete_params_piv0(params)
        _complete_params_fix(params)
        _complete_params_multipass(params)

    @classmethod
    def create_default_params(cls):
        params = ParamContainer(tag="params")
        cls._complete_params_with_default(params)
        return params

    def __init__(self, params=None, keep_correls=False, device=None, verbose=False,
                 interp_last=True, deform=False):
        if params is None:
            params = self.create_default_params()
        self.params = params
        if params.piv0.method_correl not in FFT_TAGS:
            from .correl import correlation_classes

            raise ValueError(
                "params.piv0.method_correl should be in " + str(list(correlation_classes))
            )
        if params.piv0.grid.overlap >= 1:
            raise ValueError("params.piv0.grid.overlap has to be smaller than 1")
        self.keep_correls = keep_correls
        self.interp_last = interp_last
        self.deform = deform
        self.device = device
        self.verbose = verbose
        # nothing here touches CUDA: a topology builds its works in the parent process
        # and a multi-process executor forks its workers afterwards (each worker then
        # makes its own CUDA context on its first couple)
        self._pipelines = {}
        self._lock = threading.Lock()

    def __getstate__(self):
        # pickled works (spawned workers) rebuild their pipelines on first use
        state = self.__dict__.copy()
        state["_pipelines"] = {}
        del state["_lock"]
        return state

    def __setstate__(self, state):
        self.__dict__.update(state)
        self._lock = threading.Lock()

    # --------------------------------------------------------------------
    def _pipeline(self, imshape, dtype):
        key = (tuple(imshape), np.dtype(dtype).str)
        with self._lock:
            if key not in self._pipelines:
                self._pipelines[key] = PIVPipeline(
                    self.params, imshape, dtype, device=self.device,
                    keep_correls=self.keep_correls, interp_last=self.interp_last,
                    deform=self.deform)
            return self._pipelines[key]

    def _xy_offsets(self):
        strcrop = self.params.mask.strcrop
        if strcrop is None:
            return 0, 0
        from .data_objects import get_slices_from_strcrop

        sl = get_slices_from_strcrop(strcrop)
        return (sl[1].start or 0), (sl[0].start or 0)

    def calcul_device(self, im0, im1, stream=None):
        """Run the passes on device images (torch tensors); returns device outputs."""
        pipe = self._pipeline(tuple(im0.shape), _np_dtype(im0))
        return pipe.run(im0, im1, stream=stream)

    def calcul(self, couple):
        """Compute a multipass PIV field from a couple of images.

        Several host threads may call it at once (a topology's thread executors run
        the "compute piv" work that way, topologies/piv.py:143-149): each thread runs
        its couples on a CUDA stream of its own, so their kernels overlap."""
        import torch

        couple = _as_couple(couple)
        couple.apply_mask(self.params.mask)
        im0, im1 = couple.get_arrays()
        dev = _cuda_device(self.device)
        stream = _thread_stream(dev)
        with torch.cuda.stream(stream):
            t0 = _to_device(im0, dev)
            t1 = _to_device(im1, dev)
            outs = self.calcul_device(t0, t1, stream=stream)
            return self.results_to_host(outs, couple)

    def calcul_from_arrays(self, *arrays, names=None):
        names = [f"array{i}" for i in range(len(arrays))]
        t_start = time.perf_counter()
        result = self.calcul({"arrays": arrays, "names": names})
        if self.verbose:
            print(f"Calcul done in {time.perf_counter() - t_start:.2f} s")
        return result

    # --------------------------------------------------------------------
    def results_to_host(self, outs, couple=None):
        """Device outputs -> ``MultipassPIVResults`` (upstream attributes and dtypes).

        Every array is gathered into one device buffer and copied to pinned host
        memory at once (one synchronisation)."""
        want = self._device_results(outs)
        handle = _fetch_start(list(want.values()))
        return self._host_results(outs, couple, dict(zip(want, _fetch_finish(handle))))

    def calcul_series(self, couples, streams=2):
        """Results of a series of couples, in order (a generator).  ``streams`` couples
        are in flight at once, each on its own host thread and CUDA stream: the GPU
        works on one couple's kernels while another couple's host-side steps (the TPS
        readbacks, the results) run, the role of the executors of a PIV topology
        (topologies/piv.py:143-151) for this work.
        """
        import collections

        import torch
        from concurrent.futures import ThreadPoolExecutor

        dev = _cuda_device(self.device)
        local = threading.local()

        def run(couple):
            if getattr(local, "stream", None) is None:
                local.stream = torch.cuda.Stream(device=dev)
            with torch.cuda.stream(local.stream):
                im0, im1 = couple.get_arrays()
                outs = self.calcul_device(_to_device(im0, dev), _to_device(im1, dev),
                                          stream=local.stream)
                want = self._device_results(outs)
                handle = _fetch_start(list(want.values()))
                return self._host_results(outs, couple, dict(zip(want, _fetch_finish(handle))))

        nstreams = max(1, int(streams))
        pending = collections.deque()
        with ThreadPoolExecutor(max_workers=nstreams) as pool:
            for couple in couples:
                couple = _as_couple(couple)
                couple.apply_mask(self.params.mask)
                im0, _ = couple.get_arrays()
                self._pipeline(tuple(im0.shape), _host_dtype(im0))  # built here, once
                if len(pending) >= nstreams:
                    yield pending.popleft().result()
                pending.append(pool.submit(run, couple))
            while pending:
                yield pending.popleft().result()

    def _device_results(self, outs):
        """The device tensors the host results are built from (keyed by pass and
        name); the *_smooth fields are assembled on the device here."""
        offx, offy = self._xy_offsets()
        keys = ("deltaxs_raw", "deltays_raw", "correls_max", "errors", "xs", "ys", "flags",
                "deltaxs", "deltays", "fix_flags", "diff2")
        want = {}
        for k, pd in enumerate(outs):
            for key in keys:
                want[(k, key)] = getattr(pd, key)
            if pd.planes is not None:
                want[(k, "planes")] = pd.planes
            if pd.tc_status is not None:
                want[(k, "tc_status")] = pd.tc_status
            if pd.dxin is not None:
                want[(k, "dxin")], want[(k, "dyin")] = pd.dxin, pd.dyin
            if pd.peaks_count is not None:
                want[(k, "peaks_count")], want[(k, "peaks")] = pd.peaks_count, pd.peaks
                want[(k, "replaced")] = pd.replaced
            for tag in ("tps_next", "tps_final"):
                tps = getattr(pd, tag)
                if tps is None:
                    continue
                want[(k, tag, "out_x")], want[(k, tag, "out_y")] = tps.out_x, tps.out_y
                if isinstance(tps, GridOutput):
                    want[(k, tag, "flags")] = tps.flags
                    continue
                want[(k, tag, "singular")] = tps.singular
                if tag == "tps_final":
                    # the *_smooth fields (singlepass.py:515-529): the grid with the
                    # selected vectors' values scattered in, built on the device
                    import torch

                    lay = pd.layout
                    npts = lay.nvec
                    xs_s = torch.empty(npts, dtype=torch.float32, device=tps.out_x.device)
                    ys_s = torch.empty_like(xs_s)
                    dx_s = torch.empty_like(tps.out_x)
                    dy_s = torch.empty_like(tps.out_y)
                    _lib.check(_lib.load().fi_tps_smooth_fields(
                        _lib.ptr(lay.dev["px"]), _lib.ptr(lay.dev["py"]), npts, _lib.ptr(pd.xs),
                        _lib.ptr(pd.ys), int(lay.index != 0), float(offx), float(offy),
                        _lib.ptr(tps.selection), int(tps.num_centers), _lib.ptr(tps.out_x),
                        _lib.ptr(tps.out_y), _lib.ptr(tps.smooth_x), _lib.ptr(tps.smooth_y),
                        _lib.ptr(xs_s), _lib.ptr(ys_s), _lib.ptr(dx_s), _lib.ptr(dy_s),
                        _lib.stream_handle()), "fi_tps_smooth_fields")
                    want[(k, tag, "xs_smooth")], want[(k, tag, "ys_smooth")] = xs_s, ys_s
                    want[(k, tag, "dx_smooth")], want[(k, tag, "dy_smooth")] = dx_s, dy_s
        return want

    def _host_results(self, outs, couple, got):
        """``MultipassPIVResults`` from the host copies ``got`` of ``_device_results``."""
        fx = self.params.fix
        offx, offy = self._xy_offsets()
        keys = ("deltaxs_raw", "deltays_raw", "correls_max", "errors", "xs", "ys", "flags",
                "deltaxs", "deltays", "fix_flags", "diff2")
        results = MultipassPIVResults()
        hosts = []
        for k, pd in enumerate(outs):
            lay = pd.layout
            if pd.tc_status is not None and int(got[(k, "tc_status")][0]) != 0:
                raise RuntimeError("tensor-core PIV pass: a wait on the tensor cores timed out")
            h = {key: got[(k, key)] for key in keys}
            errors = error_dict(h["errors"], h["fix_flags"], h["diff2"],
                                fx.threshold_diff_neighbour)
            secondary = [None] * lay.nvec
            replaced = {}
            if pd.peaks_count is not None:
                secondary = _secondary_peaks(got[(k, "peaks_count")], got[(k, "peaks")],
                                             lay.nvec)
                old = got[(k, "replaced")].reshape(lay.nvec, 3)
                for i in np.nonzero(h["fix_flags"] & _lib.FIX_REPLACED)[0].tolist():
                    replaced[i] = tuple(old[i])
            if lay.index == 0:
                xs = lay.gx + offx
                ys = lay.gy + offy
            else:
                xs = h["xs"].astype(np.float64) + offx
                ys = h["ys"].astype(np.float64) + offy
            nvec = lay.nvec
            if pd.planes is not None:
                planes = got[(k, "planes")].reshape(nvec, lay.n, lay.n)
                correls = [None if h["errors"][i] == 4 else planes[i] for i in range(nvec)]
            else:
                correls = [None] * nvec
            r = HeavyPIVResults(
                h["deltaxs"], h["deltays"], xs, ys, errors, correls_max=h["correls_max"],
                correls=correls, couple=couple, params=self.params,
                secondary_peaks=secondary,
            )
            if replaced:
                r.replaced_vectors = replaced
            r.indices_no_displacement = (lay.n // 2 - 1, lay.n // 2 - 1)
            r.displacement_max = lay.displacement_max
            # per-vector near-tie flags (bit 0: top-two plane values within 1e-6
            # relative; bit 1: tied minimum in the subpixel crop; bit 2: near-tie in a
            # secondary search); on these vectors the upstream result depends on float
            # rounding
            r.near_tie_flags = h["flags"]
            r.near_ties = int(np.count_nonzero(h["flags"]))
            if fx.threshold_diff_neighbour is not None:
                ierr = np.fromiter(errors, dtype=np.int64, count=len(errors))
                r.deltaxs_wrong = dict(zip(errors, h["deltaxs_raw"][ierr]))
                r.deltays_wrong = dict(zip(errors, h["deltays_raw"][ierr]))
            if pd.dxin is not None:
                r.deltaxs_input = got[(k, "dxin")]
                r.deltays_input = got[(k, "dyin")]
            hosts.append((r, h))
            results.append(r)
        for k, pd in enumerate(outs):
            r, h = hosts[k]
            if pd.tps_next is not None:
                nxt = outs[k + 1].layout
                r.deltaxs_approx = got[(k, "tps_next", "out_x")]
                r.deltays_approx = got[(k, "tps_next", "out_y")]
                r.ixvecs_approx = nxt.gx + offx
                r.iyvecs_approx = nxt.gy + offy
                if isinstance(pd.tps_next, GridOutput):
                    # cocircular cells / equidistant nearest vectors (several valid
                    # triangulations: upstream's result there depends on Qhull)
                    r.griddata_tie_flags_approx = got[(k, "tps_next", "flags")]
                else:
                    self._check_tps(got[(k, "tps_next", "singular")])
                    r.deltaxs_tps = LazyWeights(pd.tps_next, 0)
                    r.deltays_tps = LazyWeights(pd.tps_next, 1)
            if pd.tps_final is not None:
                tps = pd.tps_final
                lay = pd.layout
                r.ixvecs_final = lay.gx + offx
                r.iyvecs_final = lay.gy + offy
                r.deltaxs_final = got[(k, "tps_final", "out_x")]
                r.deltays_final = got[(k, "tps_final", "out_y")]
                if isinstance(tps, GridOutput):
                    r.griddata_tie_flags_final = got[(k, "tps_final", "flags")]
                    continue
                self._check_tps(got[(k, "tps_final", "singular")])
                r.xs_smooth = got[(k, "tps_final", "xs_smooth")]
                r.ys_smooth = got[(k, "tps_final", "ys_smooth")]
                r.deltaxs_smooth = got[(k, "tps_final", "dx_smooth")]
                r.deltays_smooth = got[(k, "tps_final", "dy_smooth")]
                r.deltaxs_tps = LazyWeights(tps, 0)
                r.deltays_tps = LazyWeights(tps, 1)
        return results

    @staticmethod
    def _check_tps(singular):
        if int(np.asarray(singular).sum()) != 0:
            raise np.linalg.LinAlgError(
                "Singular TPS subdomain system (upstream then falls back to griddata)"
            )


def _fetch_start(tensors):
    """Start the copy of device tensors to the host: the tensors are packed into one
    device byte buffer (widest elements first, so every array stays aligned) and
    copied asynchronously to pinned host memory; ``_fetch_finish`` waits for it."""
    import torch

    order = sorted(range(len(tensors)), key=lambda i: -tensors[i].element_size())
    flat = [tensors[i].contiguous().view(-1).view(torch.uint8) for i in order]
    if not flat:
        return None
    buf = torch.cat(flat) if len(flat) > 1 else flat[0]
    host = torch.empty(buf.numel(), dtype=torch.uint8, pin_memory=True)
    host.copy_(buf, non_blocking=True)
    done = torch.cuda.Event()
    done.record()
    meta = [(tuple(t.shape), t.dtype) for t in tensors]
    return host, done, order, [f.numel() for f in flat], meta


def _fetch_finish(handle):
    """numpy views (one per tensor given to ``_fetch_start``) of the pinned buffer,
    once its copy is complete."""
    import torch

    if handle is None:
        return []
    host, done, order, sizes, meta = handle
    done.synchronize()
    np_of = {torch.float64: np.float64, torch.float32: np.float32, torch.int32: np.int32,
             torch.int64: np.int64, torch.uint8: np.uint8, torch.int16: np.int16}
    raw = host.numpy()
    out = [None] * len(meta)
    off = 0
    for i, n in zip(order, sizes):
        shape, dtype = meta[i]
        out[i] = raw[off:off + n].view(np_of[dtype]).reshape(shape)
        off += n
    return out


def _fetch(tensors):
    """Device tensors -> numpy arrays with one copy (views of one pinned buffer)."""
    return _fetch_finish(_fetch_start(tensors))


def _secondary_peaks(counts, peaks, nvec):
    """``secondary_peaks`` of _loop_vectors: None where the peak search raised, else
    the list of (dx, dy, correl_max) of the other peaks (correl.py:250-273)."""
    K = peaks.size // (nvec * _lib.PEAK_FIELDS)
    pk = peaks.reshape(nvec, K, _lib.PEAK_FIELDS)
    out = [None] * nvec
    for i in range(nvec):
        c = int(counts[i])
        if c >= 0:
            out[i] = [(int(pk[i, j, 0]), int(pk[i, j, 1]), pk[i, j, 2]) for j in range(c)]
    return out


def _host_dtype(a):
    """Image element type of a host image (numpy array or torch tensor)."""
    import torch

    return _np_dtype(a) if isinstance(a, torch.Tensor) else np.asarray(a).dtype


def _np_dtype(t):
    """Image element type of a device tensor; uint16 images travel as int16 storage."""
    import torch

    return {torch.uint8: np.uint8, torch.int16: np.uint16, torch.float32: np.float32}[t.dtype]


_THREAD = threading.local()


def _as_couple(couple):
    """A couple of arrays: this package's ``ArrayCouple``, one built from a dict of
    its arguments, or a couple object of an installed fluidimage (what the couples
    queue of its PIV topology holds, topologies/piv.py:203-226: any object with
    ``get_arrays`` and ``apply_mask``)."""
    if isinstance(couple, dict):
        couple = ArrayCouple(**couple)
    if not isinstance(couple, ArrayCouple) and not (
            hasattr(couple, "get_arrays") and hasattr(couple, "apply_mask")):
        raise ValueError(f"not isinstance(couple, ArrayCouple), {type(couple) = }")
    return couple


def _cuda_device(device):
    """The torch device of a work; refuses to start CUDA in a process forked from one
    that had already started it (a forked child cannot use its parent's context)."""
    import torch

    in_bad_fork = getattr(torch.cuda, "_is_in_bad_fork", lambda: False)
    if in_bad_fork():
        raise RuntimeError(
            "CUDA was initialised in the parent of this forked process: create the "
            "work in the parent but run it only in the workers (the work itself "
            "initialises nothing before its first couple), or start the workers "
            "with 'spawn'")
    return torch.device(device or "cuda")


def _thread_stream(dev):
    """The CUDA stream of the calling host thread on ``dev`` (made on first use)."""
    import torch

    streams = getattr(_THREAD, "streams", None)
    if streams is None:
        streams = _THREAD.streams = {}
    key = (dev.type, dev.index if dev.index is not None else torch.cuda.current_device())
    if key not in streams:
        streams[key] = torch.cuda.Stream(device=dev)
    return streams[key]


def _to_device(a, dev):
    """Host image -> device tensor (uint16 data kept bit for bit in an int16 tensor)."""
    import torch

    if isinstance(a, torch.Tensor):
        return a.to(dev).contiguous()
    a = np.ascontiguousarray(a)
    if a.dtype == np.uint16:
        a = a.view(np.int16)
    elif a.dtype not in (np.uint8, np.float32):
        raise TypeError(f"image dtype {a.dtype} not supported (uint8, uint16, float32)")
    return torch.from_numpy(a).to(dev)
