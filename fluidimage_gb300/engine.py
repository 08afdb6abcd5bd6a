"""Device pipeline of the multipass PIV (one image pair at a time, one GPU).

``PIVPipeline`` holds everything that depends only on the parameters and the
image shape (window grids, displacement_max masks, device buffers) and runs the
passes of ``WorkPIV.calcul`` (works/piv/multipass.py:172-190) on device:

    pass 0        fi_piv_pass (grid windows)            -> fi_fix
    pass k >= 1   TPS(previous pass -> this grid)       -> fi_piv_pass (shifted) -> fi_fix
    final         TPS(last pass -> its own grid)

Only the window grid and the masks are computed on the host (they depend on
the parameters, not on the images).  The TPS stages read back a few integers
(number of valid vectors, subdomain populations) to size their buffers.
"""

from __future__ import annotations

import ctypes as C
import math
import threading
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

from . import _lib as L
from .errors import ERROR_STRINGS, GridError, InterpError  # noqa: F401  (ERROR_STRINGS re-exported)

_DTYPES = {np.dtype(np.uint8): L.FI_U8, np.dtype(np.uint16): L.FI_U16,
           np.dtype(np.float32): L.FI_F32}

SUPPORTED_WINDOWS = (8, 12, 16, 24, 32, 48, 64)


def _torch():
    import torch

    return torch


class KernelTimer:
    """CUDA-event timing of each library entry point on the launching stream."""

    def __init__(self):
        self.events = {}

    def record(self, name):
        torch = _torch()
        start = torch.cuda.Event(enable_timing=True)
        end = torch.cuda.Event(enable_timing=True)
        start.record()
        self.events.setdefault(name, []).append((start, end))
        return end

    def summary(self):
        torch = _torch()
        torch.cuda.synchronize()
        out = {}
        for name, pairs in self.events.items():
            ms = [a.elapsed_time(b) for a, b in pairs]
            out[name] = {"launches": len(ms), "total_ms": float(sum(ms)),
                         "avg_ms": float(sum(ms) / len(ms))}
        return out


#: set to a KernelTimer to time every library call (benchmark instrumentation)
TIMER = None


class _timed:
    def __init__(self, name):
        self.name = name
        self.end = None

    def __enter__(self):
        if TIMER is not None:
            self.end = TIMER.record(self.name)
        return self

    def __exit__(self, *exc):
        if self.end is not None:
            self.end.record()
        return False


# --------------------------------------------------------------------------------
# host-side layout (parameters only): works/piv/singlepass.py:108-141, 363-389
# --------------------------------------------------------------------------------
def crop_start_stop(shape_crop):
    n0, n1 = shape_crop
    return (n0 // 2, n1 // 2), (n0 // 2 + n0 % 2, n1 // 2 + n1 % 2)


def make_grid(imshape, shape_crop, overlap):
    """Window-centre vectors ``ixvecs, iyvecs`` (singlepass.py:108-141)."""
    len_y, len_x = imshape
    start, stop = crop_start_stop(shape_crop)
    stepy = shape_crop[0] - int(np.round(overlap * shape_crop[0]))
    stepx = shape_crop[1] - int(np.round(overlap * shape_crop[1]))
    if stepy < 1 or stepx < 1:
        raise ValueError("overlap too large for the window size")
    ixvec_max = len_x - stop[1]
    ixvecs = np.arange(start[1], ixvec_max, stepx, dtype=int)
    iyvec_max = len_y - stop[0]
    iyvecs = np.arange(start[0], iyvec_max, stepy, dtype=int)
    if ixvecs.size == 0 or iyvecs.size == 0:
        raise GridError("image smaller than the interrogation window")
    if ixvec_max - ixvecs[-1] > stepx // 2.5:
        ixvecs = np.append(ixvecs, ixvec_max)
    if iyvec_max - iyvecs[-1] > stepy // 2.5:
        iyvecs = np.append(iyvecs, iyvec_max)
    return ixvecs, iyvecs


def parse_displacement_max(displ_max, shape):
    if isinstance(displ_max, str) and displ_max.endswith("%"):
        return float(displ_max[:-1]) / 100 * max(shape)
    return displ_max


def displacement_mask(n, displacement_max):
    """``where_large_displacement`` and search box (calcul/correl.py:518-547)."""
    if displacement_max is None:
        return None, (0, n, 0, n)
    ix0 = iy0 = n // 2 - 1
    mask = np.zeros((n, n), dtype=bool)
    for i0 in range(n):
        for i1 in range(n):
            dx, dy = ix0 - i1, iy0 - i0
            mask[i0, i1] = math.sqrt(dx**2 + dy**2) > displacement_max
    rows = ~mask.all(axis=1)
    cols = ~mask.all(axis=0)
    i0s = int(np.argmax(rows)) if rows.any() else n - 1
    i1s = int(np.argmax(cols)) if cols.any() else n - 1
    i0e = int(n - np.argmax(rows[::-1])) if rows.any() else 1
    i1e = int(n - np.argmax(cols[::-1])) if cols.any() else 1
    return mask, (i0s, i0e, i1s, i1e)


def pass_shapes(shape_crop_im0, number, coeff_zoom):
    """Window shape per pass (works/piv/multipass.py:120-165)."""
    if isinstance(shape_crop_im0, (int, np.integer)):
        shape = (int(shape_crop_im0), int(shape_crop_im0))
    elif isinstance(shape_crop_im0, (tuple, list)) and len(shape_crop_im0) == 2:
        shape = tuple(shape_crop_im0)
    else:
        raise NotImplementedError("For now, shape_crop_im0 has to be one or two integer!")
    if isinstance(coeff_zoom, int):
        coeffs = [coeff_zoom] * (number - 1)
    elif len(coeff_zoom) == number - 1:
        coeffs = list(coeff_zoom)
    else:
        raise ValueError(
            "params.multipass.coeff_zoom has to be an integer or "
            "an iterable of length params.multipass.number - 1"
        )
    shapes = [tuple(int(s) for s in shape)]
    for i in range(1, number):
        shape = (shape[0] / coeffs[i - 1], shape[1] / coeffs[i - 1])
        shapes.append(tuple(int(s) for s in shape))
    return shapes


@dataclass
class PassLayout:
    index: int
    n: int
    ixvecs: np.ndarray
    iyvecs: np.ndarray
    gx: np.ndarray
    gy: np.ndarray
    displacement_max: Optional[float]
    mask: Optional[np.ndarray]
    box: tuple
    apply_subpix: bool
    dev: dict = field(default_factory=dict)

    @property
    def nvec(self):
        return self.gx.size


# --------------------------------------------------------------------------------
# TPS driver (device)
# --------------------------------------------------------------------------------
@dataclass
class TpsOutput:
    out_x: object  # float64 [npts] device
    out_y: object
    rx: object     # int32 [npts] device (rounded)
    ry: object
    smooth_x: object = None  # float64 [num_centers] (blend at the centres)
    smooth_y: object = None
    selection: object = None  # int32 [num_centers]: index of each centre in the pass
    num_centers: int = 0
    nb_subdom: int = 0
    counts_d: object = None    # int32 [nb_subdom] device: members per subdomain
    w_offsets_d: object = None  # int64 [nb_subdom] device: weight offsets
    weights: object = None
    singular: object = None
    mp_status: object = None
    iters: object = None
    nfixed: object = None
    mp_sweeps: object = None
    max_udiff: object = None

    @property
    def counts(self):
        """Members per subdomain (host copy, fetched on first use)."""
        if not hasattr(self, "_counts"):
            self._counts = self.counts_d.cpu().numpy().astype(np.int64)
        return self._counts

    @property
    def w_offsets(self):
        """Offsets of the subdomains' weights (host copy, fetched on first use)."""
        if not hasattr(self, "_woff"):
            self._woff = self.w_offsets_d.cpu().numpy()
        return self._woff


#: phi(k / 4) for k < PHI_TABLE_SIZE covers distances up to ~1024 px on the
#: half-integer lattice (32 MiB per device); larger distances use log() directly.
PHI_TABLE_SIZE = 1 << 22
#: entries of the shared table of kernel values that the final TPS evaluation asks
#: for (9 K^2 for offsets up to K - 1 grid steps: K = 26 covers subdomains of ~25 steps)
FINAL_EVAL_TABLE = 6144
#: largest subdomain handled by the mixed-precision solver (shared-memory bound)
MP_MAX_MEMBERS = 800
_PHI_TABLES = {}
_PHI_LOCK = threading.Lock()


def phi_table(device, pairs=False):
    """The per-device table of the TPS kernel values, float64 or (hi, lo) float pairs.

    Built on first use under a lock, on the calling thread's current stream, which
    is synchronised before the table is published: a table taken from the cache is
    complete whatever stream then reads it (``calcul_series`` runs couples on
    several host threads and streams).  ``PIVPipeline`` builds the tables it needs
    when it is constructed."""
    torch = _torch()
    key = (device.type, device.index if device.index is not None else torch.cuda.current_device(),
           pairs)
    table = _PHI_TABLES.get(key)
    if table is not None:
        return table
    with _PHI_LOCK:
        if key not in _PHI_TABLES:
            if pairs:
                table = torch.empty(2 * PHI_TABLE_SIZE, dtype=torch.float32, device=device)
                fn, name = L.load().fi_tps_phi_table2, "fi_tps_phi_table2"
            else:
                table = torch.empty(PHI_TABLE_SIZE, dtype=torch.float64, device=device)
                fn, name = L.load().fi_tps_phi_table, "fi_tps_phi_table"
            stream = torch.cuda.current_stream(device)
            L.check(fn(L.ptr(table), PHI_TABLE_SIZE, stream.cuda_stream), name)
            stream.synchronize()
            _PHI_TABLES[key] = table
        return _PHI_TABLES[key]


def lattice_coords(px, py, npts, stream=None):
    """Integer (2x, 2y) coordinates and the all-on-lattice flag (device tensors)."""
    torch = _torch()
    xy2 = torch.empty(2 * npts, dtype=torch.int32, device=px.device)
    flag = torch.empty(1, dtype=torch.int32, device=px.device)
    L.check(L.load().fi_tps_lattice(L.ptr(px), L.ptr(py), npts, L.ptr(xy2), L.ptr(flag),
                                    L.stream_handle(stream)), "fi_tps_lattice")
    return xy2, flag


@dataclass
class GridOutput:
    """griddata interpolation of a pass on a grid (linear on the Delaunay
    triangulation, nearest outside the hull; calcul/interpolate/griddata.py:11-27)."""

    out_x: object  # float64 [npts] device
    out_y: object
    rx: object     # int32 [npts] device (rounded)
    ry: object
    flags: object  # uint8 [npts]: GRID_COCIRCULAR, GRID_NEAREST_TIE
    num_centers: int = 0
    selection: object = None


_PINNED = threading.local()


def _readback_many(regions, stream=None):
    """Device regions ``(address, nbytes)`` -> one bytes object each, through a pinned
    buffer kept per host thread, with one synchronisation of the stream."""
    return _readback_finish(_readback_start(regions, stream, event=False))


def _readback_start(regions, stream=None, event=True):
    """Enqueue the copies of ``_readback_many`` on the stream; with ``event`` an event
    recorded after them lets ``_readback_finish`` wait for the copies alone, so the
    host can take the bytes while later work of the stream runs.  The thread's pinned
    buffer is reused by the next readback of the thread: finish before starting
    another."""
    torch = _torch()
    spans, total = [], 0
    for _, nbytes in regions:
        spans.append((total, nbytes))
        total += -(-nbytes // 16) * 16
    buf = getattr(_PINNED, "small", None)
    if buf is None or buf.numel() < total:
        buf = torch.empty(max(4096, total), dtype=torch.uint8, pin_memory=True)
        _PINNED.small = buf
    strm = stream or torch.cuda.current_stream()
    lib = L.load()
    for (addr, nbytes), (off, _) in zip(regions, spans):
        L.check(lib.fi_memcpy_d2h(buf.data_ptr() + off, addr, nbytes, strm.cuda_stream),
                "fi_memcpy_d2h")
    done = None
    if event:
        done = getattr(_PINNED, "event", None)
        if done is None:
            done = _PINNED.event = torch.cuda.Event()
        done.record(strm)
    return buf, spans, strm, done


def _readback_finish(handle):
    buf, spans, strm, done = handle
    if done is not None:
        done.synchronize()
    else:
        strm.synchronize()
    raw = buf.numpy()
    return [bytes(raw[off:off + nbytes]) for off, nbytes in spans]


def _readback_raw(addr, nbytes, stream=None):
    """``nbytes`` at device address ``addr`` -> bytes (one synchronisation)."""
    return _readback_many([(addr, nbytes)], stream)[0]


def _readback(t, stream=None):
    """Small device tensor -> numpy through pinned memory (one synchronisation)."""
    torch = _torch()
    t = t.contiguous()
    raw = _readback_raw(t.data_ptr(), t.numel() * t.element_size(), stream)
    return np.frombuffer(raw, dtype={torch.int64: np.int64, torch.uint8: np.uint8,
                                     torch.int32: np.int32}[t.dtype]).copy()


def y_bounds(py, npts, stream=None):
    """Prefix max / suffix min of py (fi_tps_y_bounds): index ranges for the
    membership scans."""
    torch = _torch()
    out = torch.empty(2 * max(npts, 1), dtype=torch.float64, device=py.device)
    L.check(L.load().fi_tps_y_bounds(L.ptr(py), npts, L.ptr(out), L.ptr(out[npts:]),
                                     L.stream_handle(stream)), "fi_tps_y_bounds")
    return out[:npts], out[npts:]


class _Carved:
    """Buffers carved from one device allocation (one allocator call instead of
    one per buffer): ``specs`` is a list of (count, torch dtype); each buffer starts
    on a 16-byte boundary.  ``addr[i]`` is the device address of buffer i (what the
    library calls take), ``tensor(i)`` a typed view (built only where a tensor is
    kept)."""

    def __init__(self, device, specs):
        torch = _torch()
        self.specs = specs
        self.offsets, nbytes = [], 0
        for count, dtype in specs:
            self.offsets.append(nbytes)
            nbytes += -(-count * dtype.itemsize // 16) * 16
        self.buf = torch.empty(max(nbytes, 16), dtype=torch.uint8, device=device)
        base = self.buf.data_ptr()
        self.addr = [base + o for o in self.offsets]

    def tensor(self, i):
        count, dtype = self.specs[i]
        o = self.offsets[i]
        return self.buf[o:o + count * dtype.itemsize].view(dtype)


#: subdomains a point can belong to: the buffered subdomains (20 % of a subdomain's
#: width added on each side, thin_plate_spline_subdom.py:80-88) overlap at most
#: pairwise along each axis, so the membership lists hold at most 4 entries per point
MEMBERS_PER_POINT = 4


def tps_subdomain_capacity(nvec, subdom_size):
    """Subdomains the layout buffers of a TPS over ``nvec`` vectors are sized for: the
    layout has nbx nby subdomains, nbx = floor(sqrt(nb / r)), nby = ceil(sqrt(nb r)),
    nb = (valid vectors) / subdom_size, r the aspect ratio of their extent, so about
    nb + sqrt(nb / r) (thin_plate_spline_subdom.py:56-62); the margin covers ratios down
    to ~1/16 (beyond, the layout runs again with the plan's count)."""
    nb = nvec / max(int(subdom_size), 1)
    return int(2 * nb + 4 * math.sqrt(nb)) + 16


def run_tps(xs, ys, dx, dy, nvec, px, py, npts, subdom_size, smoothing_coef,
            threshold, want_smooth, stream, p_lattice=None):
    """apply_interp with ThinPlateSplineSubdom on device (singlepass.py:466-548).

    ``p_lattice``: ``lattice_coords`` of the new positions (computed if None).
    """
    torch = _torch()
    lib = L.load()
    dev = xs.device
    s = L.stream_handle(stream)
    u8_, i32_, i64_, f32_, f64_ = (torch.uint8, torch.int32, torch.int64, torch.float32,
                                   torch.float64)
    # the plan and the compacted centres
    cA = _Carved(dev, [(L.TPS_PLAN_BYTES, u8_), (nvec, f64_), (nvec, f64_), (nvec, f32_),
                       (nvec, f32_), (nvec, i32_)])
    plan, cx, cy, ux, uy, sel = cA.addr
    with _timed("fi_tps_plan_make"):
        L.check(lib.fi_tps_plan_make(L.ptr(xs), L.ptr(ys), L.ptr(dx), L.ptr(dy), nvec,
                                     int(subdom_size), float(smoothing_coef), 20.0, plan, cx,
                                     cy, ux, uy, sel, s),
                "fi_tps_plan_make")
    # layout (lattice coordinates, y bounds, member counts, offsets) in buffers sized by
    # capacities: the kernels take the valid centres and the subdomains from the plan on
    # the device, and the host reads the plan header and the 6 totals in one
    # synchronisation (a plan with more subdomains than the estimate is laid out again)
    p_given = p_lattice is not None
    nv_cap, nsub_cap = nvec, tps_subdomain_capacity(nvec, subdom_size)
    while True:
        ctiles, ptiles = -(-nv_cap // 256), -(-npts // 256)
        specs = [(2 * nv_cap, i32_), (1, i32_), (2 * ctiles, f64_), (2 * ptiles, f64_),
                 (nsub_cap, i32_), (nsub_cap, i32_), (4 * nsub_cap + 6, i64_), (nsub_cap, i32_),
                 (MEMBERS_PER_POINT * nv_cap, i32_), (MEMBERS_PER_POINT * nv_cap, f64_),
                 (MEMBERS_PER_POINT * npts, i32_), (MEMBERS_PER_POINT * npts, f64_)]
        if not p_given:
            specs += [(2 * npts, i32_), (1, i32_)]
        cB = _Carved(dev, specs)
        (cxy2, clat, cbounds, pbounds, counts, ncounts, offs, order, idx, coefs, nidx,
         ncoefs) = cB.addr[:12]
        pxy2, plat = (L.ptr(p_lattice[0]), L.ptr(p_lattice[1])) if p_given else cB.addr[12:]
        L.check(lib.fi_tps_layout(plan, nsub_cap, cx, cy, nv_cap, L.ptr(px), L.ptr(py), npts,
                                  int(p_given), cxy2, clat, pxy2, plat, cbounds, pbounds,
                                  counts, ncounts, offs, order, s),
                "fi_tps_layout")
        # the plan header and the totals are final after the layout: their copy goes
        # first, and the membership lists (which need no host value) fill while the
        # host reads them and prepares the solve
        pending = _readback_start([(plan, C.sizeof(L.TpsPlan)), (offs + 32 * nsub_cap, 48)],
                                  stream)
        L.check(lib.fi_tps_members_fill(plan, nsub_cap, cx, cy, nv_cap, L.ptr(px), L.ptr(py),
                                        npts, cxy2, clat, pxy2, plat, cbounds, pbounds, offs,
                                        idx, coefs, nidx, ncoefs, s),
                "fi_tps_members_fill")
        raw_hdr, raw_tot = _readback_finish(pending)
        hdr = L.TpsPlan.from_buffer_copy(raw_hdr)
        if hdr.status == 1:
            raise InterpError("Only nan.")
        if hdr.status != 0:
            raise ValueError("TPS subdomain layout is degenerate (all vectors on one line)")
        nv, nsub = hdr.num_centers, hdr.nb_subdomx * hdr.nb_subdomy
        if nsub <= nsub_cap:
            break
        nsub_cap = nsub
    off_d, noff_d, moff_d, woff_d = (offs + 8 * k * nsub_cap for k in range(4))
    tot, ntot, msum, wsum, maxc, maxnc = (int(v) for v in np.frombuffer(raw_tot, np.int64))
    if tot > MEMBERS_PER_POINT * nv_cap or ntot > MEMBERS_PER_POINT * npts:
        raise RuntimeError("TPS layout: more subdomain members than the bound")
    use_mp = maxc <= MP_MAX_MEMBERS
    t1, nt1 = max(tot, 1), max(ntot, 1)
    # scratch of this call (the matrices dominate) apart from the outputs that the
    # results keep (weights, interpolated fields, per-subdomain statistics)
    cS = _Carved(dev, [
        (msum, f64_), (msum if use_mp else 0, f32_), (t1, f64_), (t1, f64_), (nt1, f64_),
        (nt1, f64_), (tot + 3 * nsub, i32_)])
    matrices, matrices32, smx, smy, partx, party, pivots = cS.addr
    cO = _Carved(dev, [
        (wsum, f64_), (2 * nsub, f64_), (npts, f64_), (npts, f64_),
        (nv if want_smooth else 0, f64_), (nv if want_smooth else 0, f64_), (2 * nsub, i32_),
        (2 * nsub, i32_), (nsub, i32_), (nsub, i32_), (nsub, i32_), (npts, i32_), (npts, i32_)])
    (weights, max_udiff, out_x, out_y, smooth_x, smooth_y, iters, nfixed, singular, status,
     sweeps, rx, ry) = cO.addr
    use_thr = threshold is not None
    thr = float(threshold) if use_thr else 0.0
    table = L.ptr(phi_table(dev))
    table2 = L.ptr(phi_table(dev, pairs=True))
    if use_mp:  # the solver writes status (1: needs the FP64 LU) and sweeps
        with _timed("fi_tps_solve_mp"):
            L.check(lib.fi_tps_solve_mp(
                plan, nsub, maxc, cx, cy, ux, uy, counts, off_d, idx, moff_d, matrices,
                matrices32, table, table2, PHI_TABLE_SIZE, cxy2, clat, thr, int(use_thr),
                woff_d, weights, smx, smy, iters, nfixed, status, max_udiff, sweeps, order, s),
                "fi_tps_solve_mp")
    else:
        cO.tensor(9).fill_(1)
        cO.tensor(10).zero_()
    # FP64 LU for the subdomains the mixed-precision solver flagged (or all of them)
    with _timed("fi_tps_solve"):
        L.check(lib.fi_tps_solve(plan, nsub, maxc, cx, cy, ux, uy, counts, off_d, idx, moff_d,
                                 matrices, pivots, thr, int(use_thr), woff_d, weights, smx,
                                 smy, iters, nfixed, singular, max_udiff, status, s),
                "fi_tps_solve")
    if want_smooth:
        L.check(lib.fi_tps_blend_centers(plan, nv, cx, cy, counts, off_d, idx, coefs, smx, smy,
                                         smooth_x, smooth_y, s),
                "fi_tps_blend_centers")
    with _timed("fi_tps_interpolate"):
        # the final evaluation (on the grid of the pass's own windows, whose vectors
        # sit on it or half a pixel off it) gets the larger shared table of offsets
        L.check(lib.fi_tps_interpolate(plan, nsub, maxc, maxnc, cx, cy, counts, off_d, idx,
                                       woff_d, weights, L.ptr(px), L.ptr(py), npts, ncounts,
                                       noff_d, nidx, ncoefs, partx, party, out_x, out_y, rx, ry,
                                       table, table2, PHI_TABLE_SIZE, cxy2, clat,
                                       FINAL_EVAL_TABLE if want_smooth else 0, s),
                "fi_tps_interpolate")
    # tensors for what the caller keeps (built while the GPU works)
    out = TpsOutput(
        out_x=cO.tensor(2), out_y=cO.tensor(3), rx=cO.tensor(11), ry=cO.tensor(12),
        selection=cA.tensor(5), num_centers=nv, nb_subdom=nsub, counts_d=cB.tensor(4)[:nsub],
        w_offsets_d=cB.tensor(6)[3 * nsub_cap:3 * nsub_cap + nsub], weights=cO.tensor(0),
        singular=cO.tensor(8), iters=cO.tensor(6), nfixed=cO.tensor(7),
        max_udiff=cO.tensor(1), mp_status=cO.tensor(9), mp_sweeps=cO.tensor(10),
    )
    if want_smooth:
        out.smooth_x, out.smooth_y = cO.tensor(4), cO.tensor(5)
    return out


def run_griddata(xs, ys, dx, dy, nvec, grid, px, py, npts, stream):
    """apply_interp with griddata on device (singlepass.py:498-556): the valid
    vectors of a pass (on its window grid ``grid`` = (ixvecs, iyvecs) device int32,
    nx, ny) interpolated at (px, py)."""
    torch = _torch()
    lib = L.load()
    dev = xs.device
    s = L.stream_handle(stream)
    ixvecs, iyvecs, nx, ny = grid
    u8_, i32_, f32_, f64_ = torch.uint8, torch.int32, torch.float32, torch.float64
    cA = _Carved(dev, [(L.TPS_PLAN_BYTES, u8_), (nvec, f64_), (nvec, f64_), (nvec, f32_),
                       (nvec, f32_), (nvec, i32_)])
    plan, cx, cy, ux, uy, sel = cA.addr
    # the compaction of the valid vectors (the subdomain layout it also computes is
    # not used)
    L.check(lib.fi_tps_plan_make(L.ptr(xs), L.ptr(ys), L.ptr(dx), L.ptr(dy), nvec, 200, 1.0,
                                 20.0, plan, cx, cy, ux, uy, sel, s), "fi_tps_plan_make")
    nscr = int(lib.fi_griddata_scratch_ints(nx, ny))
    cO = _Carved(dev, [(npts, f64_), (npts, f64_), (npts, i32_), (npts, i32_), (npts, u8_),
                       (nscr, i32_), (2, i32_)])
    out_x, out_y, rx, ry, flags, scratch, status = cO.addr
    hdr = L.TpsPlan.from_buffer_copy(_readback_raw(plan, C.sizeof(L.TpsPlan), stream))
    if hdr.status == 1:
        raise InterpError("Only nan.")
    if hdr.status != 0:
        raise ValueError("griddata: the vectors are all on one line (no triangulation)")
    nv = hdr.num_centers
    with _timed("fi_griddata"):
        L.check(lib.fi_griddata(cx, cy, ux, uy, sel, nv, L.ptr(ixvecs), nx, L.ptr(iyvecs), ny,
                                L.ptr(px), L.ptr(py), npts, scratch, out_x, out_y, rx, ry,
                                flags, status, s), "fi_griddata")
    st = int(np.frombuffer(_readback_raw(status, 4, stream), np.int32)[0])
    if st != 0:
        raise RuntimeError({1: "griddata: a position is off the half-integer lattice",
                            2: "griddata: no Delaunay triangle found",
                            3: "griddata: bad vector selection"}.get(st, f"griddata: {st}"))
    return GridOutput(out_x=cO.tensor(0), out_y=cO.tensor(1), rx=cO.tensor(2),
                      ry=cO.tensor(3), flags=cO.tensor(4), num_centers=nv,
                      selection=cA.tensor(5))


# --------------------------------------------------------------------------------
# the pipeline
def subpix_pinv(nsubpix):
    """Pseudo-inverse of [X^2, Y^2, X, Y, 1] over the (2 nsubpix + 1)^2 crop, the
    '2d_gaussian' least-squares operator of SubPix.prepare_subpix
    (calcul/subpix.py:86-105); float64, row-major 5 x K."""
    xs = np.arange(-nsubpix, nsubpix + 1, dtype=float)
    X, Y = np.meshgrid(xs, xs)
    X, Y = X.ravel(), Y.ravel()
    M = np.stack([X**2, Y**2, X, Y, np.ones(X.size)], axis=1)
    return np.ascontiguousarray(np.linalg.pinv(M), dtype=np.float64)


# --------------------------------------------------------------------------------
@dataclass
class PassDevice:
    """Device outputs of one pass."""

    layout: PassLayout
    deltaxs_raw: object
    deltays_raw: object
    correls_max: object
    errors: object
    xs: object
    ys: object
    flags: object
    deltaxs: object  # after fix
    deltays: object
    fix_flags: object
    diff2: object
    planes: object = None
    dxin: object = None
    dyin: object = None
    peaks_count: object = None  # secondary peaks (nb_peaks_to_search > 1)
    peaks: object = None
    peaks_err: object = None
    replaced: object = None  # [nvec, 3] old dx, dy, correl_max of replaced vectors
    tc_status: object = None  # device status word of the tensor-core pass (if it ran)
    fix_work: object = None  # WorkFIX scratch of the pass
    deformed: object = None  # (im0, im1) deformed by -/+ half the previous pass (deform mode)
    tps_next: Optional[object] = None  # TpsOutput or GridOutput: this pass on the next grid
    tps_final: Optional[object] = None  # TpsOutput or GridOutput: on its own grid


class PIVPipeline:
    """Compiled multipass configuration for one image shape and dtype."""

    def __init__(self, params, imshape, dtype, device=None, keep_correls=False,
                 interp_last=True, deform=False):
        torch = _torch()
        self.params = params
        #: deform im1 by the interpolated field between passes instead of shifting
        #: the windows by its rounded values (the to-do of singlepass.py:736-738)
        self.deform = bool(deform)
        self.imshape = tuple(int(s) for s in imshape)
        self.dtype = np.dtype(dtype)
        if self.dtype not in _DTYPES:
            raise TypeError(f"image dtype {self.dtype} not supported (uint8, uint16, float32)")
        self.device = torch.device(device if device is not None else "cuda")
        from .piv import TC_TAGS

        form = TC_TAGS.get(params.piv0.method_correl)
        #: FI_TC_* form of the tensor-core pass (32 px passes), None: FP32 FFT pass
        self.tc_form = None if form is None else L.TC_FORMS[form]
        #: device status word of the tensor-core passes (non-zero: a wait timed out)
        self.tc_status = (torch.zeros(1, dtype=torch.int32, device=self.device)
                          if self.tc_form is not None else None)
        self.keep_correls = keep_correls
        self.interp_last = interp_last
        p0, mp = params.piv0, params.multipass
        self.nb_peaks = int(p0.nb_peaks_to_search)
        if not 1 <= self.nb_peaks <= L.MAX_PEAKS:
            raise NotImplementedError(
                f"nb_peaks_to_search must be in 1..{L.MAX_PEAKS} on this backend")
        if self.nb_peaks > 1 and params.fix.threshold_diff_neighbour is None:
            raise ValueError(
                "nb_peaks_to_search > 1 needs fix.threshold_diff_neighbour (WorkFIX compares "
                "the secondary peaks with the neighbour mean, fix.py:168-176)")
        if p0.method_subpix not in L.SUBPIX_METHODS:
            raise ValueError(f"method has to be in {list(L.SUBPIX_METHODS)}")
        if p0.method_subpix == "2d_gaussian2" and p0.nsubpix is not None and p0.nsubpix != 1:
            raise ValueError(
                "Subpixel method '2d_gaussian2' doesn't require nsubpix. "
                "In this case, nsubpix has to be equal to None.")
        self.subpix_method = L.SUBPIX_METHODS[p0.method_subpix]
        self.nsubpix = 1 if p0.nsubpix is None else int(p0.nsubpix)
        if not 1 <= self.nsubpix <= L.MAX_NSUBPIX:
            raise NotImplementedError(f"nsubpix must be in 1..{L.MAX_NSUBPIX} on this backend")
        self.subpix_minv = None
        if p0.method_subpix == "2d_gaussian":
            self.subpix_minv = torch.as_tensor(subpix_pinv(self.nsubpix), device=self.device)
        shapes = pass_shapes(p0.shape_crop_im0, mp.number, mp.coeff_zoom)
        if p0.shape_crop_im1 is not None:
            s1 = p0.shape_crop_im1
            s1 = (s1, s1) if isinstance(s1, (int, np.integer)) else tuple(s1)
            if tuple(s1) != shapes[0]:
                raise ValueError("with this correlation method the input images have to "
                                 "have the same shape.")
        self.layouts: List[PassLayout] = []
        for ip, shape in enumerate(shapes):
            if shape[0] != shape[1] or shape[0] not in SUPPORTED_WINDOWS:
                raise NotImplementedError(
                    f"window {shape} not supported (square {SUPPORTED_WINDOWS})")
            n = shape[0]
            ixvecs, iyvecs = make_grid(self.imshape, shape, p0.grid.overlap)
            gx, gy = np.meshgrid(ixvecs, iyvecs)
            dmax = parse_displacement_max(p0.displacement_max, shape)
            mask, box = displacement_mask(n, dmax)
            lay = PassLayout(ip, n, ixvecs, iyvecs, gx.flatten(), gy.flatten(), dmax, mask, box,
                             apply_subpix=(ip == mp.number - 1))
            lay.dev["ixvecs"] = torch.as_tensor(ixvecs.astype(np.int32), device=self.device)
            lay.dev["iyvecs"] = torch.as_tensor(iyvecs.astype(np.int32), device=self.device)
            lay.dev["px"] = torch.as_tensor(lay.gx.astype(np.float64), device=self.device)
            lay.dev["py"] = torch.as_tensor(lay.gy.astype(np.float64), device=self.device)
            lay.dev["mask"] = (None if mask is None else
                               torch.as_tensor(mask.astype(np.uint8), device=self.device))
            xy2 = np.empty(2 * lay.nvec, dtype=np.int32)
            xy2[0::2] = 2 * lay.gx
            xy2[1::2] = 2 * lay.gy
            lay.dev["lattice"] = (torch.as_tensor(xy2, device=self.device),
                                  torch.ones(1, dtype=torch.int32, device=self.device))
            self.layouts.append(lay)
        if mp.use_tps is True or (mp.use_tps == "last" and interp_last):
            # the TPS tables, built here (the constructing thread) before any run
            dev = self.device if self.device.index is not None else torch.device(
                "cuda", torch.cuda.current_device())
            phi_table(dev)
            phi_table(dev, pairs=True)

    # ----------------------------------------------------------------------
    def run(self, im0, im1, stream=None) -> List[PassDevice]:
        """Run all passes on device images (torch tensors, same dtype/shape)."""
        torch = _torch()
        lib = L.load()
        if tuple(im0.shape) != self.imshape or tuple(im1.shape) != self.imshape:
            raise ValueError("image shape differs from the pipeline's")
        im0 = im0.contiguous()
        im1 = im1.contiguous()
        s = L.stream_handle(stream)
        dt = _DTYPES[self.dtype]
        H, W = self.imshape
        im_min = torch.empty(2, dtype=torch.float32, device=self.device)  # per run: runs
        # on several streams may overlap
        L.check(lib.fi_images_min(L.ptr(im0), L.ptr(im1), dt, H * W, L.ptr(im_min), s),
                "fi_images_min")
        mp, fx = self.params.multipass, self.params.fix
        outs: List[PassDevice] = []
        prev: Optional[PassDevice] = None
        for lay in self.layouts:
            dxin = dyin = None
            if prev is not None:
                if mp.use_tps is True:
                    prev.tps_next = run_tps(
                        prev.xs, prev.ys, prev.deltaxs, prev.deltays, prev.layout.nvec,
                        lay.dev["px"], lay.dev["py"], lay.nvec, mp.subdom_size,
                        mp.smoothing_coef, mp.threshold_tps, False, stream,
                        p_lattice=lay.dev["lattice"])
                else:  # use_tps False or 'last': griddata between passes
                    prev.tps_next = run_griddata(
                        prev.xs, prev.ys, prev.deltaxs, prev.deltays, prev.layout.nvec,
                        self._grid(prev.layout), lay.dev["px"], lay.dev["py"], lay.nvec,
                        stream)
                dxin, dyin = prev.tps_next.rx, prev.tps_next.ry
            if prev is not None and self.deform:
                cur = self._run_deformed_pass(lay, prev.tps_next, im0, im1, stream)
            else:
                cur = self._run_pass(lay, im0, im1, im_min, dxin, dyin, dt, s)
            self._run_fix(cur, fx, s)
            outs.append(cur)
            prev = cur
        if not self.interp_last:
            return outs
        try:
            if mp.use_tps is True or mp.use_tps == "last":
                prev.tps_final = run_tps(
                    prev.xs, prev.ys, prev.deltaxs, prev.deltays, prev.layout.nvec,
                    prev.layout.dev["px"], prev.layout.dev["py"], prev.layout.nvec,
                    mp.subdom_size, mp.smoothing_coef, mp.threshold_tps, True, stream,
                    p_lattice=prev.layout.dev["lattice"])
            else:
                prev.tps_final = run_griddata(
                    prev.xs, prev.ys, prev.deltaxs, prev.deltays, prev.layout.nvec,
                    self._grid(prev.layout), prev.layout.dev["px"], prev.layout.dev["py"],
                    prev.layout.nvec, stream)
        except InterpError as e:
            print("Warning: InterpError at the end of the last piv pass:", e)
        return outs

    @staticmethod
    def _grid(lay):
        return lay.dev["ixvecs"], lay.dev["iyvecs"], lay.ixvecs.size, lay.iyvecs.size

    def _run_pass(self, lay, im0, im1, im_min, dxin, dyin, dt, s) -> PassDevice:
        lib = L.load()
        out, a = self.make_pass(lay, im0, im1, im_min, dxin, dyin, dt)
        if self.tc_form is not None and lay.n == L.TC_WINDOW:
            out.tc_status = self.tc_status
            with _timed(f"fi_piv_pass_tc[n={lay.n}]"):
                L.check(lib.fi_piv_pass_tc(C.byref(a), self.tc_form, L.ptr(self.tc_status), s),
                        "fi_piv_pass_tc")
        else:
            with _timed(f"fi_piv_pass[n={lay.n}]"):
                L.check(lib.fi_piv_pass(C.byref(a), s), "fi_piv_pass")
        return out

    def _run_deformed_pass(self, lay, field, im0, im1, stream):
        """A pass on the images deformed by ``field`` (the previous pass interpolated on
        this pass's grid) with the central scheme, im0 by -d/2 and im1 by +d/2:
        windows at the grid points, the measured residual plus the field value as
        the displacement of the grid point.  The minima are those of the float
        images."""
        torch = _torch()
        lib = L.load()
        from .deform import warp

        s = L.stream_handle(stream)
        nodes = torch.stack([field.out_x, field.out_y]).to(torch.float32).reshape(
            1, 2, lay.iyvecs.size, lay.ixvecs.size).contiguous()
        if "xn" not in lay.dev:
            lay.dev["xn"], lay.dev["yn"] = lay.dev["ixvecs"].float(), lay.dev["iyvecs"].float()
        xn, yn = lay.dev["xn"], lay.dev["yn"]
        f0 = warp(nodes, xn, yn, im0.unsqueeze(0), -0.5, stream)[0]
        f1 = warp(nodes, xn, yn, im1.unsqueeze(0), 0.5, stream)[0]
        im_min = torch.empty(2, dtype=torch.float32, device=self.device)
        H, W = self.imshape
        L.check(lib.fi_images_min(L.ptr(f0), L.ptr(f1), L.FI_F32, H * W, L.ptr(im_min), s),
                "fi_images_min")
        out = self._run_pass(lay, f0, f1, im_min, None, None, L.FI_F32, s)
        out.deformed = (f0, f1)
        # displacement = field at the vector (the grid point) + measured residual
        out.deltaxs_raw += field.out_x.to(torch.float32)
        out.deltays_raw += field.out_y.to(torch.float32)
        out.dxin, out.dyin = field.rx, field.ry
        return out

    def make_pass(self, lay, im0, im1, im_min, dxin, dyin, dt):
        """The outputs of a pass (device tensors) and its fi_piv_pass_args."""
        torch = _torch()
        nvec, dev = lay.nvec, self.device
        f32 = dict(dtype=torch.float32, device=dev)
        u8 = dict(dtype=torch.uint8, device=dev)
        out = PassDevice(
            layout=lay, deltaxs_raw=torch.empty(nvec, **f32), deltays_raw=torch.empty(nvec, **f32),
            correls_max=torch.empty(nvec, **f32), errors=torch.empty(nvec, **u8),
            xs=torch.empty(nvec, **f32), ys=torch.empty(nvec, **f32),
            flags=torch.empty(nvec, **u8), deltaxs=torch.empty(nvec, **f32),
            deltays=torch.empty(nvec, **f32), fix_flags=torch.empty(nvec, **u8),
            diff2=torch.empty(nvec, **f32), dxin=dxin, dyin=dyin,
        )
        if self.keep_correls:
            out.planes = torch.empty(nvec * lay.n * lay.n, **f32)
        K = self.nb_peaks - 1
        if K > 0:
            out.peaks_count = torch.empty(nvec, dtype=torch.int32, device=dev)
            out.peaks = torch.empty(nvec * K * L.PEAK_FIELDS, **f32)
            out.peaks_err = torch.empty(nvec * K, **u8)
            out.replaced = torch.empty(3 * nvec, **f32)
        H, W = self.imshape
        a = L.PivPassArgs()
        a.im0, a.im1, a.dtype, a.height, a.width = L.ptr(im0), L.ptr(im1), dt, H, W
        a.im_min = L.ptr(im_min)
        a.n = lay.n
        a.ixvecs, a.nx = L.ptr(lay.dev["ixvecs"]), lay.ixvecs.size
        a.iyvecs, a.ny = L.ptr(lay.dev["iyvecs"]), lay.iyvecs.size
        a.dxin, a.dyin = L.ptr(dxin), L.ptr(dyin)
        a.mask = L.ptr(lay.dev["mask"])
        a.box_i0_start, a.box_i0_stop, a.box_i1_start, a.box_i1_stop = lay.box
        a.particle_radius = int(self.params.piv0.particle_radius)
        a.apply_subpix = int(lay.apply_subpix)
        a.deltaxs, a.deltays = L.ptr(out.deltaxs_raw), L.ptr(out.deltays_raw)
        a.correls_max, a.errors = L.ptr(out.correls_max), L.ptr(out.errors)
        a.xs, a.ys = L.ptr(out.xs), L.ptr(out.ys)
        a.norms = None
        a.planes = L.ptr(out.planes)
        a.flags = L.ptr(out.flags)
        a.subpix_method, a.nsubpix = self.subpix_method, self.nsubpix
        a.subpix_minv = L.ptr(self.subpix_minv)
        a.nb_peaks = self.nb_peaks
        a.peaks_count, a.peaks, a.peaks_err = (L.ptr(out.peaks_count), L.ptr(out.peaks),
                                               L.ptr(out.peaks_err))
        return out, a

    def _run_fix(self, cur: PassDevice, fx, s):
        lib = L.load()
        a = self.make_fix(cur, fx)
        if a.use_threshold and (a.nx < 2 or a.ny < 2):
            raise GridError(f"WorkFIX's neighbour test needs a vector grid of at least 2 x 2 "
                            f"(this one is {a.ny} x {a.nx})")
        with _timed("fi_fix"):
            L.check(lib.fi_fix(C.byref(a), s), "fi_fix")

    def make_fix(self, cur: PassDevice, fx):
        """The fi_fix_args of a pass's WorkFIX (its work buffer kept on ``cur``)."""
        torch = _torch()
        lay = cur.layout
        a = L.FixArgs()
        a.nx, a.ny = lay.ixvecs.size, lay.iyvecs.size
        a.deltaxs, a.deltays = L.ptr(cur.deltaxs_raw), L.ptr(cur.deltays_raw)
        a.correls_max, a.errors = L.ptr(cur.correls_max), L.ptr(cur.errors)
        a.correl_min = float(fx.correl_min)
        a.use_displacement_max = int(bool(fx.displacement_max))
        a.displacement_max = float(fx.displacement_max or 0.0)
        a.use_threshold = int(fx.threshold_diff_neighbour is not None)
        a.threshold = float(fx.threshold_diff_neighbour or 0.0)
        a.deltaxs_out, a.deltays_out = L.ptr(cur.deltaxs), L.ptr(cur.deltays)
        a.fix_flags, a.diff2 = L.ptr(cur.fix_flags), L.ptr(cur.diff2)
        cur.fix_work = torch.empty(2 * lay.nvec, dtype=torch.float32, device=self.device)
        a.work = L.ptr(cur.fix_work)
        a.nb_peaks = self.nb_peaks
        if self.nb_peaks > 1:  # WorkFIX secondary peaks (fix.py:135-236)
            a.peaks_count, a.peaks, a.peaks_err = (L.ptr(cur.peaks_count), L.ptr(cur.peaks),
                                                   L.ptr(cur.peaks_err))
            a.dxin, a.dyin = L.ptr(cur.dxin), L.ptr(cur.dyin)
            a.threshold64 = float(fx.threshold_diff_neighbour)
            a.displacement_max64 = float(fx.displacement_max or 0.0)
            a.correls_max_out = L.ptr(cur.correls_max)
            a.replaced = L.ptr(cur.replaced)
        return a


# --------------------------------------------------------------------------------
# device -> host results
# --------------------------------------------------------------------------------
def error_dict(err, fix_flags, diff2, threshold):
    """Rebuild ``errors`` of _loop_vectors + WorkFIX (fix.py:66-236) from the codes."""
    err = np.asarray(err)
    fix_flags = np.asarray(fix_flags)
    # WorkFIX deletes the errors of replaced vectors (fix.py:229-234)
    sel = np.nonzero(((err != 0) | (fix_flags != 0)) & ((fix_flags & L.FIX_REPLACED) == 0))[0]
    if sel.size == 0:
        return {}
    codes = err[sel].tolist()
    flags = fix_flags[sel].tolist()
    diffs = np.sqrt(np.asarray(diff2)[sel].astype(np.float64)).tolist()
    texts = ((1, "correl < correl_min"), (2, "delta2 < displacement_max2"),
             (4, "diff neighbour too large"))
    errors = {}
    for i, e, f, d in zip(sel.tolist(), codes, flags, diffs):
        s = ERROR_STRINGS.get(e) if e else None
        for bit, text in texts:
            if f & bit:
                s = text if s is None else s + " + " + text
        if f & 4:
            s += f" (diff = {d:.2f})"
        errors[i] = s
    return errors
