"""fi_fix_static: the allocation-free WorkFIX entry point.

Some callers cannot allocate device memory (a host framework that owns a fixed
device-memory budget, or a latency-critical loop where cudaMalloc and its implicit
device synchronisation are not allowed), so they cannot provide fi_fix's work
buffer.  fi_fix_static keeps that scratch in a static device array of the library.
This test calls both entry points through the C ABI on the same inputs, twice in a
row with different inputs (the static scratch keeps the previous call's contents),
and requires identical outputs (both run the same float32 kernels, so the
tolerance is exact equality).  It covers the three kernel paths: the neighbour
test alone, the neighbour test with secondary-peak replacement (which reads the
scratch again), and no neighbour test (no scratch).
"""

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _inputs(seed, ny, nx, dev):
    import torch

    rng = np.random.default_rng(seed)
    n = ny * nx
    dx = rng.normal(0.0, 2.0, n).astype(np.float32)
    dy = rng.normal(0.0, 2.0, n).astype(np.float32)
    bad = rng.random(n) < 0.05
    dx[bad] = np.nan
    dy[bad] = np.nan
    cmax = rng.random(n).astype(np.float32)
    err = (rng.random(n) < 0.03).astype(np.uint8)
    to = lambda a: torch.from_numpy(a).to(dev)  # noqa: E731
    return to(dx), to(dy), to(cmax), to(err)


def _secondary(seed, n, dev, K=2):
    """Secondary peaks of every vector: counts, (dx, dy, correl_max, replacement x,
    replacement y) and fit errors, with input shifts (a pass >= 1)."""
    import torch

    rng = np.random.default_rng(100 + seed)
    count = rng.integers(-1, K + 1, n).astype(np.int32)
    peaks = np.zeros((n, K, 5), np.float32)
    peaks[:, :, 0] = rng.integers(-4, 5, (n, K))
    peaks[:, :, 1] = rng.integers(-4, 5, (n, K))
    peaks[:, :, 2] = rng.random((n, K))
    peaks[:, :, 3] = peaks[:, :, 0] + rng.normal(0, 0.3, (n, K))
    peaks[:, :, 4] = peaks[:, :, 1] + rng.normal(0, 0.3, (n, K))
    perr = (rng.random((n, K)) < 0.1).astype(np.uint8)
    dxin = rng.integers(-1, 2, n).astype(np.int32)
    dyin = rng.integers(-1, 2, n).astype(np.int32)
    to = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)  # noqa: E731
    return K + 1, to(count), to(peaks.ravel()), to(perr.ravel()), to(dxin), to(dyin)


def _run(lib, L, fn, inputs, ny, nx, with_work, threshold=True, secondary=None):
    import torch

    dx, dy, cmax, err = inputs
    n = ny * nx
    dev = dx.device
    ox = torch.full((n,), -7.0, device=dev)
    oy = torch.full((n,), -7.0, device=dev)
    flags = torch.zeros(n, dtype=torch.uint8, device=dev)
    diff2 = torch.zeros(n, device=dev)
    cmax_out = cmax.clone()
    replaced = torch.full((3 * n,), -9.0, device=dev)
    work = torch.empty(2 * n, device=dev) if with_work else None
    a = L.FixArgs()
    a.nx, a.ny = nx, ny
    a.deltaxs, a.deltays = dx.data_ptr(), dy.data_ptr()
    a.correls_max, a.errors = cmax.data_ptr(), err.data_ptr()
    a.correl_min = 0.2
    a.use_displacement_max = 1
    a.displacement_max = 5.0
    a.use_threshold = int(threshold)
    a.threshold = 1.5
    a.deltaxs_out, a.deltays_out = ox.data_ptr(), oy.data_ptr()
    a.fix_flags, a.diff2 = flags.data_ptr(), diff2.data_ptr()
    a.work = work.data_ptr() if work is not None else None
    a.nb_peaks = 1
    if secondary is not None:
        nb, count, peaks, perr, dxin, dyin = secondary
        a.nb_peaks = nb
        a.peaks_count, a.peaks, a.peaks_err = count.data_ptr(), peaks.data_ptr(), perr.data_ptr()
        a.dxin, a.dyin = dxin.data_ptr(), dyin.data_ptr()
        a.threshold64 = 1.5
        a.displacement_max64 = 30.0
        a.correls_max_out = cmax_out.data_ptr()
        a.replaced = replaced.data_ptr()
    L.check(fn(C.byref(a), L.stream_handle()), "fix")
    torch.cuda.synchronize()
    return [t.cpu().numpy() for t in (ox, oy, flags, diff2, cmax_out, replaced)]


@pytest.mark.parametrize("mode", ["threshold", "secondary_peaks", "no_threshold"])
def test_fix_static_matches_fix_twice(mode):
    import torch

    from fluidimage_gb300 import _lib as L

    lib = L.load()
    dev = torch.device("cuda")
    for call, (seed, ny, nx) in enumerate([(1, 61, 73), (2, 127, 127)]):
        inputs = _inputs(seed, ny, nx, dev)
        kw = dict(threshold=(mode != "no_threshold"),
                  secondary=_secondary(seed, ny * nx, dev) if mode == "secondary_peaks"
                  else None)
        want = _run(lib, L, lib.fi_fix, inputs, ny, nx, with_work=True, **kw)
        got = _run(lib, L, lib.fi_fix_static, inputs, ny, nx, with_work=False, **kw)
        for g, w in zip(got, want):
            np.testing.assert_array_equal(g, w, err_msg=f"{mode}, call {call}")
        assert np.isnan(got[0]).sum() > 0
        if mode == "secondary_peaks":
            assert (got[2] & L.FIX_REPLACED).sum() > 0  # the replacement stage ran


def test_fix_static_rejects_oversized_grids():
    from fluidimage_gb300 import _lib as L

    lib = L.load()
    a = L.FixArgs()
    a.nx, a.ny = 1024, 1024
    assert lib.fi_fix_static(C.byref(a), None) == L.FI_OK - 1
    assert b"exceed the static scratch limit" in lib.fi_last_error()
