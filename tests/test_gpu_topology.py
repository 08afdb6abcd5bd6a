"""The work under a topology's executors on the GPU: several host threads calling
``calcul`` at once (thread executors), and worker processes forked from a process
that built the work but never used CUDA (``multi_exec_async``); both give the
results of one-at-a-time calls, bit for bit."""

import numpy as np
import pytest

from fluidimage_gb300 import WorkPIV, workloads


def _pairs(count):
    (im0, im1), _ = workloads.config2_images(shape=(512, 512))
    return [(np.roll(im0, 29 * k, axis=1), np.roll(im1, 29 * k, axis=1)) for k in range(count)]


def _assert_same(a, b):
    for pa, pb in zip(a.passes, b.passes):
        np.testing.assert_array_equal(pa.deltaxs, pb.deltaxs)
        np.testing.assert_array_equal(pa.deltays, pb.deltays)
        assert pa.errors == pb.errors
    np.testing.assert_array_equal(a.passes[-1].deltaxs_final, b.passes[-1].deltaxs_final)
    np.testing.assert_array_equal(a.passes[-1].deltays_final, b.passes[-1].deltays_final)


@pytest.mark.gpu
def test_threads_calling_calcul():
    from concurrent.futures import ThreadPoolExecutor

    params = workloads.config2_params(WorkPIV.create_default_params())
    pairs = _pairs(6)
    work = WorkPIV(params)
    singles = [work.calcul({"arrays": p, "names": ("a", "b")}) for p in pairs]
    shared = WorkPIV(params)
    with ThreadPoolExecutor(max_workers=3) as pool:
        futures = [pool.submit(shared.calcul, {"arrays": p, "names": ("a", "b")})
                   for p in pairs]
        results = [f.result(timeout=300) for f in futures]
    for a, b in zip(singles, results):
        _assert_same(a, b)


_FORK_SCRIPT = r"""
import multiprocessing as mp
import sys
from pathlib import Path

import numpy as np
import torch

sys.path.insert(0, sys.argv[1])
out = Path(sys.argv[2])
from fluidimage_gb300 import WorkPIV, workloads

(im0, im1), _ = workloads.config2_images(shape=(512, 512))
pairs = [(np.roll(im0, 29 * k, axis=1), np.roll(im1, 29 * k, axis=1)) for k in range(4)]
work = WorkPIV(workloads.config2_params(WorkPIV.create_default_params()))
assert not torch.cuda.is_initialized()


def worker(index):
    for k in range(index, len(pairs), 2):
        r = work.calcul({"arrays": pairs[k], "names": ("a", "b")})
        last = r.passes[-1]
        np.savez(out / f"pair{k}.npz", dx=last.deltaxs, dy=last.deltays,
                 fx=last.deltaxs_final, fy=last.deltays_final)


procs = [mp.get_context("fork").Process(target=worker, args=(i,)) for i in range(2)]
for p in procs:
    p.start()
codes = []
for p in procs:
    p.join(240)
    if p.is_alive():
        p.kill()
        p.join()
    codes.append(p.exitcode)
if codes != [0, 0]:
    sys.exit(f"worker exit codes {codes}")
for k, pair in enumerate(pairs):
    last = work.calcul({"arrays": pair, "names": ("a", "b")}).passes[-1]
    got = np.load(out / f"pair{k}.npz")
    for key, ref in (("dx", last.deltaxs), ("dy", last.deltays),
                     ("fx", last.deltaxs_final), ("fy", last.deltays_final)):
        np.testing.assert_array_equal(got[key], ref)
print("fork ok")
"""


@pytest.mark.gpu
def test_forked_workers(tmp_path):
    """The pattern of ``multi_exec_async``: the work is built in the parent, which
    has not used CUDA, and forked worker processes run couples on their own CUDA
    contexts; the parent's own results afterwards are the same."""
    import subprocess
    import sys
    from pathlib import Path

    repo = str(Path(__file__).resolve().parents[1])
    proc = subprocess.run([sys.executable, "-c", _FORK_SCRIPT, repo, str(tmp_path)],
                          capture_output=True, text=True, timeout=600)
    assert proc.returncode == 0, proc.stdout[-2000:] + proc.stderr[-4000:]
    assert "fork ok" in proc.stdout
