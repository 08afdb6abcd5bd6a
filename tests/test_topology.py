"""The GPU work inside a PIV topology: parameter completion, the subclass of the
topology, and the fork guard (CPU); thread and fork executors on the GPU
(``test_gpu_topology.py``)."""

import pytest

from fluidimage_gb300 import ParamContainer, WorkPIV
from fluidimage_gb300.topology import topology_piv_class


class _TopologyStandIn:
    """The two uses topologies/piv.py makes of ``WorkVelocimetry`` (:58-76 and
    :142-149): the class completes the topology's parameters, an instance's
    ``calcul`` becomes the "compute piv" work."""

    WorkVelocimetry = None

    @classmethod
    def create_default_params(cls):
        params = ParamContainer(tag="params")
        params._set_child("saving", attribs={"path": None, "how": "ask", "postfix": "piv"})
        cls.WorkVelocimetry._complete_params_with_default(params)
        params._set_child("preproc", attribs={"im2im": None})
        return params

    def __init__(self, params):
        self.params = params
        self.work_piv = self.WorkVelocimetry(self.params)
        self.works = {"compute piv": self.work_piv.calcul}


def test_complete_params_with_default():
    params = ParamContainer(tag="params")
    WorkPIV._complete_params_with_default(params)
    assert params == WorkPIV.create_default_params()


def test_topology_subclass_uses_gpu_work():
    cls = topology_piv_class(_TopologyStandIn)
    assert issubclass(cls, _TopologyStandIn) and cls.WorkVelocimetry is WorkPIV
    params = cls.create_default_params()
    for tag in ("saving", "series", "piv0", "fix", "multipass", "mask", "preproc"):
        assert tag in params._tag_children
    params.multipass.number = 2
    topo = cls(params)
    assert isinstance(topo.work_piv, WorkPIV)
    assert topo.works["compute piv"].__self__ is topo.work_piv
    # building the work starts no CUDA context (workers are forked after it)
    import torch

    assert not torch.cuda.is_initialized()


def test_pickled_work_drops_pipelines():
    import pickle

    work = WorkPIV()
    work._pipelines["key"] = object()
    clone = pickle.loads(pickle.dumps(work))
    assert clone._pipelines == {} and clone.params == work.params
    assert clone._lock is not work._lock


def test_bad_fork_refused(monkeypatch):
    """A worker forked after its parent used CUDA refuses the couple before any
    CUDA call (the guard reads torch's own flag)."""
    import numpy as np
    import torch

    monkeypatch.setattr(torch.cuda, "_is_in_bad_fork", lambda: True, raising=False)
    im = np.zeros((64, 64), np.uint8)
    with pytest.raises(RuntimeError, match="forked"):
        WorkPIV().calcul({"arrays": (im, im), "names": ("a", "b")})
    with pytest.raises(RuntimeError, match="forked"):
        next(WorkPIV().calcul_series([{"arrays": (im, im), "names": ("a", "b")}]))
    assert not torch.cuda.is_initialized()
