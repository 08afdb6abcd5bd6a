"""This package's ``WorkPIV`` as the "compute piv" work of fluidimage's PIV topology.

``TopologyPIV`` (topologies/piv.py:24-157) takes its work class from its class
attribute ``WorkVelocimetry`` (:53): its default parameters come from
``WorkVelocimetry._complete_params_with_default`` (:74) and its "compute piv" work
is ``WorkVelocimetry(params).calcul`` (:142-149).  ``topology_piv_class`` returns the
subclass of an installed fluidimage's ``TopologyPIV`` whose work is this package's
``WorkPIV``; listing the series, reading the images, the preprocessing, pairing the
arrays and saving the results stay upstream's (the results' ``save`` writes
upstream's HDF5 layout, ``data_objects.MultipassPIVResults.save``).

Executors (executors/): the work is built in the topology's process and starts
CUDA only on its first couple.  A multi-process executor (``multi_exec_async``,
upstream's default on Linux, forks one process per slice of the series,
executors/multi_exec_async.py:114-190) therefore gives each worker process a CUDA
context of its own; a worker forked from a process that had already used CUDA
raises ``RuntimeError`` on its first couple instead of using the parent's context.
Thread executors (``exec_async``) call ``calcul`` from several threads of one
process: each thread runs its couples on a CUDA stream of its own, so the couples'
kernels overlap in one context.  On one GPU that is the better fit (one context,
no per-process copy of the pipelines).

Usage::

    from fluidimage_gb300.topology import topology_piv_class

    TopologyPIV = topology_piv_class()
    params = TopologyPIV.create_default_params()
    params.series.path = "images/*.png"
    TopologyPIV(params).compute(executor="exec_async")
"""

from __future__ import annotations

from .piv import WorkPIV


def topology_piv_class(base=None):
    """Subclass of ``base`` (default: ``fluidimage.topologies.piv.TopologyPIV``)
    whose "compute piv" work is :class:`fluidimage_gb300.WorkPIV`."""
    if base is None:
        from fluidimage.topologies.piv import TopologyPIV as base
    return type(
        "TopologyPIVGB300",
        (base,),
        {
            "WorkVelocimetry": WorkPIV,
            "__module__": __name__,
            "__doc__": f"{base.__name__} with its PIV work on the GPU "
                       "(fluidimage_gb300.WorkPIV).",
        },
    )
