"""``WorkBOS``: background-oriented schlieren on the GPU (works/bos.py:19-91).

BOS is PIV between one reference image and each image of a series: the work wraps
a ``WorkPIV`` with the same parameters plus ``params.reference``.  Here the (masked)
reference image is copied to the GPU once and stays in HBM; each call uploads only
the new image.  Image files are not read by this package: the series is given as
arrays (``images``: a mapping name -> array, or a sequence of (name, array) pairs,
in the role of the reference's ``params.images`` serie of files).
"""

from __future__ import annotations

import collections

import numpy as np

from .data_objects import ArrayCouple
from .params import ParamContainer
from .piv import (WorkPIV, _complete_params_fix, _complete_params_multipass,
                  _complete_params_piv0, _fetch_finish, _fetch_start, _host_dtype,
                  _to_device)


class ArrayCoupleBOS(ArrayCouple):
    """Couple (reference, image), named after the image (data_objects/piv.py:207-211)."""

    def __init__(self, names=None, arrays=None, params_mask=None, serie=None, paths=None):
        super().__init__(names=names, arrays=arrays, params_mask=params_mask, serie=serie,
                         paths=paths)
        self.name = self.names[-1]


class WorkBOS:
    """Work for BOS computation (works/bos.py:19-91).

    Parameters
    ----------
    params : ParamContainer from :meth:`create_default_params` (``params.reference``:
        index in the sorted image names, or a name).
    images : mapping name -> array, or sequence of (name, array): the series.
    reference_image : optional array used as the reference (then
        ``params.reference`` only names it).
    device, keep_correls, interp_last : as for ``WorkPIV``.
    """

    @classmethod
    def create_default_params(cls):
        params = ParamContainer(tag="params")
        params._set_child("images", attribs={"path": "", "str_subset": None})
        _complete_params_piv0(params)
        _complete_params_fix(params)
        _complete_params_multipass(params)
        params._set_attrib("reference", 0)
        return params

    def __init__(self, params=None, images=None, reference_image=None, device=None,
                 keep_correls=False, interp_last=True):
        if params is None:
            params = self.create_default_params()
        self.params = params
        self.work_piv = WorkPIV(params, keep_correls=keep_correls, device=device,
                                interp_last=interp_last)
        if images is None:
            images = {}
        self.images = collections.OrderedDict(
            sorted(images.items()) if isinstance(images, dict) else list(images))
        self._init_reference(reference_image)
        self._reference_device = None

    def _init_reference(self, reference_image):
        reference = self.params.reference
        names = sorted(self.images)
        if isinstance(reference, (int, np.integer)):
            if reference_image is not None and not names:
                self.name_reference = f"array{int(reference)}"
            else:
                self.name_reference = names[int(reference)]
        else:
            self.name_reference = str(reference)
            if reference_image is None and self.name_reference not in self.images:
                raise ValueError("Bad value of params.reference:" + self.name_reference)
        self.image_reference = (reference_image if reference_image is not None
                                else self.images[self.name_reference])

    def _couple(self, image, name):
        return ArrayCoupleBOS(names=(self.name_reference, name),
                              arrays=(self.image_reference, image),
                              params_mask=self.params.mask)

    def _reference_on_device(self, couple):
        """The masked reference image, uploaded once (it stays in HBM)."""
        import torch

        if self._reference_device is None:
            dev = torch.device(self.work_piv.device or "cuda")
            self._reference_device = _to_device(couple.get_arrays()[0], dev)
        return self._reference_device

    def calcul(self, tuple_image_name):
        """BOS displacement field of one image (``MultipassPIVResults``)."""
        import torch

        image, name = tuple_image_name
        couple = self._couple(image, name)
        dev = torch.device(self.work_piv.device or "cuda")
        ref = self._reference_on_device(couple)
        outs = self.work_piv.calcul_device(ref, _to_device(couple.get_arrays()[1], dev))
        return self.work_piv.results_to_host(outs, couple)

    def get_tuple_image_name(self, index_image=0):
        """An image of the series and its name (works/__init__.py:214-219)."""
        name = list(self.images)[index_image]
        return self.images[name], name

    def process_1_image(self, index_serie=0):
        return self.calcul(self.get_tuple_image_name(index_serie))

    def calcul_series(self, tuples_image_name=None, streams=2):
        """Results for a series of (image, name) (default: the work's images), in
        order, with ``streams`` images in flight (``WorkPIV.calcul_series``)."""
        import threading

        import torch
        from concurrent.futures import ThreadPoolExecutor

        if tuples_image_name is None:
            tuples_image_name = ((arr, name) for name, arr in self.images.items())
        dev = torch.device(self.work_piv.device or "cuda")
        work = self.work_piv
        local = threading.local()

        def run(couple, ref):
            if getattr(local, "stream", None) is None:
                local.stream = torch.cuda.Stream(device=dev)
            with torch.cuda.stream(local.stream):
                # the reference was written on the creating stream
                local.stream.wait_stream(torch.cuda.default_stream(dev))
                outs = work.calcul_device(ref, _to_device(couple.get_arrays()[1], dev),
                                          stream=local.stream)
                want = work._device_results(outs)
                handle = _fetch_start(list(want.values()))
                return work._host_results(outs, couple, dict(zip(want, _fetch_finish(handle))))

        nstreams = max(1, int(streams))
        pending = collections.deque()
        with ThreadPoolExecutor(max_workers=nstreams) as pool:
            for image, name in tuples_image_name:
                couple = self._couple(image, name)
                ref = self._reference_on_device(couple)
                work._pipeline(tuple(ref.shape), _host_dtype(couple.get_arrays()[0]))
                if len(pending) >= nstreams:
                    yield pending.popleft().result()
                pending.append(pool.submit(run, couple, ref))
            while pending:
                yield pending.popleft().result()
