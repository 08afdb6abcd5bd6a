"""PIV data objects with the attributes of the upstream ones.

``ArrayCouple``, ``HeavyPIVResults`` and ``MultipassPIVResults`` follow
``fluidimage/data_objects/piv.py:78-204, 214-320, 538-600``: same attribute
names, dtypes and container behaviour (``passes``, ``piv0``, ``piv1``, ...,
indexing).  HDF5 saving is not provided.
"""

from __future__ import annotations

import numpy as np


def get_slices_from_strcrop(strcrop):
    """``'100:600, :'`` -> tuple of slices (data_objects/piv.py:71-75)."""
    return tuple(
        slice(*(int(i) if i else None for i in part.strip().split(":")))
        for part in strcrop.split(",")
    )


class ArrayCouple:
    """Couple of arrays (images), optionally masked with ``params.mask.strcrop``."""

    def __init__(self, names=None, arrays=None, params_mask=None, serie=None, paths=None):
        if arrays is None:
            raise ValueError("ArrayCouple needs arrays (reading image files is not provided)")
        self.params_mask = params_mask
        self.paths = paths
        self.serie = serie
        if names is None:
            names = ("array0", "array1")
        self.names = tuple(names)
        self.name = "-".join(self.names)
        self.shape_images = arrays[0].shape
        self.arrays = self._mask_arrays(arrays)

    def apply_mask(self, params_mask):
        if self.params_mask is not None and params_mask is None:
            raise NotImplementedError
        if self.params_mask is not None and params_mask == self.params_mask:
            return
        if self.params_mask is not None:
            raise NotImplementedError
        self.params_mask = params_mask
        self.arrays = self._mask_arrays(self.arrays)

    def _mask_array(self, array):
        if self.params_mask is None or self.params_mask.strcrop is None:
            return array
        return array[get_slices_from_strcrop(self.params_mask.strcrop)]

    def _mask_arrays(self, arrays):
        return tuple(self._mask_array(a) for a in arrays)

    def get_arrays(self):
        return self.arrays


class HeavyPIVResults:
    """Displacements and peaks of one pass.

    Attributes: ``deltaxs, deltays`` (float32), ``xs, ys``, ``correls_max``
    (float32), ``errors`` (dict index -> explanation), ``correls`` (list of
    planes or None), ``secondary_peaks``, ``couple``, ``params``; plus the
    interpolated fields added by the next pass or by the final interpolation
    (``deltaxs_approx``, ``deltaxs_final``, ``deltaxs_smooth``, ...).
    """

    def __init__(self, deltaxs=None, deltays=None, xs=None, ys=None, errors=None,
                 correls_max=None, correls=None, couple=None, params=None,
                 secondary_peaks=None, indices_no_displacement=None):
        self.deltaxs = deltaxs
        self.deltays = deltays
        self.xs = xs
        self.ys = ys
        self.errors = errors
        self.correls_max = correls_max
        self.correls = correls
        self.couple = couple
        self.params = params
        self.secondary_peaks = secondary_peaks
        self.indices_no_displacement = indices_no_displacement

    def get_images(self):
        return self.couple.get_arrays()


class MultipassPIVResults:
    """Result of a multipass PIV computation (``passes``, ``piv0``, ``piv1``...)."""

    def __init__(self):
        self.passes = []

    def __getitem__(self, key):
        return self.passes[key]

    def __len__(self):
        return len(self.passes)

    def append(self, results):
        i = len(self.passes)
        self.passes.append(results)
        self.__dict__[f"piv{i}"] = results
