"""PIV data objects with the attributes of the upstream ones.

``ArrayCouple``, ``HeavyPIVResults`` and ``MultipassPIVResults`` follow
``fluidimage/data_objects/piv.py:78-204, 214-320, 538-600``: same attribute
names, dtypes and container behaviour (``passes``, ``piv0``, ``piv1``, ...,
indexing).

``save`` writes upstream's HDF5 layout (data_objects/piv.py:363-455, 586-618) with
h5py, which must then be installed: the file, group, dataset and attribute names,
the float64 -> float32 conversion of the saved arrays, the dictionaries as
``keys`` / ``values`` datasets with the error ``codes``, and the per-subdomain TPS
weights, so that upstream's readers (``MultipassPIVResults(str_path=...)``) and
tools open the files.  ``MultipassPIVResults(str_path=...)`` reads them back.  The
parameters group is written by the parameters' own ``_save_as_hdf5`` (fluiddyn's
when the results come from an upstream topology, ``params.ParamContainer``'s
otherwise).
"""

from __future__ import annotations

import os

import numpy as np

#: file-format constants of upstream's PIV files (data_objects/piv.py:256-276,
#: 426-440, 590-604): the datasets and dictionaries of a pass, the error codes
KEYS_SAVED = (
    "xs", "ys", "xs_smooth", "ys_smooth", "deltaxs", "deltays", "correls_max",
    "deltaxs_approx", "deltays_approx", "ixvecs_approx", "iyvecs_approx",
    "deltaxs_final", "deltays_final", "deltaxs_smooth", "deltays_smooth",
    "ixvecs_final", "iyvecs_final",
)
DICTS_SAVED = ("errors", "deltaxs_wrong", "deltays_wrong")
ERROR_CODES = (
    (b"Correlation peak touching", 1),
    (b"correl < correl_min", 2),
    (b"delta2 < displacement_max2", 3),
    (b"diff neighbour too large", 4),
)
MODULE_NAME = "fluidimage.data_objects.piv"
CONVENTIONS = "fluidimage.data_objects.piv.MultipassPIVResults v1"


def _h5py():
    try:
        import h5py
    except ImportError as exc:
        raise ModuleNotFoundError(
            "saving or loading PIV results in HDF5 files needs h5py") from exc
    return h5py


def get_name_piv(serie, prefix="piv"):
    """File name of the results of a couple of a fluiddyn series
    (data_objects/piv.py:38-57): ``<prefix>_<indices>.h5``, the indices of each
    dimension written first-last when they differ."""
    text = ""
    for idim, inds in enumerate(serie.get_slicing_tuples()):
        first = serie.get_str_for_name_from_idim_idx(idim, inds[0])
        part = first
        if len(inds) > 1:
            last = serie.get_str_for_name_from_idim_idx(idim, inds[1] - 1)
            if last != first:
                part += ("" if first.isalpha() and len(first) == 1 else "-") + last
        if idim > 1:
            text += serie.get_index_separators[idim - 1]
        text += part
    return f"{prefix}_{text}.h5"


def get_name_bos(name, serie):
    """File name of BOS results (data_objects/piv.py:60-64): the image name without
    the series' base name and file extension, after ``bos``."""
    name = name[len(serie.base_name):]
    if serie.extension_file is not None:
        name = name[: -len(serie.extension_file) - 1]
    return f"bos{name}.h5"


def get_slices_from_strcrop(strcrop):
    """``'100:600, :'`` -> tuple of slices (data_objects/piv.py:71-75)."""
    return tuple(
        slice(*(int(i) if i else None for i in part.strip().split(":")))
        for part in strcrop.split(",")
    )


class ArrayCouple:
    """Couple of arrays (images), optionally masked with ``params.mask.strcrop``."""

    def __init__(self, names=None, arrays=None, params_mask=None, serie=None, paths=None,
                 hdf5_parent=None):
        if hdf5_parent is not None:
            self._load(hdf5_parent["couple"], params_mask)
            return
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
        if self.arrays is None:
            raise ValueError("a couple read from a results file holds no arrays")
        return self.arrays

    def save(self, path=None, hdf5_parent=None):
        """The ``couple`` group of a results file (data_objects/piv.py:174-189)."""
        if path is not None or hdf5_parent is None:
            raise NotImplementedError("a couple is saved inside a results file")
        group = hdf5_parent.create_group("couple")
        group.attrs["names"] = repr(tuple(self.names)).encode()
        group.attrs["paths"] = repr(self.paths).encode()
        group.create_dataset("shape_images", data=self.shape_images)

    def _load(self, group, params_mask):
        import ast

        def text(value):
            return value.decode() if isinstance(value, bytes) else str(value)

        self.params_mask = params_mask
        self.names = tuple(ast.literal_eval(text(group.attrs["names"])))
        self.paths = ast.literal_eval(text(group.attrs["paths"]))
        self.name = "-".join(self.names)
        self.serie = None
        self.arrays = None
        self.shape_images = (tuple(int(v) for v in group["shape_images"][...])
                             if "shape_images" in group else None)


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

    # ------------------------------------------------------------------ HDF5
    def _get_name(self, kind=None):
        """The file name upstream gives these results (data_objects/piv.py:349-361)."""
        serie = getattr(self.couple, "serie", None)
        if kind is None:
            if serie is None:
                return self.couple.name + ".h5"
            return get_name_piv(serie, prefix="piv")
        if kind == "bos" and serie is not None:
            return get_name_bos(self.couple.name, serie)
        raise NotImplementedError(f"file name of kind {kind!r} without a series")

    def save(self, path=None, out_format=None, kind=None):
        """Write this pass as a results file (data_objects/piv.py:363-380); returns
        its path."""
        if out_format == "uvmat":
            raise NotImplementedError("the UVmat (netCDF) format is not provided")
        name = self._get_name(kind)
        path_file = os.path.join(path, name) if path is not None else name
        with _h5py().File(path_file, "w") as file:
            file.attrs["class_name"] = "HeavyPIVResults"
            file.attrs["module_name"] = MODULE_NAME
            self._save_in_hdf5_object(file)
        return path_file

    def _save_in_hdf5_object(self, file, tag="piv0"):
        """The group ``tag`` of this pass, with the parameters and the couple written
        first if the file lacks them (data_objects/piv.py:382-455)."""
        if "class_name" not in file.attrs.keys():
            file.attrs["class_name"] = "HeavyPIVResults"
            file.attrs["module_name"] = MODULE_NAME
        if "params" not in file.keys():
            self.params._save_as_hdf5(hdf5_parent=file)
        if "couple" not in file.keys():
            self.couple.save(hdf5_parent=file)
        group = file.create_group(tag)
        group.attrs["class_name"] = "HeavyPIVResults"
        group.attrs["module_name"] = MODULE_NAME
        attrs = self.__dict__
        for key in KEYS_SAVED:
            arr = attrs.get(key)
            if arr is None:
                continue
            arr = np.asarray(arr)
            group.create_dataset(key, data=arr.astype(np.float32)
                                 if arr.dtype == np.float64 else arr)
        for name in DICTS_SAVED:
            table = attrs.get(name)
            if table is None:
                continue
            sub = group.create_group(name)
            keys, values = list(table.keys()), list(table.values())
            # as upstream: the entries are encoded when the first one is text
            if keys and isinstance(keys[0], str):
                keys = [k.encode() for k in keys]
            if values and isinstance(values[0], str):
                values = [v.encode() for v in values]
            sub.create_dataset("keys", data=keys)
            sub.create_dataset("values", data=values)
            if name == "errors":
                codes = np.full(len(values), np.iinfo(np.uint8).max, dtype=np.uint8)
                for i, text in enumerate(values):
                    for prefix, code in ERROR_CODES:
                        if text.startswith(prefix):
                            codes[i] = code
                            break
                sub.create_dataset("codes", data=codes)
        if "deltaxs_tps" in attrs:
            for comp in ("deltaxs_tps", "deltays_tps"):
                sub = group.create_group(comp)
                for i, arr in enumerate(attrs[comp]):
                    sub.create_dataset(f"subdom{i}", data=arr)

    def _load_from_hdf5_object(self, group):
        """Read a pass group written by ``_save_in_hdf5_object``."""
        for key in KEYS_SAVED:
            if key in group:
                self.__dict__[key] = group[key][...]
        for name in DICTS_SAVED:
            if name not in group:
                continue
            sub = group[name]
            keys = [k.decode() if isinstance(k, bytes) else k.item() if hasattr(k, "item")
                    else k for k in sub["keys"][...]]
            values = [v.decode() if isinstance(v, bytes) else v for v in sub["values"][...]]
            self.__dict__[name] = dict(zip(keys, values))
        if "deltaxs_tps" in group:
            for comp in ("deltaxs_tps", "deltays_tps"):
                sub = group[comp]
                count = len(list(sub.keys()))
                self.__dict__[comp] = [sub[f"subdom{i}"][...] for i in range(count)]


class MultipassPIVResults:
    """Result of a multipass PIV computation (``passes``, ``piv0``, ``piv1``...).

    ``MultipassPIVResults(str_path=path)`` reads a file written by ``save``
    (data_objects/piv.py:620-646)."""

    def __init__(self, str_path=None):
        self.passes = []
        if str_path is not None:
            self._load(str_path)

    def __getitem__(self, key):
        return self.passes[key]

    def __len__(self):
        return len(self.passes)

    def append(self, results):
        i = len(self.passes)
        self.passes.append(results)
        self.__dict__[f"piv{i}"] = results

    def _get_name(self, kind=None):
        if hasattr(self, "file_name"):
            return self.file_name
        return self.passes[0]._get_name(kind)

    def save(self, path=None, out_format=None, kind=None, version=None):
        """Write the passes as one results file (data_objects/piv.py:586-618):
        ``path`` is the file (``.h5``) or its directory (the file then gets the name
        upstream gives it); returns the file's path.  ``fluidimage_version`` records
        ``version`` (default: this package's)."""
        if out_format == "uvmat":
            raise NotImplementedError("the UVmat (netCDF) format is not provided")
        name = self._get_name(kind)
        if path is None:
            path_file = name
        elif os.path.splitext(path)[1] in (".h5", ".nc"):
            path_file = path
        else:
            path_file = os.path.join(path, name)
        if version is None:
            from . import __version__

            version = f"fluidimage_gb300 {__version__}"
        with _h5py().File(path_file, "w") as file:
            file.attrs["class_name"] = "MultipassPIVResults"
            file.attrs["module_name"] = MODULE_NAME
            file.attrs["Conventions"] = CONVENTIONS
            file.attrs["nb_passes"] = len(self.passes)
            file.attrs["fluidimage_version"] = version
            file.attrs["fluidimage_hg_rev"] = ""
            for i, r in enumerate(self.passes):
                r._save_in_hdf5_object(file, tag=f"piv{i}")
        return path_file

    def _load(self, path):
        from .params import ParamContainer

        self.file_name = os.path.basename(path)
        with _h5py().File(path, "r") as file:
            self.params = ParamContainer(hdf5_object=file["params"])
            params_mask = getattr(self.params, "mask", None)
            self.couple = ArrayCouple(hdf5_parent=file, params_mask=params_mask)
            for i in range(int(file.attrs["nb_passes"])):
                r = HeavyPIVResults(couple=self.couple, params=self.params)
                r._load_from_hdf5_object(file[f"piv{i}"])
                self.append(r)
