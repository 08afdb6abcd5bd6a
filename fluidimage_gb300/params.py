"""Parameter tree with the attribute API of fluiddyn's ``ParamContainer``.

Only the subset used by the PIV works is provided: ``_set_child``,
``_set_attribs``, ``_set_doc``, attribute access and assignment restricted to
declared parameters (misspelt parameters raise ``AttributeError`` as upstream),
and the HDF5 group of a results file (``_save_as_hdf5``, ``hdf5_object=``).
"""

from __future__ import annotations

import copy

import numpy as np


class ParamContainer:
    def __init__(self, tag="params", attribs=None, doc="", hdf5_object=None):
        object.__setattr__(self, "_tag", tag)
        object.__setattr__(self, "_tag_children", [])
        object.__setattr__(self, "_key_attribs", [])
        object.__setattr__(self, "_doc", doc)
        if hdf5_object is not None:
            self._load_from_hdf5_object(hdf5_object)
        if attribs:
            self._set_attribs(attribs)

    # ------------------------------------------------------------------ HDF5
    def _save_as_hdf5(self, path_file=None, hdf5_parent=None):
        """The tree as HDF5 groups (one per container, named by its tag) whose
        attributes are the parameters: None is stored as the text ``"None"``,
        sequences as arrays.  This restates the layout of fluiddyn's
        ``ParamContainer._save_as_hdf5`` (fluiddyn is not a dependency here; a tree
        built by fluiddyn saves itself)."""
        if hdf5_parent is None:
            from .data_objects import _h5py

            with _h5py().File(path_file, "w") as file:
                self._save_as_hdf5(hdf5_parent=file)
            return
        group = hdf5_parent.create_group(self._tag)
        for key in self._key_attribs:
            value = getattr(self, key)
            if value is None:
                value = "None"
            elif isinstance(value, (list, tuple)):
                value = np.asarray(value)
            elif isinstance(value, dict):
                value = repr(value)
            group.attrs[key] = value
        for tag in self._tag_children:
            getattr(self, tag)._save_as_hdf5(hdf5_parent=group)

    def _load_from_hdf5_object(self, group):
        for key, value in group.attrs.items():
            if isinstance(value, bytes):
                value = value.decode()
            if isinstance(value, str) and value == "None":
                value = None
            elif isinstance(value, np.ndarray):
                value = value.tolist()
            elif isinstance(value, np.generic):
                value = value.item()
            self._set_attrib(key, value)
        for tag in group.keys():
            child = ParamContainer(tag=tag, hdf5_object=group[tag])
            self._tag_children.append(tag)
            object.__setattr__(self, tag, child)

    def _set_attrib(self, key, value):
        if key not in self._key_attribs:
            self._key_attribs.append(key)
        object.__setattr__(self, key, value)

    def _set_attribs(self, attribs):
        for key, value in attribs.items():
            self._set_attrib(key, value)

    def _set_child(self, tag, attribs=None, doc=None):
        if tag in self._tag_children:
            child = getattr(self, tag)
            if attribs:
                child._set_attribs(attribs)
        else:
            child = ParamContainer(tag=tag, attribs=attribs, doc=doc or "")
            self._tag_children.append(tag)
            object.__setattr__(self, tag, child)
        return child

    def _set_doc(self, doc):
        object.__setattr__(self, "_doc", doc)

    def _get_formatted_docs(self):
        return self._doc

    def __setattr__(self, key, value):
        if key not in self._key_attribs and key not in self._tag_children:
            raise AttributeError(
                f"{key!r} is not a parameter of {self._tag!r} "
                f"(parameters: {self._key_attribs}, children: {self._tag_children})"
            )
        object.__setattr__(self, key, value)

    def __deepcopy__(self, memo):
        new = ParamContainer(tag=self._tag, doc=self._doc)
        for key in self._key_attribs:
            new._set_attrib(key, copy.deepcopy(getattr(self, key), memo))
        for tag in self._tag_children:
            child = copy.deepcopy(getattr(self, tag), memo)
            new._tag_children.append(tag)
            object.__setattr__(new, tag, child)
        return new

    def __eq__(self, other):
        if not isinstance(other, ParamContainer):
            return NotImplemented
        return (
            self._key_attribs == other._key_attribs
            and self._tag_children == other._tag_children
            and all(getattr(self, k) == getattr(other, k) for k in self._key_attribs)
            and all(getattr(self, k) == getattr(other, k) for k in self._tag_children)
        )

    def __repr__(self):
        items = ", ".join(f"{k}={getattr(self, k)!r}" for k in self._key_attribs)
        kids = ", ".join(self._tag_children)
        return f"<ParamContainer {self._tag}: {items}; children: {kids}>"
