"""In-memory stand-in for the part of h5py's API that PIV results files use (no
HDF5 library exists where the tests run).  ``File(path, "w")`` records a tree of
groups, datasets and attributes under ``path``; ``File(path, "r")`` returns it.
Values are stored as h5py would hand them back: datasets as numpy arrays (lists
converted by ``np.asarray``), sequence attributes as arrays.  Test infrastructure
only."""

from __future__ import annotations

import numpy as np

FILES: dict = {}


class Attrs(dict):
    def __setitem__(self, key, value):
        if isinstance(value, (list, tuple)):
            value = np.asarray(value)
        super().__setitem__(key, value)


class Dataset:
    def __init__(self, name, data, parent):
        self.name = name
        self.parent = parent
        self.data = np.array(np.asarray(data))
        self.attrs = Attrs()
        self.dtype = self.data.dtype
        self.shape = self.data.shape

    def __getitem__(self, item):
        return self.data[item]

    def __iter__(self):
        return iter(self.data)

    def __len__(self):
        return len(self.data)


class Group:
    def __init__(self, name="/", parent=None):
        self.name = name
        self.parent = parent if parent is not None else self
        self.attrs = Attrs()
        self.children = {}

    def _new(self, name, node):
        if name in self.children:
            raise ValueError(f"name already exists: {name}")
        self.children[name] = node
        return node

    def create_group(self, name):
        return self._new(name, Group(self._path(name), self))

    def create_dataset(self, name, data=None):
        return self._new(name, Dataset(self._path(name), data, self))

    def _path(self, name):
        return (self.name.rstrip("/") + "/" + name) if self.name != "/" else "/" + name

    def __getitem__(self, path):
        node = self
        for part in path.strip("/").split("/"):
            node = node.children[part]
        return node

    def __contains__(self, name):
        try:
            self[name]
        except KeyError:
            return False
        return True

    def keys(self):
        return list(self.children)

    def items(self):
        return list(self.children.items())

    def __iter__(self):
        return iter(self.children)


class File(Group):
    def __init__(self, path, mode="r"):
        path = str(path)
        if mode == "w":
            super().__init__()
            FILES[path] = self
        elif mode == "r":
            src = FILES[path]
            super().__init__()
            self.attrs, self.children = src.attrs, src.children
            for node in self.children.values():
                node.parent = self
        else:
            raise ValueError(f"mode {mode!r}")

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        return False


def tree(node):
    """Nested plain description of a recorded node (for comparisons)."""
    out = {"attrs": {k: _plain(v) for k, v in node.attrs.items()}}
    if isinstance(node, Dataset):
        out["dtype"] = node.dtype.str if node.dtype.kind != "S" else "S"
        out["data"] = _plain(node.data)
    else:
        out["children"] = {k: tree(v) for k, v in node.children.items()}
    return out


def _plain(value):
    if isinstance(value, np.ndarray):
        return ("array", value.dtype.kind, value.shape, value.tolist())
    if isinstance(value, np.generic):
        return value.item()
    return value
