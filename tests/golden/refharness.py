"""Import harness for the upstream fluidimage sources (golden-fixture generation only).

The upstream package normally needs Pythran-compiled extensions, fluiddyn, h5py and
matplotlib.  None of these is needed by the PIV numerics themselves: with transonic's
``boost`` replaced by the identity decorator, every ``@boost`` function runs as the plain
Python/numpy code it is written in ("pure-Python transonic mode"), which is the same
source Pythran compiles.  This module installs the smallest stand-ins that let
``fluidimage.works.piv``, ``fluidimage.calcul.*`` import unmodified from a read-only
source tree, so that ``make_golden.py`` can run ``WorkPIV.calcul`` and record its
outputs.

Only ``tests/golden/make_golden.py`` uses this module; nothing at test, smoke or bench
time imports it, because the upstream sources are not present where those run.
"""

from __future__ import annotations

import os
import sys
import types
from pathlib import Path

#: environment variable naming the upstream ``src`` directory (the one holding the
#: ``fluidimage`` package); ``install`` also takes the path as its argument
SRC_ENV = "FLUIDIMAGE_REFERENCE_SRC"


class _Stub(types.ModuleType):
    """Module whose missing attributes are dummy classes (enough for imports)."""

    def __getattr__(self, name):  # pragma: no cover - trivial
        if name.startswith("__"):
            raise AttributeError(name)
        value = type(name, (), {"__init__": lambda self, *a, **k: None})
        setattr(self, name, value)
        return value


class ParamContainer:
    """Attribute tree with the subset of fluiddyn's ParamContainer API used by PIV."""

    def __init__(self, tag=None, attribs=None, **kwargs):
        object.__setattr__(self, "_tag", tag)
        object.__setattr__(self, "_tag_children", [])
        object.__setattr__(self, "_key_attribs", [])
        if attribs:
            for key, value in attribs.items():
                self._set_attrib(key, value)

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
            child = ParamContainer(tag=tag, attribs=attribs)
            self._tag_children.append(tag)
            object.__setattr__(self, tag, child)
        return child

    def _set_doc(self, doc):
        object.__setattr__(self, "_doc", doc)

    def _set_internal_attr(self, key, value):
        object.__setattr__(self, key, value)

    def _get_formatted_docs(self):
        return ""

    def __setattr__(self, key, value):
        if key not in self._key_attribs and key not in self._tag_children:
            raise AttributeError(f"{key} is not a parameter of {self._tag}")
        object.__setattr__(self, key, value)


def _identity_boost(obj=None, **kwargs):
    if obj is None:
        return lambda f: f
    return obj


class _ArrayFactory:
    def __getitem__(self, item):
        return object


def install(src: Path | str | None = None):
    """Install the stand-ins and the ``fluidimage`` namespace package from the
    upstream ``src`` directory ``src`` (default: the ``FLUIDIMAGE_REFERENCE_SRC``
    environment variable)."""
    if src is None:
        src = os.environ.get(SRC_ENV)
    if not src:
        raise RuntimeError(f"give the upstream src directory (argument or ${SRC_ENV})")
    src = Path(src)
    if not (src / "fluidimage" / "works" / "piv").is_dir():
        raise RuntimeError(f"{src} does not hold the upstream fluidimage package")
    if "fluidimage" in sys.modules and getattr(sys.modules["fluidimage"], "_graft_harness", False):
        return sys.modules["fluidimage"]
    sys.dont_write_bytecode = True

    transonic = types.ModuleType("transonic")
    transonic.boost = _identity_boost
    transonic.Array = _ArrayFactory()
    transonic.Type = lambda *args: object
    transonic.jit = _identity_boost

    class Transonic:
        is_compiled = False

        def __init__(self, *args, **kwargs):
            pass

    transonic.Transonic = Transonic
    sys.modules["transonic"] = transonic

    fluiddyn = _Stub("fluiddyn")
    fluiddyn_util = _Stub("fluiddyn.util")
    paramcontainer = types.ModuleType("fluiddyn.util.paramcontainer")
    paramcontainer.ParamContainer = ParamContainer
    serieofarrays = _Stub("fluiddyn.util.serieofarrays")
    fluiddyn.util = fluiddyn_util
    fluiddyn_util.paramcontainer = paramcontainer
    fluiddyn_util.serieofarrays = serieofarrays
    sys.modules.update(
        {
            "fluiddyn": fluiddyn,
            "fluiddyn.util": fluiddyn_util,
            "fluiddyn.util.paramcontainer": paramcontainer,
            "fluiddyn.util.serieofarrays": serieofarrays,
        }
    )
    for name in ("h5py", "h5netcdf", "matplotlib", "matplotlib.pyplot"):
        sys.modules[name] = _Stub(name)

    pkg = types.ModuleType("fluidimage")
    pkg.__path__ = [str(src / "fluidimage")]
    pkg.ParamContainer = ParamContainer
    pkg.__version__ = "0.5.3"
    pkg.imread = lambda path: None
    pkg._graft_harness = True
    sys.modules["fluidimage"] = pkg

    version = types.ModuleType("fluidimage._version")
    version.__version__ = "0.5.3"
    version.hg_rev = "?"
    sys.modules["fluidimage._version"] = version

    util = types.ModuleType("fluidimage.util")
    util.safe_eval = eval
    sys.modules["fluidimage.util"] = util
    return pkg
