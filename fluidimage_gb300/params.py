"""Parameter tree with the attribute API of fluiddyn's ``ParamContainer``.

Only the subset used by the PIV works is provided: ``_set_child``,
``_set_attribs``, ``_set_doc``, attribute access and assignment restricted to
declared parameters (misspelt parameters raise ``AttributeError`` as upstream).
"""

from __future__ import annotations

import copy


class ParamContainer:
    def __init__(self, tag="params", attribs=None, doc=""):
        object.__setattr__(self, "_tag", tag)
        object.__setattr__(self, "_tag_children", [])
        object.__setattr__(self, "_key_attribs", [])
        object.__setattr__(self, "_doc", doc)
        if attribs:
            self._set_attribs(attribs)

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
