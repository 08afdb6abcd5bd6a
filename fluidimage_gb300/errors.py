"""Error carriers with the upstream semantics.

``PIVError`` mirrors ``fluidimage.calcul.errors.PIVError`` (calcul/errors.py:4-15):
keyword arguments become attributes (``explanation``, ``results``, ...).
``InterpError`` mirrors works/piv/singlepass.py:33-34.
"""


class PIVError(Exception):
    """No peak"""

    def __init__(self, *args, **kwargs):
        self.explanation = "General no peak error"
        for key, value in kwargs.items():
            self.__dict__[key] = value
        super().__init__(*args)


class InterpError(ValueError):
    pass


class GridError(ValueError, IndexError):
    """A vector grid the work cannot run on.  Upstream fails there with an
    IndexError (an empty window grid, singlepass.py:128-133; WorkFIX's neighbour
    mean on a grid narrower than 2, mean_neighbors.py:5-125); this error is an
    IndexError too, with the reason."""


ERROR_STRINGS = {
    1: "Correlation peak touching boundary.",
    2: "Correlation peak touching nan.",
    3: "wrong subpix",
    4: "Bad im_crop shape.",
    5: "Correlation plane without any finite value.",
    6: "close boundary",
}
