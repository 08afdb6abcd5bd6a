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


ERROR_STRINGS = {
    1: "Correlation peak touching boundary.",
    2: "Correlation peak touching nan.",
    3: "wrong subpix",
    4: "Bad im_crop shape.",
    5: "Correlation plane without any finite value.",
    6: "close boundary",
}
