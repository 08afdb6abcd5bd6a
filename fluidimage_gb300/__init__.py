"""GB300-native (sm_103a) PIV hot path with the fluidimage plugin and WorkPIV API.

Importing the package is cheap: the CUDA library is loaded on first use by
``fluidimage_gb300._lib`` (and fails loudly when it is missing).
"""

__version__ = "0.1.0"
