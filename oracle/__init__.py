"""CPU oracle for the fluidimage PIV hot path — TEST INFRASTRUCTURE ONLY.

``oracle.piv`` restates, in numpy, the upstream fluidimage 0.5.3 algorithms that the
GB300 kernels replace (window grid, padding, cropping, FFT cross-correlation,
peak search, '2d_gaussian2' subpixel fit, WorkFIX, thin-plate-spline subdomain
interpolation, multipass driver).  Every function cites the upstream file:line it
follows.

Parity is pinned: ``tests/test_oracle_golden.py`` checks this restatement against
golden vectors recorded by running the upstream sources themselves
(``tests/golden/make_golden.py``).

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline arm of
``bench.py`` may import this package, and only as a checker or as the timed CPU
baseline.  The product package ``fluidimage_gb300`` never imports it.
"""
