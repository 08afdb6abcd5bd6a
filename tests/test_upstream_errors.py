"""After ``register_upstream()`` the plugin's errors are instances of the installed
fluidimage's ``PIVError`` too, so that upstream's handlers (``except PIVError`` in
works/piv/singlepass.py:328, 339 and works/piv/fix.py:202) catch them, with the
attributes upstream reads (``explanation``, ``results``).  Runs in a child process
with the upstream sources of ``baseline/_ref/src`` (skipped where they are absent)."""

import subprocess
import sys
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parents[1]
SRC = REPO / "baseline" / "_ref" / "src"

CODE = f"""
import sys
sys.path.insert(0, {str(REPO / "tests" / "golden")!r})
sys.path.insert(0, {str(REPO)!r})
import refharness
refharness.install({str(SRC)!r})
import fluidimage_gb300
from fluidimage_gb300.correl import CorrelGB300
from fluidimage_gb300.errors import PIVError
assert fluidimage_gb300.register_upstream()
from fluidimage.calcul.correl import correlation_classes
from fluidimage.calcul.errors import PIVError as UpstreamPIVError
assert correlation_classes["gb300"] is CorrelGB300
e = CorrelGB300._piv_error(explanation="Correlation peak touching boundary.")
e.results = (1, 2, 0.5)
assert isinstance(e, UpstreamPIVError) and isinstance(e, PIVError)
assert e.explanation == "Correlation peak touching boundary." and e.results == (1, 2, 0.5)
try:
    raise e
except UpstreamPIVError as caught:
    assert caught.results == (1, 2, 0.5)
d = CorrelGB300._piv_error()
assert d.explanation == "General no peak error"
print("ok")
"""


def test_plugin_errors_are_upstream_errors():
    if not (SRC / "fluidimage" / "works" / "piv").is_dir():
        pytest.skip("upstream sources not installed in baseline/_ref/src "
                    "(tests/golden/install_reference.py)")
    run = subprocess.run([sys.executable, "-c", CODE], capture_output=True, text=True,
                         timeout=300)
    assert run.returncode == 0, run.stdout + run.stderr
    assert run.stdout.strip().endswith("ok")
