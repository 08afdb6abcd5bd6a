"""Install the upstream fluidimage Python sources into ``baseline/_ref/src``.

``pip install --target baseline/_ref <fluidimage project>`` cannot build the package
here: its build backend (meson-python, with Pythran for the optional compiled
kernels) is not installed and there is no network.  The PIV path runs from the
Python sources alone (``refharness`` supplies transonic's identity ``boost`` and
small stand-ins for fluiddyn, h5py and matplotlib), so this recipe copies the
package's ``.py`` files, unmodified, into the git-ignored ``baseline/_ref/src``,
where ``tests/test_gpu_upstream.py`` finds them.

Usage: ``python tests/golden/install_reference.py <fluidimage project root>``
(the directory holding ``src/fluidimage``).
"""

from __future__ import annotations

import shutil
import sys
from pathlib import Path

REPO = Path(__file__).resolve().parents[2]
TARGET = REPO / "baseline" / "_ref" / "src"


def install(project: Path) -> Path:
    src = project / "src" / "fluidimage"
    if not (src / "works" / "piv").is_dir():
        raise SystemExit(f"{project} does not hold src/fluidimage")
    dest = TARGET / "fluidimage"
    if dest.exists():
        shutil.rmtree(dest)
    count = 0
    for path in sorted(src.rglob("*.py")):
        out = dest / path.relative_to(src)
        out.parent.mkdir(parents=True, exist_ok=True)
        shutil.copyfile(path, out)
        count += 1
    (TARGET.parent / "INSTALLED.txt").write_text(
        f"fluidimage Python sources ({count} files), unmodified, from {project}\n")
    return dest


if __name__ == "__main__":
    if len(sys.argv) != 2:
        raise SystemExit(__doc__)
    print("installed into", install(Path(sys.argv[1]).resolve()))
