"""Results files: ``MultipassPIVResults.save`` writes upstream's HDF5 layout
(data_objects/piv.py:363-455, 586-618) and ``MultipassPIVResults(str_path=...)``
reads it back.  No HDF5 library exists where the tests run, so h5py is replaced by
a recording stand-in (``tests/fake_h5py.py``).  With the upstream sources installed
(``baseline/_ref/src``), a child process saves the same results with upstream's
own writer and compares the two recorded files, then reads this package's file with
upstream's reader."""

import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

import fake_h5py
import results_fixture
from fluidimage_gb300 import ArrayCouple, HeavyPIVResults, MultipassPIVResults, WorkPIV

REPO = Path(__file__).resolve().parents[1]
SRC = REPO / "baseline" / "_ref" / "src"


@pytest.fixture
def h5(monkeypatch):
    monkeypatch.setitem(sys.modules, "h5py", fake_h5py)
    fake_h5py.FILES.clear()
    return fake_h5py


def _results():
    im = np.zeros((64, 80), np.uint16)
    couple = ArrayCouple(names=("im0.png", "im1.png"), arrays=(im, im))
    params = WorkPIV.create_default_params()
    params.multipass.number = 2
    return results_fixture.build(HeavyPIVResults, MultipassPIVResults, couple, params)


def test_layout(h5, tmp_path):
    results = _results()
    path = results.save(str(tmp_path))
    assert path == str(tmp_path / "im0.png-im1.png.h5")
    f = h5.FILES[path]
    assert f.attrs["class_name"] == "MultipassPIVResults"
    assert f.attrs["module_name"] == "fluidimage.data_objects.piv"
    assert f.attrs["Conventions"] == "fluidimage.data_objects.piv.MultipassPIVResults v1"
    assert f.attrs["nb_passes"] == 2
    assert f.keys() == ["params", "couple", "piv0", "piv1"]
    assert f["couple"].attrs["names"] == b"('im0.png', 'im1.png')"
    assert f["couple"].attrs["paths"] == b"None"
    np.testing.assert_array_equal(f["couple/shape_images"][...], [64, 80])
    g0 = f["piv0"]
    assert g0.attrs["class_name"] == "HeavyPIVResults"
    assert g0["xs"].dtype == np.float32 and g0["deltaxs"].dtype == np.float32
    assert g0["deltaxs_approx"].dtype == np.float32
    assert "deltaxs_final" not in g0 and "deltaxs_final" in f["piv1"]
    np.testing.assert_array_equal(g0["errors/keys"][...], [3, 7, 9])
    assert list(g0["errors/values"][...]) == [
        b"Correlation peak touching boundary.", b"diff neighbour too large (diff2 = 5.25)",
        b"correl < correl_min"]
    np.testing.assert_array_equal(g0["errors/codes"][...], [1, 4, 2])
    assert g0["deltaxs_wrong/values"].dtype == np.float32
    assert f["piv1/errors/keys"].shape == (0,)
    assert f["piv1/errors/codes"].dtype == np.uint8
    assert f["piv0/deltaxs_tps"].keys() == ["subdom0", "subdom1"]
    assert f["params/multipass"].attrs["number"] == 2
    assert f["params/piv0"].attrs["displacement_max"] == "None"


def test_roundtrip(h5, tmp_path):
    results = _results()
    path = results.save(str(tmp_path / "field.h5"))
    assert path.endswith("field.h5")
    back = MultipassPIVResults(str_path=path)
    assert len(back.passes) == 2 and back.file_name == "field.h5"
    assert back.couple.names == ("im0.png", "im1.png")
    assert back.couple.shape_images == (64, 80)
    assert back.params.multipass.number == 2
    assert back.params.piv0.displacement_max is None
    assert back.params.piv0.method_correl == "gb300"
    for a, b in zip(results.passes, back.passes):
        for key in ("xs", "ys", "deltaxs", "deltays", "correls_max", "deltaxs_approx",
                    "deltaxs_final", "deltays_smooth", "ixvecs_final", "xs_smooth"):
            va = getattr(a, key, None)
            if va is None:
                assert getattr(b, key, None) is None
                continue
            vb = getattr(b, key)
            assert vb.dtype == np.float32
            np.testing.assert_array_equal(vb, np.asarray(va).astype(np.float32))
        assert b.errors == a.errors
        assert b.deltaxs_wrong == a.deltaxs_wrong
        for wa, wb in zip(a.deltaxs_tps, b.deltaxs_tps):
            np.testing.assert_array_equal(wa, wb)
    # a pass alone, named from its couple
    one = results.passes[0].save(str(tmp_path))
    assert one == str(tmp_path / "im0.png-im1.png.h5")
    assert h5.FILES[one].attrs["class_name"] == "HeavyPIVResults"


def test_save_needs_h5py(monkeypatch, tmp_path):
    monkeypatch.setitem(sys.modules, "h5py", None)
    with pytest.raises(ModuleNotFoundError, match="h5py"):
        _results().save(str(tmp_path))


CHILD = f"""
import sys
sys.path.insert(0, {str(REPO / "tests" / "golden")!r})
sys.path.insert(0, {str(REPO / "tests")!r})
sys.path.insert(0, {str(REPO)!r})
import numpy as np
import refharness
refharness.install({str(SRC)!r})
import fake_h5py, results_fixture
sys.modules["h5py"] = fake_h5py
import fluidimage.data_objects.piv as up
up.h5py = fake_h5py
import fluidimage_gb300 as gb
from fluidimage_gb300 import data_objects as ours

im = np.zeros((64, 80), np.uint16)
params = gb.WorkPIV.create_default_params()
params.multipass.number = 2
mine = results_fixture.build(ours.HeavyPIVResults, ours.MultipassPIVResults,
                             ours.ArrayCouple(names=("a.png", "b.png"), arrays=(im, im)), params)
theirs = results_fixture.build(up.HeavyPIVResults, up.MultipassPIVResults,
                               up.ArrayCouple(names=("a.png", "b.png"), arrays=(im, im)), params)
p_mine = mine.save("mine.h5")
p_theirs = theirs.save("theirs.h5")
t_mine = fake_h5py.tree(fake_h5py.FILES[p_mine])
t_theirs = fake_h5py.tree(fake_h5py.FILES[p_theirs])
for t in (t_mine, t_theirs):
    for key in ("fluidimage_version", "fluidimage_hg_rev"):
        assert key in t["attrs"]
        t["attrs"][key] = None
assert list(t_mine["children"]) == list(t_theirs["children"]), (t_mine["children"].keys(), t_theirs["children"].keys())
for name in t_theirs["children"]:
    assert t_mine["children"][name] == t_theirs["children"][name], name
assert t_mine == t_theirs
# upstream's reader on this package's file
with fake_h5py.File(p_mine, "r") as f:
    for i, r in enumerate(mine.passes):
        back = up.HeavyPIVResults(hdf5_object=f[f"piv{{i}}"], couple=r.couple, params=params)
        for key in up.HeavyPIVResults._keys_to_be_saved:
            if getattr(r, key, None) is not None:
                np.testing.assert_array_equal(getattr(back, key),
                                              np.asarray(getattr(r, key)).astype(np.float32))
        assert sorted(back.errors.values()) == sorted(r.errors.values())
        assert len(back.deltaxs_tps) == len(r.deltaxs_tps)
    c = up.ArrayCouple(hdf5_parent=f)
    assert c.names == ("a.png", "b.png") and c.paths is None
print("ok")
"""


def test_same_file_as_upstream_writer(tmp_path):
    if not (SRC / "fluidimage" / "data_objects" / "piv.py").is_file():
        pytest.skip("upstream sources not installed in baseline/_ref/src "
                    "(tests/golden/install_reference.py)")
    run = subprocess.run([sys.executable, "-c", CHILD], capture_output=True, text=True,
                         timeout=300, cwd=tmp_path)
    assert run.returncode == 0, run.stdout[-3000:] + run.stderr[-3000:]
    assert run.stdout.strip().endswith("ok")


@pytest.mark.gpu
def test_save_gpu_results(h5, tmp_path):
    """A field computed on the GPU (errors, wrong vectors, TPS weights and the final
    interpolation) saved and read back."""
    from fluidimage_gb300 import workloads

    (im0, im1), _ = workloads.config2_images(shape=(512, 512))
    params = workloads.config2_params(WorkPIV.create_default_params())
    results = WorkPIV(params).calcul({"arrays": (im0, im1), "names": ("f0.png", "f1.png")})
    path = results.save(str(tmp_path))
    assert path.endswith("f0.png-f1.png.h5")
    back = MultipassPIVResults(str_path=path)
    assert len(back.passes) == len(results.passes)
    for a, b in zip(results.passes, back.passes):
        np.testing.assert_array_equal(b.deltaxs, a.deltaxs)
        np.testing.assert_array_equal(b.xs, a.xs.astype(np.float32))
        assert b.errors == a.errors
        assert len(b.deltaxs_tps) == len(a.deltaxs_tps)
        for wa, wb in zip(a.deltaxs_tps, b.deltaxs_tps):
            np.testing.assert_array_equal(wb, wa)
    last, blast = results.passes[-1], back.passes[-1]
    np.testing.assert_array_equal(blast.deltaxs_final, last.deltaxs_final.astype(np.float32))
    np.testing.assert_array_equal(blast.deltays_smooth, last.deltays_smooth.astype(np.float32))
    codes = h5.FILES[path]["piv0/errors/codes"][...]
    assert codes.shape == (len(results.passes[0].errors),)


def test_file_names_from_series():
    """Names built from a fluiddyn series (data_objects/piv.py:38-64), with a
    stand-in series of two files ``im_001a``/``im_001b``."""
    from fluidimage_gb300.data_objects import get_name_bos, get_name_piv

    class Serie:
        base_name = "im_"
        extension_file = "png"
        get_index_separators = ("_",)

        def __init__(self, tuples):
            self.tuples = tuples

        def get_slicing_tuples(self):
            return self.tuples

        def get_str_for_name_from_idim_idx(self, idim, idx):
            return f"{idx:03d}" if idim == 0 else "abcdefgh"[idx]

    assert get_name_piv(Serie([(1, 2), (0, 2)])) == "piv_001ab.h5"
    assert get_name_piv(Serie([(4, 6)])) == "piv_004-005.h5"
    assert get_name_piv(Serie([(4,)]), prefix="bos") == "bos_004.h5"
    assert get_name_bos("im_007.png", Serie([(7,)])) == "bos007.h5"
