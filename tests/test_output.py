"""HDF5/XDMF output (pylbm/hdf5.py H5File) read back by the golden-file reader."""
import os
import sys

import numpy as np
import pytest

from pylbm_gb300.output import H5File, write_h5

sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))
import h5lite  # noqa: E402


def test_datasets_round_trip(tmp_path):
    rng = np.random.default_rng(0)
    data = {"rho": rng.normal(size=(16, 8)), "x_0": np.linspace(0, 1, 8), "qz": rng.normal(size=(3, 4, 5)),
            "scalar_like": np.array([2.5])}
    path = str(tmp_path / "f.h5")
    write_h5(path, data)
    back = h5lite.read(path)
    assert sorted(back) == sorted(data)
    for k, v in data.items():
        assert back[k].shape == v.shape and np.array_equal(back[k], v)


def test_h5file_layout_matches_pylbm(tmp_path):
    x, y = np.linspace(0.5, 7.5, 8) / 8, np.linspace(0.5, 3.5, 4) / 4
    rho = np.add.outer(x, 10 * y)
    h5 = H5File(None, "sol", str(tmp_path), 3)
    h5.set_grid(x, y)
    h5.add_scalar("rho", rho)
    h5.add_vector("velocity", [rho, 2 * rho])
    h5.save()
    back = h5lite.read(str(tmp_path / "sol_3.h5"))
    assert np.array_equal(back["x_0"], x) and np.array_equal(back["x_1"], y)
    assert np.array_equal(back["rho"], rho.T)  # stored transposed, as pylbm does
    assert back["velocity"].shape == (4, 8, 3) and np.array_equal(back["velocity"][..., 1], 2 * rho.T)
    xdmf = (tmp_path / "sol_3.xdmf").read_text()
    assert '"2DRectMesh" NumberOfElements="8 4"' in xdmf and "sol_3.h5:/rho" in xdmf


def test_reads_the_same_structure_as_pylbm_files(tmp_path):
    """Our file has the message set h5py writes for the reference's goldens."""
    path = str(tmp_path / "g.h5")
    write_h5(path, {"a": np.ones((4, 2))})
    f = h5lite._File(open(path, "rb").read())
    _, header, cache, _ = f.entry(f.root_entry)
    assert cache == 1
    (name, addr), = f.group_entries(*np.frombuffer(f.entry(f.root_entry)[3], dtype="<u8"))
    assert name == "a"
    assert [m[0] for m in f.messages(addr)] == [0x0001, 0x0003, 0x0005, 0x0008, 0x0012]


def test_box_arguments_of_interior_indices():
    """Index normalisation behind sim.m[key, ...] (no GPU)."""
    from pylbm_gb300.simulation import Simulation

    class Fake:
        dim = 2

        class domain:
            shape_in = [10, 6]
    box = Simulation._box_args
    assert box(Fake, (slice(None), 2)) == ([0, 2], [10, 1], [1, 1], (1,))
    assert box(Fake, (slice(8, 1, -3), -1)) == ([8, 5], [3, 1], [-3, 1], (1,))
    assert box(Fake, (3,)) == ([3, 0], [1, 6], [1, 1], (0,))
    for bad in [(10, 0), (0, slice(4, 4)), (0, 0, 0)]:
        with pytest.raises(IndexError):
            box(Fake, bad)
