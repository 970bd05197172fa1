"""The VTK writer (gbmhd/vtk.py): a file of order 2 with eight linear sub-hexahedra per cell over
its 27 nodes, read back array by array (CPU)."""
import numpy as np

from gbmhd.vtk import FIELDS, read_vtu_arrays, sub_hexes, write_vtu


def test_sub_hexes_cover_the_cell_once():
    h = sub_hexes()
    assert h.shape == (8, 8)
    # every node of the 3x3x3 lattice appears; the centre node in all eight sub-cells
    counts = np.bincount(h.ravel(), minlength=27)
    assert counts[13] == 8 and counts[0] == 1 and counts.sum() == 64


def test_vtu_round_trip(tmp_path):
    rng = np.random.default_rng(0)
    nf = rng.standard_normal((5, 27, 13))
    path = write_vtu(str(tmp_path / "f.vtu"), nf)
    a = read_vtu_arrays(path)
    assert np.array_equal(a["Points"], nf[:, :, 0:3].reshape(-1, 3))
    for name, sl in FIELDS:
        got = a[name]
        want = nf[:, :, sl].reshape(-1, sl.stop - sl.start)
        assert np.array_equal(got.reshape(want.shape), want), name
    assert a["connectivity"].max() == 5 * 27 - 1 and len(a["connectivity"]) == 5 * 8 * 8
    assert np.array_equal(a["offsets"], 8 * np.arange(1, 41))
    assert np.all(a["types"] == 12)
