"""Recovery and XYZ files in the reference's formats (host side, no GPU)."""
import os

import numpy as np

from proteinsim2015_gb300 import io


def _state(n, seed=0):
    rng = np.random.default_rng(seed)
    return {k: rng.uniform(-3, 110, 3 * n) for k in ("pos", "pos0", "frc", "frc0")}


def test_recovery_round_trip_exact(tmp_path):
    st = _state(50)
    mass, rad = np.full(50, 1.0), np.full(50, 0.5)
    p = tmp_path / "recovery.txt"
    io.write_recovery(p, st, mass, rad, exact=True)
    text = p.read_text()
    assert not text.endswith("\n") and text.count("\n") == 49   # writeSystem's layout
    assert all(len(line.split()) == 14 for line in text.split("\n"))
    back = io.read_recovery(p)
    for k in st:
        assert np.array_equal(back[k], st[k])
    assert np.array_equal(back["mass"], mass) and np.array_equal(back["radius"], rad)


def test_default_format_is_the_streams_six_digits(tmp_path):
    st = {"pos": np.array([1.23456789, 1e-7, 123456789.0]), "pos0": np.array([0.0, -0.5, 2.0]),
          "frc": np.array([1.0, 2.5, -1e10]), "frc0": np.array([3.0, 4.0, 5.0])}
    p = tmp_path / "r.txt"
    io.write_recovery(p, st, [1.0], [0.5])
    assert p.read_text() == "1.23457 1e-07 1.23457e+08 0 -0.5 2 1 2.5 -1e+10 3 4 5 1 0.5"


def test_xyz_frame(tmp_path):
    p = tmp_path / "f.xyz"
    io.write_xyz(p, [0.5, 1.25, 2.0, 3.0, 4.0, 5.123456789], 99.6)
    assert p.read_text() == "2\nCurrent Time: 100\nH 0.5 1.25 2\nH 3 4 5.12346\n"
    io.write_series(tmp_path / "s.txt", 10.0, 0.25)
    io.write_series(tmp_path / "s.txt", 20.0, 0.5)
    assert (tmp_path / "s.txt").read_text() == "10 0.25\n20 0.5\n"


class _FakeSystem:
    """Stands in for a System: fixed coordination numbers and clusters."""

    def __init__(self, coor, groups):
        self.coor = np.asarray(coor, np.int32)
        self.groups = [np.asarray(g) for g in groups]

    def clusters(self, r_contact=1.2, min_size=4):
        return None, self.groups, 0

    def interactions(self, r_contact=1.2):
        return self.coor, int(self.coor.sum())


def test_post_analysis_histograms(tmp_path):
    from proteinsim2015_gb300 import io
    coor = [0, 2, 2, 3, 1, 2, 5, 2, 3, 3, 1, 0]
    groups = [[1, 2, 3, 5, 6], [7, 8, 9, 10, 11, 0]]
    files = io.post_analysis(_FakeSystem(coor, groups), str(tmp_path), ["-CH", "--clusthist",
                                                                        "-CLC", "--other"])
    names = [os.path.basename(f) for f in files]
    assert names == ["coordinationHistogram.txt", "clusterSizeHistogram.txt",
                     "clusterCoorHistogram.txt"]
    read = {n: open(os.path.join(str(tmp_path), n)).read() for n in names}
    assert read["coordinationHistogram.txt"] == "0 2\n1 2\n2 4\n3 3\n5 1\n"
    assert read["clusterSizeHistogram.txt"] == "5 1\n6 1\n"
    # members 1 2 3 5 6 7 8 9 10 11 0 -> coor 2 2 3 2 5 2 3 3 1 0 0
    assert read["clusterCoorHistogram.txt"] == "0 2\n1 1\n2 4\n3 3\n5 1\n"
