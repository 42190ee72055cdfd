"""The analysis subsystems against the reference's own output on the same
state (tests/golden/reference_analysis.npz, written by the reference rebuilt
from its sources): updateInteractions' coordination numbers
(systemHandling.cpp:94-161), findClusters' clusters (analysisCluster.cpp:
26-83), getTemperature / meanDisplacement / <EAP> (analysisGeneral.cpp:26-55,
analysisOutput.cpp:117-123), and the recovery.txt and .xyz files of
writeSystem / writeSystemXYZ (analysisOutput.cpp:31-74)."""
import os

import numpy as np
import pytest

from conftest import ROOT
from proteinsim2015_gb300 import io as pio

pytestmark = pytest.mark.gpu

NPZ = os.path.join(ROOT, "tests", "golden", "reference_analysis.npz")


@pytest.fixture(scope="module")
def ref_state():
    return np.load(NPZ)


def _system(psim, d, precision, skin=0.0, force=None):
    n, box, cs, scale = (int(v) for v in d["geom"])
    g = psim.geometry(n, box, cs, scale)
    f = force or psim.make_force("AO", 1.1, kT=1.0, well_depth=0.25)
    s = psim.System(g, f, gamma=1.0, dt=0.001, kT=1.0, precision=precision, skin=skin)
    s.upload(d["pos"], d["radius"], mass=d["mass"], vel=d["vel"], pos0=d["pos0"], frc=d["frc"],
             frc0=d["frc0"])
    return s


@pytest.mark.parametrize("precision,skin", [(0, 0.0), (1, 0.0), (1, "auto")])
def test_coordination_numbers_are_the_references(psim, ref_state, precision, skin):
    # FP64: counted inside the force pass with the reference's test; mixed:
    # in FP32 inside the pass (no list), or by the separate FP64 walk (the AO
    # pair list's cutoff 1.1 is below the contact distance 1.2)
    s = _system(psim, ref_state, precision, skin)
    coor, total = s.interactions(1.2)
    want = ref_state["coor"]
    if precision == 0 or skin == "auto":
        assert np.array_equal(coor, want)
    else:   # FP32 separations: a pair within ~1e-6 of 1.2 may count differently
        assert np.count_nonzero(coor != want) <= 2
    assert total == int(np.sum(coor))
    s.close()


def test_clusters_are_the_references(psim, ref_state):
    s = _system(psim, ref_state, 0)
    root, groups, avg = s.clusters(1.2, 4)
    clu = ref_state["cluster_of"]
    assert len(groups) == int(ref_state["n_clusters"])
    for k, grp in enumerate(groups):   # findClusters' order: by smallest member
        assert np.array_equal(np.sort(grp), np.flatnonzero(clu == k))
    sizes = [len(g) for g in groups]
    assert avg == sum(sizes) // len(sizes)   # writeClusters' integer mean
    s.close()


def test_observables_are_the_references(psim, ref_state):
    s = _system(psim, ref_state, 0)
    T, msd, eap = ref_state["stats"]
    assert s.temperature() == pytest.approx(T, rel=1e-12)
    assert s.mean_displacement() == pytest.approx(msd, rel=1e-12)
    # <EAP>: per particle in FP32 as particle::calculatePotential; the
    # reference also sums the particles in FP32, here the sum is FP64
    assert s.potential() == pytest.approx(eap, rel=1e-5)
    s.close()


def test_recovery_and_xyz_files_are_the_references(psim, ref_state, tmp_path):
    s = _system(psim, ref_state, 0)
    st = s.download()
    s.close()
    for k in ("pos", "pos0", "frc", "frc0"):
        assert np.array_equal(st[k], ref_state[k])
    rec = tmp_path / "recovery.txt"
    pio.write_recovery(str(rec), st, ref_state["mass"], ref_state["radius"])
    assert rec.read_text() == str(ref_state["recovery_txt"])
    xyz = tmp_path / "frame.xyz"
    pio.write_xyz(str(xyz), st["pos"], float(ref_state["time"]))
    assert xyz.read_text() == str(ref_state["xyz"])
    # and back: the recovery file read as the reference's readParticles does
    back = pio.read_recovery(str(rec))
    assert np.allclose(back["pos"], st["pos"], rtol=1e-5, atol=1e-4)


def test_fused_count_in_the_mixed_pair_list(psim):
    # a pair list of cutoff 2.5 >= 1.2 holds every contact: the count comes
    # out of the list pass itself; against the FP64 form's exact count it may
    # differ only on pairs within FP32 rounding of 1.2
    from proteinsim2015_gb300 import init
    n, box, scale = 6000, 21.5, 7          # rho 0.6, below the RSA jamming density
    pos = init.rsa(n, box, 1.0, seed=41).reshape(-1)
    g = psim.geometry(n, box, box / scale, scale)
    lj = psim.make_force("LJ", 2.5, kT=1.5, well_depth=1 / 1.5, lj_num=6, yukawa_strength=0.0)
    s = psim.System(g, lj, precision=psim.PRECISION_MIXED, skin="auto")
    assert s.skin > 0
    s.upload(pos, np.full(n, 0.5))
    fused, tf = s.interactions(1.2)
    s.close()
    s64 = psim.System(g, lj, precision=psim.PRECISION_FP64)
    s64.upload(pos, np.full(n, 0.5))
    exact, te = s64.interactions(1.2)
    s64.close()
    assert np.count_nonzero(fused != exact) <= 2 and abs(tf - te) <= 4
