"""Snapshot frames copied on the side stream while the system steps, and
recovery images that restart a system (RecoverySystem semantics)."""
import numpy as np
import pytest

from gpu_helpers import rsa_state
from proteinsim2015_gb300 import io

pytestmark = pytest.mark.gpu


def make(psim, pos, rad, n, box=12.0, scale=4):
    g = psim.geometry(n, box, box / scale, scale)
    s = psim.System(g, psim.make_force("AO", 1.1, kT=1.0, well_depth=0.25), dt=0.002,
                    precision=psim.PRECISION_MIXED)
    s.upload(pos, rad)
    return s


def test_frame_overlaps_steps_and_recovery_restarts(psim, tmp_path):
    n = 500
    pos, rad = rsa_state(n, 12.0, seed=80)
    a, b = make(psim, pos, rad, n), make(psim, pos, rad, n)
    w = io.SnapshotWriter(a, str(tmp_path / "trial"), exact=True)
    a.step(5)
    path = w.frame(5.0)
    a.step_async(7)          # the copy of step 5's positions overlaps these steps
    w.wait()
    a.sync()
    b.step(5)
    lines = open(path).read().split("\n")
    assert lines[0] == str(n) and lines[1] == "Current Time: 5"
    got = np.array([[float(v) for v in line.split()[1:]] for line in lines[2:2 + n]]).reshape(-1)
    assert np.array_equal(got, b.download()["pos"])
    # a recovery image of step 12, read back into a fresh system: the next
    # step is firstStep, as after RecoverySystem
    rec = w.recovery(12.0, np.ones(n), rad)
    assert rec.endswith("snapshots/time-12/recovery.txt")
    c = make(psim, pos, rad, n)
    st = io.recover(c, rec)
    assert c.get_step()[0] == 0
    d = c.download()
    ref = a.download()
    for k in ("pos", "frc", "frc0"):
        assert np.array_equal(d[k], ref[k]), k
    c.step(3)
    assert np.all(np.isfinite(c.download()["pos"]))
    for s in (a, b, c):
        s.close()


def test_post_analysis_histograms_match_all_pairs(psim, tmp_path):
    n, box = 1500, 14.0   # phi ~ 0.29: clusters of many contacts closer than 1.2
    pos, rad = rsa_state(n, box, seed=81)
    s = make(psim, pos, rad, n, box=box, scale=4)
    s.step(5)
    p = s.download()["pos"].reshape(-1, 3)
    d = p[:, None, :] - p[None, :, :]
    a = np.abs(d)
    d = np.where(a > box / 2, a - box, a)      # pbcDist (utilities.cpp:79-104)
    r = np.sqrt(np.sum(d * d, axis=2))
    np.fill_diagonal(r, np.inf)
    coor = np.sum(r < 1.2, axis=1)
    files = io.post_analysis(s, str(tmp_path), ["-CH", "-CLH", "-CLC"])
    assert len(files) == 3
    assert open(files[0]).read() == io.histogram_text(coor)
    _, groups, _ = s.clusters(1.2, 4)
    assert open(files[1]).read() == io.histogram_text([len(g) for g in groups])
    assert open(files[2]).read() == io.histogram_text(coor[np.concatenate(groups)])
    s.close()


def test_device_rsa_is_the_host_rsa(psim):
    # the same trials in the same order, kept by the same rule: chunks of
    # trials evaluated in parallel give the host's sequence exactly
    from proteinsim2015_gb300 import init
    for n, phi, seed in ((20000, 0.30, 5), (3000, 0.05, 6), (5000, 0.34, 7)):
        box = (n * np.pi / 6.0 / phi) ** (1.0 / 3.0)
        host = init.rsa_native(n, box, 1.0, seed=seed)   # n < 2^17: on the host
        dev = init.rsa_native(n, box, 1.0, seed=seed, device=0)
        assert np.array_equal(host, dev), (n, phi)
        d = dev[:, None, :] - dev[None, :200, :]
        d -= box * np.round(d / box)
        r = np.sqrt(np.sum(d * d, axis=2))
        assert np.sum(r < 1.0 - 1e-12) == 200   # only the particles themselves
