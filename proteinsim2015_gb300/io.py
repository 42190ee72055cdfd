"""Snapshot and recovery files in the reference's formats.

    write_recovery   analysisManager::writeSystem (analysisOutput.cpp:53-74):
                     one line per particle, 14 space-separated columns
                     x y z x0 y0 z0 fx fy fz fx0 fy0 fz0 mass radius,
                     no newline after the last line
    read_recovery    system::readParticles (systemRecovery.cpp:43-81)
    write_xyz        analysisManager::writeSystemXYZ (analysisOutput.cpp:31-51)
    write_series     analysisManager::writeToStream (analysisOutput.cpp:91-97)
    SnapshotWriter   the snapshot directory layout of writeSystemState
                     (analysisOutput.cpp:99-114), with the positions copied to
                     the host on a side stream while the steps go on
    post_analysis    analysisManager::postAnalysis (analysisPost.cpp:26-52): the
                     coordination, cluster-size and cluster-coordination
                     histograms (analysisCluster.cpp:135-203) of the device state

The reference writes doubles with the stream's default format (6 significant
digits, as printf's %g), so its recovery files hold 6 digits; ``exact=True``
writes 17 so that a recovered state continues bit for bit.
"""
import os
import threading

import numpy as np

DEFAULT_FMT = "%g"
EXACT_FMT = "%.17g"


def _fmt(exact):
    return EXACT_FMT if exact else DEFAULT_FMT


def write_recovery(path, state, mass, radius, exact=False):
    """state: a System.download() dict (pos, pos0, frc, frc0: 3n each)."""
    n = len(radius)
    cols = [np.asarray(state[k], dtype=np.float64).reshape(n, 3) for k in ("pos", "pos0", "frc",
                                                                          "frc0")]
    table = np.hstack(cols + [np.asarray(mass, np.float64).reshape(n, 1),
                              np.asarray(radius, np.float64).reshape(n, 1)])
    f = _fmt(exact)
    lines = [" ".join(f % v for v in row) for row in table]
    with open(path, "w") as fh:
        fh.write("\n".join(lines))


def read_recovery(path):
    """The 14 columns back: dict of pos, pos0, frc, frc0 (3n), mass, radius (n).
    The reference reads mass and radius into floats (systemRecovery.cpp:63)."""
    table = np.loadtxt(path, ndmin=2)
    if table.shape[1] != 14:
        raise ValueError("%s: expected 14 columns, found %d" % (path, table.shape[1]))
    out = {k: table[:, 3 * j:3 * j + 3].reshape(-1).copy()
           for j, k in enumerate(("pos", "pos0", "frc", "frc0"))}
    out["mass"] = table[:, 12].astype(np.float32).astype(np.float64)
    out["radius"] = table[:, 13].astype(np.float32).astype(np.float64)
    return out


def write_xyz(path, pos, current_time, exact=False):
    """XYZ frame: count, 'Current Time: <rounded time>', then 'H x y z' lines."""
    p = np.asarray(pos, dtype=np.float64).reshape(-1, 3)
    f = _fmt(exact)
    with open(path, "w") as fh:
        fh.write("%d\n" % len(p))
        fh.write("Current Time: %d\n" % int(round(current_time)))
        for x, y, z in p:
            fh.write("H %s %s %s\n" % (f % x, f % y, f % z))


def write_series(path, current_time, value):
    """One 'time value' line appended to a time series file."""
    with open(path, "a") as fh:
        fh.write("%s %s\n" % (DEFAULT_FMT % current_time, DEFAULT_FMT % value))


def recover(system, path, exact_velocities=None):
    """Upload a recovery file into a System: like RecoverySystem the next step
    is the integrator's firstStep (the step counter restarts at 0) and the
    velocities are zero unless given."""
    st = read_recovery(path)
    system.upload(st["pos"], st["radius"], mass=st["mass"], vel=exact_velocities,
                  pos0=st["pos0"], frc=st["frc"], frc0=st["frc0"])
    return st


class SnapshotWriter:
    """Movie frames and recovery images in the reference's layout:

        <trial>/movie/system-<t>.xyz
        <trial>/snapshots/time-<t>/recovery.txt

    frame() starts a device-to-host copy of the positions on the system's side
    stream and returns at once; the file is written by a host thread after
    the copy, while the GPU keeps stepping.  recovery() downloads the whole
    state (synchronous)."""

    def __init__(self, system, trial, exact=False):
        self.system = system
        self.trial = trial
        self.exact = exact
        os.makedirs(os.path.join(trial, "movie"), exist_ok=True)
        os.makedirs(os.path.join(trial, "snapshots"), exist_ok=True)
        self._host = np.empty(3 * system.n)
        self._thread = None

    def _name(self, t):
        return str(int(round(t)))

    def frame(self, current_time):
        self.wait()
        self.system.snapshot_async(self._host)
        path = os.path.join(self.trial, "movie", "system-%s.xyz" % self._name(current_time))

        def finish(buf=self._host):
            self.system.snapshot_wait()
            write_xyz(path, buf, current_time, self.exact)

        self._thread = threading.Thread(target=finish)
        self._thread.start()
        return path

    def recovery(self, current_time, mass, radius):
        self.wait()
        d = os.path.join(self.trial, "snapshots", "time-%s" % self._name(current_time))
        os.makedirs(d, exist_ok=True)
        path = os.path.join(d, "recovery.txt")
        write_recovery(path, self.system.download(), mass, radius, self.exact)
        return path

    def wait(self):
        if self._thread is not None:
            self._thread.join()
            self._thread = None


def histogram_text(values):
    """The reference's histogram file: "key count" per line for every value
    that occurs, keys ascending (a std::map<int, int> written in order)."""
    keys, counts = np.unique(np.asarray(values, dtype=np.int64), return_counts=True)
    return "".join("%d %d\n" % (k, c) for k, c in zip(keys, counts))


POST_TESTS = {
    "--coorhist": "coordinationHistogram.txt", "-CH": "coordinationHistogram.txt",
    "--clusthist": "clusterSizeHistogram.txt", "-CLH": "clusterSizeHistogram.txt",
    "--clustcoor": "clusterCoorHistogram.txt", "-CLC": "clusterCoorHistogram.txt",
}


def post_analysis(system, trial_name, tests, r_contact=1.2):
    """analysisManager::postAnalysis (analysisPost.cpp:26-52) on a System: the
    clusters of more than 4 particles in contact (findClusters,
    analysisCluster.cpp:26-83), then for each test flag in order
      --coorhist  / -CH   coordinationHistogram.txt: particles per
                          coordination number (analysisCluster.cpp:184-203)
      --clusthist / -CLH  clusterSizeHistogram.txt: clusters per size
                          (analysisCluster.cpp:135-156)
      --clustcoor / -CLC  clusterCoorHistogram.txt: the clustered particles
                          per coordination number (analysisCluster.cpp:158-182)
    Coordination numbers are those of updateInteractions (contacts closer than
    r_contact, systemHandling.cpp:94-161).  Returns the files written."""
    _, groups, _ = system.clusters(r_contact, 4)
    coor, _ = system.interactions(r_contact)
    coor = np.asarray(coor)
    written = []
    for t in tests:
        name = POST_TESTS.get(t)
        if name is None:
            continue
        if name == "coordinationHistogram.txt":
            text = histogram_text(coor)
        elif name == "clusterSizeHistogram.txt":
            text = histogram_text([len(g) for g in groups])
        else:
            members = np.concatenate(groups) if groups else np.empty(0, np.int64)
            text = histogram_text(coor[members])
        path = os.path.join(trial_name, name)
        with open(path, "w") as fh:
            fh.write(text)
        written.append(path)
    return written
