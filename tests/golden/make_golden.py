"""Generate tests/golden/*.npz from the reference itself.

The reference (SawyerHopkins/ProteinSim2015) ships no tests, fixtures or
golden vectors, so these are produced by running its own hot-path code,
rebuilt from its sources by oracle/build_ref.sh (oracle/_ref), on seeded
inputs.  Inputs are stored next to the outputs so the fixtures stand alone
(the GPU machine has no reference tree).

    python tests/golden/make_golden.py [--settings-only]

--settings-only writes the settings and analysis fixtures but not
reference_hotpath.npz.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import ref  # noqa: E402
from proteinsim2015_gb300 import init  # noqa: E402


def state_small(n, box, seed):
    pos = init.rsa(n, box, 1.0, seed=seed)
    return pos.reshape(-1), np.full(n, 0.5)


# settings.cfg texts whose run constants the reference derives
# (system::setSystemConstants): its own ClusteredUI/settings.cfg, read from the
# reference tree, and synthetic ones around the integer-box quantisation
SETTINGS_CASES = {
    "c0_scale7": "nParticles = 4000\nconc = 0.2\nscale = 7\nradius = 0.5\n",
    "c0_scale4": "nParticles = 4000\nconc = 0.2\nscale = 4\n",
    "c0_scale3": "nParticles = 4000\nconc = 0.2\nscale = 3\nradius = 0.5\nmass = 2\n",
    "big_radius": "nParticles = 1000\nconc = 0.1\nscale = 5\nradius = 0.75\n",
    "defaults": "force = AOPotential\n",
}


def settings_fixtures():
    """reference_settings.npz: settings texts and the (nParticles, boxSize,
    cellSize, cellScale) and concentration the reference derives from each."""
    out = {}
    cases = dict(SETTINGS_CASES)
    with open(os.path.join(ref.REFERENCE, "ClusteredUI", "settings.cfg")) as fh:
        cases["reference_settings_cfg"] = fh.read()
    for key, text in cases.items():
        path = ref.write_settings({})
        with open(path, "w") as fh:
            fh.write(text)
        try:
            n, box, cell, scale, conc = ref.system_constants(path)
        finally:
            os.unlink(path)
        out["text_" + key] = np.array(text)
        out["ints_" + key] = np.array([n, box, cell, scale], np.int64)
        out["conc_" + key] = np.array(conc)
    path = os.path.join(HERE, "reference_settings.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes")


def analysis_fixtures():
    """reference_analysis.npz: an aggregated AO state (N = 2000, L = 18, 6
    cells a side, 4 kT contact attraction, 2,000 steps of the oracle's loop
    driven by the reference's own noise stream) and the reference's analysis
    of it: updateInteractions' coordination numbers, findClusters' clusters,
    getTemperature / meanDisplacement / <EAP>, and the text of writeSystem's
    recovery.txt and writeSystemXYZ's .xyz frame."""
    import tempfile
    from oracle import port
    port.build()
    port.set_threads(os.cpu_count() or 1)
    n, box, cs, scale, dt, steps = 2000, 18, 3, 6, 0.001, 2000   # box = cs * scale
    pos, rad = state_small(n, box, seed=29)
    vel = init.maxwell(n, 1.0, seed=29).reshape(-1)
    st = port.State(pos, rad, vel=vel)
    noise = port.ReferenceNoise(n, 90210)
    err, *_ = port.run(port.geom(n, box, cs, scale),
                       port.make_force(port.AO, 1.1, kT=1.0, well_depth=0.25),
                       port.vgb_coeffs(1.0, dt, 1.0), dt, st, steps, noise.take(steps),
                       vel_freq=0)
    assert err == 0
    d = tempfile.mkdtemp(prefix="psimref_analysis_")
    prefix = os.path.join(d, "recovery")
    t = steps * dt
    coor, clu, nc, stats = ref.analysis(n, box, cs, scale, st.pos, st.pos0, st.vel, st.frc,
                                        st.frc0, rad, st.mass, t, prefix)
    with open(prefix + ".txt") as fh:
        recovery = fh.read()
    with open(prefix + ".xyz") as fh:
        xyz = fh.read()
    out = dict(geom=np.array([n, box, cs, scale]), time=np.array(t), pos=st.pos, pos0=st.pos0,
               vel=st.vel, frc=st.frc, frc0=st.frc0, radius=rad, mass=st.mass,
               coor=coor, cluster_of=clu, n_clusters=np.array(nc), stats=stats,
               recovery_txt=np.array(recovery), xyz=np.array(xyz))
    path = os.path.join(HERE, "reference_analysis.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes", "clusters", nc, "mean coor", coor.mean())


def main():
    if not ref.available():
        if not ref.build():
            sys.exit("reference sources not found; cannot generate golden fixtures")
    settings_fixtures()
    analysis_fixtures()
    if "--settings-only" in sys.argv:
        return
    out = {}
    # ---- case A: AO-type state, L=12, cellSize 3, scale 4 (N=300)
    n, box, cs, scale = 300, 12, 3, 4
    pos, rad = state_small(n, box, seed=11)
    hi, cse, srt = ref.build_cells(n, box, cs, scale, pos, rad)
    pr = hi.reshape(-1, 2)
    order = np.lexsort((pr[:, 1], pr[:, 0]))  # the reference's sort is unstable
    out.update(cellsA_pos=pos, cellsA_radius=rad, cellsA_geom=np.array([n, box, cs, scale]),
               cellsA_hash_index=pr[order].reshape(-1), cellsA_cse=cse)
    srt_stable = srt.reshape(-1, 4)[order].reshape(-1)
    out["cellsA_sorted"] = srt_stable
    hi_s = pr[order].reshape(-1).astype(np.int32)
    forces = {
        "AO": ("AO", {"kT": 1.0, "wellDepth": 4.0, "cutOff": 1.1}),
        "AOq": ("AO", {"kT": 1.5, "wellDepth": 0.25, "cutOff": 1.2}),
        "LJ6": ("LJ", {"kT": 1.5, "wellDepth": 1 / 1.5, "cutOff": 2.5, "ljNum": 6,
                       "yukawaStrength": 0, "debyeLength": 0.5}),
        "LJ18": ("LJ", {"kT": 1.0, "wellDepth": 3.0, "cutOff": 2.5, "ljNum": 18,
                        "yukawaStrength": 8.0, "debyeLength": 0.5}),
        "YUK": ("LJ", {"kT": 1.0, "wellDepth": 1.0, "cutOff": 3.0, "ljNum": 0,
                       "yukawaStrength": 2183.93, "debyeLength": 0.25}),
        "CAL": ("Cal", {"cutOff": 1.1}),
    }
    for key, (plugin, settings) in forces.items():
        f = ref.forces(plugin, settings, n, box, cs, scale, srt_stable, hi_s, cse)
        out["forceA_%s" % key] = f
        out["forceA_%s_settings" % key] = np.array(repr(settings))
    # ---- vGB coefficients (known-answer set-up)
    for g in (1.0, 0.5, 0.01, 0.049, 2.0):
        c = ref.vgb_coeffs({"gamma": g, "timeStep": 0.001, "kT": 1.0, "nParticles": 1})
        out["vgb_%g" % g] = np.array([c[k] for k in ref.VGB_KEYS])
    c = ref.vgb_coeffs({"gamma": 1.0, "timeStep": 0.002, "kT": 1.5, "nParticles": 1})
    out["vgb_lj"] = np.array([c[k] for k in ref.VGB_KEYS])
    # ---- trajectories with injected noise (system::run loop body)
    for tag, plugin, settings, steps, vel_freq in (
            ("AO", "AO", {"kT": 1.0, "wellDepth": 4.0, "cutOff": 1.1}, 20, 3),
            ("LJ", "LJ", {"kT": 1.5, "wellDepth": 1 / 1.5, "cutOff": 2.5, "ljNum": 6,
                          "yukawaStrength": 0, "debyeLength": 0.5}, 10, 0)):
        rng = np.random.default_rng(5)
        vel = init.maxwell(n, settings["kT"], seed=7).reshape(-1)
        noise = rng.standard_normal(steps * n * 6)
        run_settings = dict(settings, gamma=1.0, nParticles=n, velFreq=vel_freq, mass=1.0,
                            seed=90210, timeStep=0.001)
        p = pos.copy()
        p0, v = np.zeros(3 * n), vel.copy()
        fr, fr0 = np.zeros(3 * n), np.zeros(3 * n)
        mass = np.ones(n)
        hi_t, cse_t, srt_t, lf = ref.run(plugin, run_settings, n, box, cs, scale, steps, noise, p,
                                         p0, v, fr, fr0, rad, mass)
        out.update({"traj%s_vel0" % tag: vel, "traj%s_noise" % tag: noise,
                    "traj%s_meta" % tag: np.array([steps, vel_freq]),
                    "traj%s_settings" % tag: np.array(repr(run_settings)),
                    "traj%s_pos" % tag: p, "traj%s_pos0" % tag: p0, "traj%s_vel" % tag: v,
                    "traj%s_frc" % tag: fr, "traj%s_frc0" % tag: fr0})
    # ---- the reference's per-particle generator
    for seed in (90210, 180420, 7):
        out["rng_%d" % seed] = ref.rng_draws(seed, 256)
    path = os.path.join(HERE, "reference_hotpath.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
