"""The device-resident step loop (force -> push -> nextSystem -> rebuild)
against the reference's golden trajectories and the oracle."""
import numpy as np
import pytest

from conftest import settings_of
from gpu_helpers import TRAJ_TOL, lattice_state, rel_norm, rsa_state
from oracle import port

pytestmark = pytest.mark.gpu


def make_system(psim, n, box, scale, force, precision=0, noise_mode=1, gamma=1.0, dt=0.001,
                kT=1.0, vel_freq=1000, seed=90210):
    g = psim.geometry(n, box, box / scale, scale)
    return psim.System(g, force, gamma=gamma, dt=dt, kT=kT, vel_freq=vel_freq, seed=seed,
                       precision=precision, noise_mode=noise_mode)


@pytest.mark.parametrize("tag", ["AO", "LJ"])
def test_trajectory_matches_reference_golden(psim, golden, tag, force_pass):
    n, box, cs, scale = (int(v) for v in golden["cellsA_geom"])
    s = settings_of(golden, "traj%s_settings" % tag)
    steps, vel_freq = (int(v) for v in golden["traj%s_meta" % tag])
    plugin = {"AO": "AOPotential", "LJ": "LennardJones"}[tag]
    text = "".join("%s = %r\n" % kv for kv in s.items())
    p = psim.force_params_from_settings(plugin, text)
    sysm = make_system(psim, n, box, scale, p, precision=0, gamma=s["gamma"], dt=s["timeStep"],
                       kT=s["kT"], vel_freq=vel_freq)
    sysm.upload(golden["cellsA_pos"], golden["cellsA_radius"], vel=golden["traj%s_vel0" % tag])
    sysm.set_noise(golden["traj%s_noise" % tag], steps)
    sysm.step(steps)
    out = sysm.download()
    L = float(box)
    for k in ("pos", "pos0", "vel"):
        ref = golden["traj%s_%s" % (tag, k)]
        assert np.max(np.abs(out[k] - ref)) <= TRAJ_TOL, k
    for k in ("frc", "frc0"):
        ref = golden["traj%s_%s" % (tag, k)]
        assert np.max(np.abs(out[k] - ref)) <= 1e-9 * np.max(np.abs(ref)), k


def test_100_steps_match_oracle_fp64(psim, force_pass):
    n, box, scale = 4000, 21.0, 7            # the reference-constructible AO box
    pos, rad = rsa_state(n, box, seed=21)
    rng = np.random.default_rng(8)
    vel = rng.standard_normal(3 * n)
    steps, dt = 100, 0.001
    noise = rng.standard_normal(steps * n * 6)
    p = psim.make_force("AO", 1.1, kT=1.0, well_depth=0.25)
    sysm = make_system(psim, n, box, scale, p, precision=0, vel_freq=0)
    sysm.upload(pos, rad, vel=vel)
    sysm.set_noise(noise, steps)
    sysm.step(steps)
    out = sysm.download()
    g = port.geom(n, box, box / scale, scale)
    st = port.State(pos, rad, vel=vel)
    err, hi, cse, srt, _ = port.run(g, port.force_from_params(p.as_dict()),
                                    port.vgb_coeffs(1.0, dt, 1.0), dt, st, steps, noise,
                                    vel_freq=0)
    assert err == 0
    assert np.max(np.abs(out["pos"] - st.pos)) <= TRAJ_TOL
    assert np.max(np.abs(out["pos0"] - st.pos0)) <= TRAJ_TOL
    assert np.max(np.abs(out["vel"] - st.vel)) <= 1e-6 * np.max(np.abs(st.vel))
    # the cell list after the last rebuild
    ghi, gcse, gsrt = sysm.download_cells()
    assert np.array_equal(ghi, hi) and np.array_equal(gcse, cse)
    assert np.max(np.abs(gsrt - srt)) <= TRAJ_TOL
    assert sysm.get_step() == (steps, 0)


def test_mixed_precision_forces_within_1e5(psim):
    # the LJ liquid at rho = 0.8 after a short melt: mixed vs plain force
    pos, rad, box = lattice_state(10, (4 / 0.8) ** (1 / 3), 0.05, seed=5)
    n = len(rad)
    scale = int(box // 2.5)
    p = psim.make_force("LJ", 2.5, kT=1.5, well_depth=1 / 1.5, lj_num=6, yukawa_strength=0.0)
    sysm = make_system(psim, n, box, scale, p, precision=0, noise_mode=0, dt=0.002, kT=1.5)
    rng = np.random.default_rng(1)
    sysm.upload(pos, rad, vel=rng.standard_normal(3 * n) * np.sqrt(1.5))
    sysm.step(200)
    st = sysm.download()
    hi, cse, srt = sysm.download_cells()
    g = psim.geometry(n, box, box / scale, scale)
    f64 = psim.force_evaluate(p, g, srt, hi, cse, precision=0)
    f32 = psim.force_evaluate(p, g, srt, hi, cse, precision=1)
    assert rel_norm(f32, f64) <= 1e-5
    assert np.all(np.isfinite(st["pos"]))


def test_mixed_system_tracks_fp64_system(psim):
    n, box, scale = 4000, 21.0, 7
    pos, rad = rsa_state(n, box, seed=22)
    p = psim.make_force("AO", 1.1, kT=1.0, well_depth=0.25)
    outs = []
    for prec in (0, 1):
        s = make_system(psim, n, box, scale, p, precision=prec, noise_mode=0)
        s.upload(pos, rad)
        s.step(50)
        outs.append(s.download())
    d = outs[0]["pos"] - outs[1]["pos"]
    d -= box * np.round(d / box)
    assert np.max(np.abs(d)) < 1e-6


def test_deterministic_and_graph_phases(psim):
    # 13 steps cross every buffer phase of the captured graphs twice
    n, box, scale = 3000, 20.0, 6
    pos, rad = rsa_state(n, box, seed=23)
    p = psim.make_force("CAL", 1.1)
    res = []
    for _ in range(2):
        s = make_system(psim, n, box, scale, p, precision=1, noise_mode=0, vel_freq=2)
        s.upload(pos, rad)
        for k in (1, 5, 7):
            s.step(k)
        res.append(s.download())
    for k in res[0]:
        assert np.array_equal(res[0][k], res[1][k])


@pytest.mark.parametrize("skin", [0.0, 0.1])
def test_multi_step_graphs_match_single_steps(psim, skin):
    # a long call runs graphs of 12 steps (after single steps up to a multiple
    # of 6): the same state as one step per call, through list rebuilds too
    n, box, scale = 3000, 20.0, 6
    pos, rad = rsa_state(n, box, seed=24)
    p = psim.make_force("AO", 1.1, kT=1.0, well_depth=0.25)
    g = psim.geometry(n, box, box / scale, scale)
    res = []
    for calls in ((3, 60), (1,) * 63):
        s = psim.System(g, p, gamma=1.0, dt=0.002, kT=1.0, vel_freq=5, seed=9,
                        precision=psim.PRECISION_MIXED, skin=skin)
        s.upload(pos, rad)
        for k in calls:
            s.step(k)
        out = s.download()
        out["builds"] = np.array([s.list_builds()])
        res.append(out)
        s.close()
    for k in res[0]:
        assert np.array_equal(res[0][k], res[1][k]), k
    if skin > 0:
        assert res[0]["builds"][0] > 1


def test_snapshot_async_equals_download(psim):
    n, box, scale = 2000, 16.0, 5
    pos, rad = rsa_state(n, box, seed=24)
    s = make_system(psim, n, box, scale, psim.make_force("AO", 1.1, well_depth=0.5),
                    precision=1, noise_mode=0)
    s.upload(pos, rad)
    s.step(3)
    host = np.empty(3 * n)
    s.snapshot_async(host)
    s.step_async(4)
    s.snapshot_wait()
    s.sync()
    ref = s.download()["pos"]  # positions now 4 steps later
    s2 = make_system(psim, n, box, scale, psim.make_force("AO", 1.1, well_depth=0.5),
                     precision=1, noise_mode=0)
    s2.upload(pos, rad)
    s2.step(3)
    assert np.array_equal(host, s2.download()["pos"])
    assert not np.array_equal(host, ref)


def test_overlap_stops_the_run_with_7704(psim):
    n, box, scale = 500, 12.0, 4
    pos, rad = rsa_state(n, box, seed=25)
    pos = pos.reshape(-1, 3)
    pos[1] = pos[0] + np.array([0.3, 0.0, 0.0])  # plant an overlapping pair
    pos = np.mod(pos, box).reshape(-1)
    s = make_system(psim, n, box, scale, psim.make_force("AO", 1.1, well_depth=0.5),
                    precision=0, noise_mode=0)
    s.upload(pos, rad)
    with pytest.raises(psim.PsimError) as e:
        s.step(5)
    assert e.value.code == psim.ERR_OVERLAP
    assert s.get_step()[0] == 0   # stopped in the first step's force pass
    with pytest.raises(psim.PsimError):
        s.step(1)                 # the error stays latched until a new upload


def test_injected_noise_range_is_checked(psim):
    n, box, scale = 100, 12.0, 4
    pos, rad = rsa_state(n, box, seed=26)
    s = make_system(psim, n, box, scale, psim.make_force("CAL", 1.1), precision=0)
    s.upload(pos, rad)
    s.set_noise(np.zeros(2 * n * 6), 2)
    s.step(2)
    with pytest.raises(psim.PsimError) as e:
        s.step(1)
    assert e.value.code == psim.ERR_INPUT


def test_free_particle_temperature_and_diffusion(psim):
    # Philox noise, no interactions (LJ with wellDepth 0): the vGB velocities
    # give kT/m per component, and the mean-square displacement follows the
    # Ornstein-Uhlenbeck law 6 (kT / m gamma) (t - (1 - e^{-gamma t}) / gamma).
    n, box, scale = 20000, 120.0, 40
    rng = np.random.default_rng(30)
    pos = rng.uniform(0, box, 3 * n)
    rad = np.full(n, 1e-6)
    p = psim.make_force("LJ", 0.02, kT=1.0, well_depth=0.0, lj_num=6, yukawa_strength=0.0)
    gamma, dt, chunk, chunks = 1.0, 0.01, 50, 20
    s = make_system(psim, n, box, scale, p, precision=1, noise_mode=0, gamma=gamma, dt=dt,
                    kT=1.0, vel_freq=0)
    s.upload(pos, rad, vel=rng.standard_normal(3 * n))
    prev = pos.copy()
    disp = np.zeros(3 * n)
    temps = []
    for _ in range(chunks):
        s.step(chunk)
        st = s.download()
        d = st["pos"] - prev
        d -= box * np.round(d / box)   # unwrap: a chunk moves ~1, far below L/2
        disp += d
        prev = st["pos"]
        temps.append(np.mean(st["vel"] ** 2))
    T = np.mean(temps[4:])
    assert abs(T - 1.0) < 0.03, T
    t = chunk * chunks * dt
    msd = np.mean(np.sum(disp.reshape(-1, 3) ** 2, axis=1))
    expect = 6.0 * (t - (1.0 - np.exp(-gamma * t)) / gamma)  # D = kT/(m gamma) = 1
    assert abs(msd / expect - 1.0) < 0.05, (msd, expect)
