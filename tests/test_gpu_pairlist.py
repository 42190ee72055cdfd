"""The mixed form's Verlet pair list: the same pair terms as the 27-cell walk
every step, so a run with a skin follows the run without one up to FP32
summation order, across list rebuilds and periodic wraps."""
import numpy as np
import pytest

from gpu_helpers import lattice_state, rel_norm, rsa_state

pytestmark = pytest.mark.gpu

DT, KT = 0.002, 1.5


def run(psim, g, force, pos, rad, vel, noise, steps, skin, precision=1):
    s = psim.System(g, force, gamma=1.0, dt=DT, kT=KT, vel_freq=1000, seed=7,
                    precision=precision, noise_mode=psim.NOISE_INJECTED, skin=skin)
    s.upload(pos, rad, vel=vel)
    s.set_noise(noise, steps)
    s.step(steps)
    out = s.download()
    out["builds"] = s.list_builds()
    hi, cse, srt = s.download_cells()
    out["hi"], out["cse"] = hi, cse
    s.close()
    return out


def lj_liquid(psim):
    # rho = 0.8 LJ, 2048 particles in a 13.7 box: 4^3 cells of 3.42 leave room
    # for a 0.9 skin; a quarter of the particles sit in boundary cells
    pos, rad, box = lattice_state(8, (4 / 0.8) ** (1 / 3), 0.08, seed=40)
    n = len(rad)
    g = psim.geometry(n, box, box / 4, 4)
    p = psim.make_force("LJ", 2.5, kT=KT, well_depth=1 / KT, lj_num=6, yukawa_strength=0.0)
    return g, p, pos, rad


def ao_colloids(psim):
    n, box, scale = 4000, 21.0, 7
    pos, rad = rsa_state(n, box, seed=41)
    return psim.geometry(n, box, box / scale, scale), psim.make_force("AO", 1.1, kT=1.0,
                                                                        well_depth=0.25), pos, rad


def ao_yukawa(psim):
    n, box, scale = 3000, 26.0, 6
    pos, rad = rsa_state(n, box, seed=42)
    p = psim.make_force("AO_YUK", 1.1, kT=1.0, well_depth=0.1875, cutoff2=3.0, well_depth2=1.0,
                        yukawa_strength=2183.93, debye_length=0.25, lj_num=0)
    return psim.geometry(n, box, box / scale, scale), p, pos, rad


SYSTEMS = {"lj_liquid": lj_liquid, "ao": ao_colloids, "ao_yukawa": ao_yukawa}


@pytest.mark.parametrize("name", sorted(SYSTEMS))
@pytest.mark.parametrize("skin", [0.1, 0.4])
def test_pairlist_run_follows_cell_walk(psim, name, skin):
    g, p, pos, rad = SYSTEMS[name](psim)
    n = g.n_particles
    rng = np.random.default_rng(43)
    vel = rng.standard_normal(3 * n) * np.sqrt(KT)
    steps = 60
    noise = rng.standard_normal(steps * n * 6)
    ref = run(psim, g, p, pos, rad, vel, noise, steps, 0.0)
    got = run(psim, g, p, pos, rad, vel, noise, steps, skin)
    assert ref["builds"] == 0
    assert got["builds"] >= 1                      # the list was rebuilt on the way
    # a missing or doubled pair term would show as an O(1) relative force error;
    # the FP32 summation order alone moves the steep AO core's forces ~1e-7
    assert rel_norm(got["frc"], ref["frc"]) < 1e-5
    d = got["pos"] - ref["pos"]
    d -= g.box_size * np.round(d / g.box_size)
    assert np.max(np.abs(d)) < 1e-6
    assert rel_norm(got["vel"], ref["vel"]) < 1e-5
    # the reference's cell list is still rebuilt every step
    assert np.array_equal(got["hi"], ref["hi"]) and np.array_equal(got["cse"], ref["cse"])


def test_pairlist_run_tracks_fp64(psim):
    g, p, pos, rad = lj_liquid(psim)
    n = g.n_particles
    rng = np.random.default_rng(44)
    vel = rng.standard_normal(3 * n) * np.sqrt(KT)
    steps = 40
    noise = rng.standard_normal(steps * n * 6)
    ref = run(psim, g, p, pos, rad, vel, noise, steps, 0.0, precision=0)
    got = run(psim, g, p, pos, rad, vel, noise, steps, 0.3)
    assert rel_norm(got["frc"], ref["frc"]) < 1e-5
    d = got["pos"] - ref["pos"]
    d -= g.box_size * np.round(d / g.box_size)
    assert np.max(np.abs(d)) < 1e-6


def test_pairlist_is_deterministic(psim):
    g, p, pos, rad = ao_colloids(psim)
    outs = []
    for _ in range(2):
        s = psim.System(g, p, gamma=1.0, dt=0.001, kT=1.0, precision=psim.PRECISION_MIXED,
                        noise_mode=psim.NOISE_PHILOX, skin=0.2)
        s.upload(pos, rad)
        for k in (1, 5, 7, 30):
            s.step(k)
        outs.append(s.download())
        s.close()
    for k in outs[0]:
        assert np.array_equal(outs[0][k], outs[1][k])


def test_pairlist_overlap_is_7704(psim):
    n, box, scale = 500, 12.0, 4
    pos, rad = rsa_state(n, box, seed=45)
    pos = pos.reshape(-1, 3)
    pos[1] = pos[0] + np.array([0.3, 0.0, 0.0])
    pos = np.mod(pos, box).reshape(-1)
    g = psim.geometry(n, box, box / scale, scale)
    s = psim.System(g, psim.make_force("AO", 1.1, well_depth=0.5), precision=psim.PRECISION_MIXED,
                    noise_mode=psim.NOISE_PHILOX, skin=0.4)
    s.upload(pos, rad)
    with pytest.raises(psim.PsimError) as e:
        s.step(3)
    assert e.value.code == psim.ERR_OVERLAP


def test_pairlist_skin_is_checked(psim):
    g, p, pos, rad = lj_liquid(psim)
    with pytest.raises(psim.PsimError) as e:     # cellSize 3.42 < 2.5 + 1.0
        psim.System(g, p, precision=psim.PRECISION_MIXED, skin=1.0)
    assert e.value.code == psim.ERR_INPUT
    with pytest.raises(psim.PsimError) as e:     # the plain FP64 form walks the cells
        psim.System(g, p, precision=psim.PRECISION_FP64, skin=0.3)
    assert e.value.code == psim.ERR_INPUT
    assert psim.auto_skin(g, p) == pytest.approx(0.4)


@pytest.mark.parametrize("skin,precision", [(0.0, 0), (0.0, 1), (0.4, 1)])
def test_system_forces_match_dropin_fp64(psim, skin, precision):
    # the force at the current state, from the pass the next step runs,
    # against the drop-in FP64 evaluation on the system's own cell list
    g, p, pos, rad = lj_liquid(psim)
    s = psim.System(g, p, gamma=1.0, dt=DT, kT=KT, precision=precision,
                    noise_mode=psim.NOISE_PHILOX, skin=skin)
    s.upload(pos, rad, vel=np.random.default_rng(46).standard_normal(3 * g.n_particles))
    s.step(37)
    f = s.forces()
    hi, cse, srt = s.download_cells()
    ref = psim.force_evaluate(p, g, srt, hi, cse, precision=psim.PRECISION_FP64)
    s.close()
    assert rel_norm(f, ref) < (1e-12 if precision == 0 else 1e-5)


def test_pairlist_with_unequal_radii(psim):
    # two radii: the list keeps full 32-byte records (uniform radii use the
    # compact 16-byte ones, which every test above runs)
    g, p, pos, rad = lj_liquid(psim)
    rad = rad.copy()
    rad[::3] = 0.45
    n = g.n_particles
    rng = np.random.default_rng(47)
    vel = rng.standard_normal(3 * n) * np.sqrt(KT)
    steps = 40
    noise = rng.standard_normal(steps * n * 6)
    ref = run(psim, g, p, pos, rad, vel, noise, steps, 0.0)
    got = run(psim, g, p, pos, rad, vel, noise, steps, 0.4)
    assert got["builds"] >= 1
    assert rel_norm(got["frc"], ref["frc"]) < 1e-5
    d = got["pos"] - ref["pos"]
    d -= g.box_size * np.round(d / g.box_size)
    assert np.max(np.abs(d)) < 1e-6


@pytest.mark.parametrize("lanes", [2, 4])
def test_lanes_per_particle_give_the_same_forces(psim, lanes):
    # the list pass with 2 or 4 threads per particle: the same pair terms, the
    # lanes' Kahan sums added in lane order -- against the one-lane pass and
    # FP64 within the mixed form's tolerance, and reproducible run to run
    g, p, pos, rad = lj_liquid(psim)
    f64 = psim.System(g, p, precision=0)
    f64.upload(pos, rad)
    ref = f64.forces()
    f64.close()
    s = psim.System(g, p, precision=1, skin=0.4)
    s.upload(pos, rad)
    one = s.forces()
    s.set_list_lanes(lanes)
    many = s.forces()
    again = s.forces()
    assert np.array_equal(many, again)
    assert rel_norm(many, ref) < 1e-5 and rel_norm(many, one) < 1e-6
    # stepping: graphs captured with the new setting
    s.step(20)
    assert np.all(np.isfinite(s.download()["pos"]))
    s.close()


def test_pairlist_in_a_large_box(psim):
    # a dilute LJ gas (rho = 0.1) filling a 126-wide box: the compact records'
    # fixed-point coordinates (units of 2^-27) wrap modulo 2^32 several times
    # over the box, and the pairs across its faces use halo records beyond
    # [0, L) -- the list pass still gives the FP64 forces and follows the
    # cell walk step for step
    pos, rad, box = lattice_state(37, (4 / 0.1) ** (1 / 3), 0.3, seed=49)
    n = len(rad)
    scale = int(box // 2.9)
    g = psim.geometry(n, box, box / scale, scale)
    p = psim.make_force("LJ", 2.5, kT=KT, well_depth=1 / KT, lj_num=6, yukawa_strength=0.0)
    f64 = psim.System(g, p, precision=0)
    f64.upload(pos, rad)
    ref = f64.forces()
    f64.close()
    s = psim.System(g, p, precision=1, skin=0.4)
    s.upload(pos, rad)
    assert rel_norm(s.forces(), ref) < 1e-5
    s.close()
    rng = np.random.default_rng(50)
    vel = rng.standard_normal(3 * n) * np.sqrt(KT)
    steps = 40
    noise = rng.standard_normal(steps * n * 6)
    walk = run(psim, g, p, pos, rad, vel, noise, steps, 0.0)
    lst = run(psim, g, p, pos, rad, vel, noise, steps, 0.4)
    assert lst["builds"] >= 1
    assert rel_norm(lst["frc"], walk["frc"]) < 1e-5
    d = lst["pos"] - walk["pos"]
    d -= g.box_size * np.round(d / g.box_size)
    # a wrong record (a separation off by a wrap of 2^31 units) would show as
    # an O(1) force error above; most positions agree to ~1e-13, and close
    # binary collisions of the gas on the r^-13 core amplify the FP32
    # summation difference (measured after 40 steps: 99.9th percentile
    # 1.1e-8, largest 4.3e-6, one particle of 2e5)
    assert np.percentile(np.abs(d), 99.9) < 1e-6
    assert np.max(np.abs(d)) < 1e-4


def test_direct_walk_on_a_sparse_grid_matches_fp64(psim):
    # AO colloids at the gel's volume fraction on cells of 1.2 (one particle
    # per cell on average): the mixed form without a skin takes the direct
    # walk (queues kept across the 27 cells, images applied to the
    # neighbour), the plain FP64 form the staged walk in the reference's
    # order -- the same forces, and the same bits run to run
    from proteinsim2015_gb300 import batch, init
    n, phi = 20000, 0.30
    box = (n * np.pi / 6.0 / phi) ** (1.0 / 3.0)
    f = batch.ao_params(psim, 6.0, 0.08)
    scale = int(box // 1.2)
    g = psim.geometry(n, box, box / scale, scale)
    assert n < 4 * scale ** 3
    pos = init.rsa(n, box, 1.0, seed=51).reshape(-1)
    rad = np.full(n, 0.5)
    f64 = psim.System(g, f, precision=0)
    f64.upload(pos, rad)
    ref = f64.forces()
    f64.close()
    outs = []
    for _ in range(2):
        s = psim.System(g, f, gamma=1.0, dt=0.001, kT=1.0, precision=1,
                        noise_mode=psim.NOISE_PHILOX)
        s.upload(pos, rad)
        got = s.forces()
        assert rel_norm(got, ref) < 1e-5
        s.step(25)
        outs.append((got, s.download()))
        s.close()
    assert np.array_equal(outs[0][0], outs[1][0])
    for k in outs[0][1]:
        assert np.array_equal(outs[0][1][k], outs[1][1][k])
