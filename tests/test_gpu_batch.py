"""Batches of independent replicas (psim_batch_create): one launch per phase
over all replicas, each replica stepping bit for bit like the system built
from its own settings."""
import numpy as np
import pytest

from proteinsim2015_gb300 import init

pytestmark = pytest.mark.gpu


def ao_replica(psim, n, phi, contact_kT, q, seed):
    """A replica as config C2 draws them: AO colloids (sigma = 1) at volume
    fraction phi, contact attraction contact_kT, polymer/colloid ratio q."""
    box = (n * np.pi / 6.0 / phi) ** (1.0 / 3.0)
    rc = 1.0 + q
    scale = max(3, int(np.floor(box / rc)))
    g = psim.geometry(n, box, box / scale, scale)
    wd = contact_kT * q / (1.5 + q)        # U(1) = -kT wd (rc + 0.5) / (rc - 1)
    f = psim.make_force("AO", rc, kT=1.0, well_depth=wd)
    pos = init.rsa(n, box, 1.0, seed=seed).reshape(-1)
    return g, f, pos


REPLICAS = [(700, 0.10, 2.0, 0.10), (2500, 0.25, 4.0, 0.15), (1200, 0.05, 1.0, 0.20),
            (3100, 0.30, 6.0, 0.05), (513, 0.20, 3.0, 0.12)]


@pytest.mark.parametrize("precision", [0, 1])
def test_batch_steps_like_its_replicas(psim, precision):
    reps, states = [], []
    for k, (n, phi, a, q) in enumerate(REPLICAS):
        g, f, pos = ao_replica(psim, n, phi, a, q, seed=60 + k)
        reps.append((g, f, 1000 + 17 * k))
        states.append(pos)
    rng = np.random.default_rng(61)
    vels = [rng.standard_normal(3 * g.n_particles) for g, _, _ in reps]
    b = psim.Batch(reps, gamma=1.0, dt=0.001, kT=1.0, vel_freq=7, precision=precision)
    b.upload(np.concatenate(states), np.full(b.n, 0.5), vel=np.concatenate(vels))
    for k in (1, 5, 13):          # crosses graph phases and velocity steps
        b.step(k)
    out = b.download()
    assert b.get_step()[0] == 19
    for k, (g, f, seed) in enumerate(reps):
        s = psim.System(g, f, gamma=1.0, dt=0.001, kT=1.0, vel_freq=7, seed=seed,
                        precision=precision)
        s.upload(states[k], np.full(g.n_particles, 0.5), vel=vels[k])
        s.step(19)
        ref = s.download()
        s.close()
        for key in ("pos", "pos0", "vel", "frc", "frc0"):
            assert np.array_equal(b.split(out[key])[k], ref[key]), (k, key)
    b.close()


def test_batch_refuses_mixed_plugins(psim):
    g1, f1, _ = ao_replica(psim, 500, 0.1, 2.0, 0.1, seed=62)
    f2 = psim.make_force("LJ", 1.1, kT=1.0, well_depth=1.0, lj_num=6)
    with pytest.raises(psim.PsimError) as e:
        psim.Batch([(g1, f1, 1), (g1, f2, 2)])
    assert e.value.code == psim.ERR_INPUT
    f3 = psim.make_force("AO_YUK", 1.1, kT=1.0, well_depth=0.2, cutoff2=1.1, well_depth2=1.0,
                         yukawa_strength=1.0, debye_length=0.25, lj_num=0)
    with pytest.raises(psim.PsimError):
        psim.Batch([(g1, f3, 1)])


def test_batch_with_pair_list_follows_batch_without(psim):
    # the same replicas with grids that allow a 0.2 skin.  After steps across
    # list rebuilds (all replicas rebuild together), the list pass and the cell
    # walk give the same forces on the list run's state, and one more step
    # from that state moves both alike (the steep AO core makes longer
    # trajectories diverge from FP32 summation order alone)
    skin = 0.2
    reps, states = [], []
    for k, (n, phi, a, q) in enumerate(REPLICAS):
        g0, f, pos = ao_replica(psim, n, phi, a, q, seed=60 + k)
        box = g0.box_size
        scale = max(3, int(np.floor(box / (f.cutoff + skin))))
        reps.append((psim.geometry(n, box, box / scale, scale), f, 1000 + 17 * k))
        states.append(pos)
    rng = np.random.default_rng(63)
    vel = np.concatenate([rng.standard_normal(3 * g.n_particles) for g, _, _ in reps])
    lst = psim.Batch(reps, gamma=1.0, dt=0.002, kT=1.0, vel_freq=7, skin=skin)
    lst.upload(np.concatenate(states), np.full(lst.n, 0.5), vel=vel)
    for k in (1, 5, 13, 41):
        lst.step(k)
    assert lst.list_builds() >= 1
    st = lst.download()
    walk = psim.Batch(reps, gamma=1.0, dt=0.002, kT=1.0, vel_freq=7)
    walk.upload(st["pos"], np.full(walk.n, 0.5), vel=st["vel"], pos0=st["pos0"], frc=st["frc"],
                frc0=st["frc0"])
    lst.upload(st["pos"], np.full(lst.n, 0.5), vel=st["vel"], pos0=st["pos0"], frc=st["frc"],
               frc0=st["frc0"])
    fl, fw = lst.forces(), walk.forces()
    assert np.linalg.norm(fl - fw) < 1e-5 * np.linalg.norm(fw)
    lst.step(1)
    walk.step(1)
    a, b = lst.download(), walk.download()
    for k, (g, _, _) in enumerate(reps):
        d = lst.split(a["pos"])[k] - walk.split(b["pos"])[k]
        d -= g.box_size * np.round(d / g.box_size)   # a wrap at the box edge
        # dt^2 times the FP32 force difference (~1e-5 of the steep cores' forces)
        assert np.max(np.abs(d)) < 1e-7, k
    # the cell list exported for the current positions is the same
    assert all(np.array_equal(x, y) for x, y in zip(lst.download_cells()[:2],
                                                     walk.download_cells()[:2]))
    lst.close()
    walk.close()


def test_batch_pair_list_needs_room(psim):
    g, f, _ = ao_replica(psim, 500, 0.1, 2.0, 0.1, seed=64)
    with pytest.raises(psim.PsimError) as e:
        psim.Batch([(g, f, 1)], skin=g.cell_size)   # cellSize < cutOff + skin
    assert e.value.code == psim.ERR_INPUT


def test_batch_list_lanes_and_tuner(psim):
    # the batched list pass with 1, 2 and 4 threads per particle, and the
    # tuner that picks one on the live batch
    from proteinsim2015_gb300 import batch
    skin = 0.2
    reps, states = [], []
    for k, (n, phi, a, q) in enumerate(REPLICAS):
        g0, f, pos = ao_replica(psim, n, phi, a, q, seed=70 + k)
        box = g0.box_size
        scale = max(3, int(np.floor(box / (f.cutoff + skin))))
        reps.append((psim.geometry(n, box, box / scale, scale), f, 2000 + 13 * k))
        states.append(pos)
    b = psim.Batch(reps, gamma=1.0, dt=0.001, kT=1.0, vel_freq=7, skin=skin)
    b.upload(np.concatenate(states), np.full(b.n, 0.5))
    forces = {}
    for lanes in (1, 2, 4):
        b.set_list_lanes(lanes)
        forces[lanes] = b.forces()
    for lanes in (2, 4):
        assert np.linalg.norm(forces[lanes] - forces[1]) < 1e-6 * np.linalg.norm(forces[1])
    best, rates = batch.tune_lanes(b, steps=20, warmup=2)
    assert best in (1, 2, 4) and set(rates) == {1, 2, 4} and all(r > 0 for r in rates.values())
    b.close()
    with pytest.raises(psim.PsimError):
        psim.System(reps[0][0], reps[0][1]).set_list_lanes(3)
