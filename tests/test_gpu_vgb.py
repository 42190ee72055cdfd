"""brownianIntegrator::nextSystem on the GPU (reference-layout drop-in)
against the oracle with identical injected noise."""
import numpy as np
import pytest

from gpu_helpers import rsa_state
from oracle import port

pytestmark = pytest.mark.gpu


@pytest.fixture(params=["direct", "copies"])
def host_access(request, monkeypatch):
    """Both drop-in paths: the GPU on the caller's arrays in place (a device
    with pageable host memory access), or copies in and out in chunks."""
    monkeypatch.setenv("PSIM_DROPIN_COPIES", "1" if request.param == "copies" else "0")
    return request.param


def _setup(n=2000, box=20.0, seed=3):
    pos, rad = rsa_state(n, box, seed)
    rng = np.random.default_rng(seed)
    return dict(pos=pos, pos0=pos.copy(), vel=rng.standard_normal(3 * n),
                frc=rng.standard_normal(3 * n) * 50, frc0=rng.standard_normal(3 * n) * 50,
                mass=rng.uniform(0.5, 2.0, n), n=n, box=box, rng=rng)


@pytest.mark.parametrize("gamma,dt", [(1.0, 0.001), (0.01, 0.001), (5.0, 0.002)])
def test_next_system_matches_oracle(psim, gamma, dt, host_access):
    s = _setup()
    n, box = s["n"], s["box"]
    vel_freq = 1
    it = psim.Integrator(n, gamma=gamma, dt=dt, kT=1.0, vel_freq=vel_freq)
    g = port.geom(n, box, box / 5, 5)
    c = port.vgb_coeffs(gamma, dt, 1.0)
    gp = {k: s[k].copy() for k in ("pos", "pos0", "vel", "frc", "frc0")}
    op = {k: s[k].copy() for k in ("pos", "pos0", "vel", "frc", "frc0")}
    mem, memc = np.zeros(3 * n), np.zeros(3 * n)
    vc = 0
    for step in range(6):
        noise = s["rng"].standard_normal(6 * n)
        pf = s["rng"].standard_normal(3 * n) * 30
        it.next_system(step * dt if step else 0.0, box, gp["pos"], gp["pos0"], gp["vel"],
                       gp["frc"], gp["frc0"], s["mass"], noise=noise, particle_force=pf)
        port.lib().oracle_push_force(n, port._p(pf), port._p(op["frc"]), port._p(op["frc0"]))
        first = step == 0
        vs = (not first) and (vel_freq == 0 or vc == vel_freq)
        err = port.lib().oracle_vgb_step(port.C.byref(g), port.C.byref(c), dt, int(first), int(vs),
                                         port._p(noise), port._p(op["pos"]), port._p(op["pos0"]),
                                         port._p(op["vel"]), port._p(op["frc"]),
                                         port._p(op["frc0"]), port._p(s["mass"]), port._p(mem),
                                         port._p(memc))
        assert err == 0
        if not first:
            vc = 0 if vc == vel_freq else vc + 1
        for k in ("pos", "pos0", "vel", "frc", "frc0"):
            # same IEEE operations in the same order, no FMA: expected bit-exact
            assert np.max(np.abs(gp[k] - op[k])) <= 1e-15 * max(1.0, np.max(np.abs(op[k]))), (k, step)


def test_out_of_bounds_is_reported_as_7703(psim, host_access):
    n, box = 4, 12.0
    it = psim.Integrator(n, gamma=1.0, dt=0.001, kT=1.0)
    pos = np.array([1.0, 1.0, 1.0, 5.0, 5.0, 5.0, 9.0, 9.0, 9.0, 2.0, 8.0, 3.0])
    z = np.zeros(3 * n)
    # a force that throws particle 0 beyond one box length: the single +-L wrap
    # of safeMod cannot bring it back (particle.cpp:67-69)
    pf = z.copy()
    pf[0] = -1e11
    with pytest.raises(psim.PsimError) as e:
        it.next_system(0.0, box, pos, pos.copy(), z.copy(), z.copy(), z.copy(), np.ones(n),
                       noise=np.zeros(6 * n), particle_force=pf)
    assert e.value.code == psim.ERR_PARTICLE_BOUNDS


def test_gamma_zero_is_refused(psim):
    with pytest.raises(psim.PsimError) as e:
        psim.Integrator(10, gamma=0.0)
    assert e.value.code == psim.ERR_INPUT


def test_philox_noise_is_keyed_by_particle(psim, host_access):
    # the copies and the update run in chunks: every particle keeps its own
    # Philox stream (no two particles move alike without forces)
    n, box = 4096, 40.0
    rng = np.random.default_rng(5)
    pos = rng.uniform(5.0, 35.0, 3 * n)
    z = np.zeros(3 * n)
    it = psim.Integrator(n, gamma=1.0, dt=0.001, kT=1.0, vel_freq=1000, seed=77)
    p, p0, v, f, f0 = pos.copy(), pos.copy(), z.copy(), z.copy(), z.copy()
    for step in range(3):
        it.next_system(step * 0.001, box, p, p0, v, f, f0, np.ones(n), particle_force=z)
    d = (p - pos).reshape(-1, 3)
    assert np.all(np.isfinite(d)) and np.unique(d, axis=0).shape[0] == n
    assert 0.5 < np.var(d) / np.var(d[: n // 8]) < 2.0   # the same spread in every chunk
    it.close()


def test_direct_and_copied_paths_agree(psim, monkeypatch):
    # the same Philox keys and the same FP64 operations: identical arrays,
    # through a first step, normal steps and a velocity step, without and
    # with the force push
    s = _setup(n=3001, seed=8)
    n, box = s["n"], s["box"]
    out = {}
    for mode in ("0", "1"):
        monkeypatch.setenv("PSIM_DROPIN_COPIES", mode)
        it = psim.Integrator(n, gamma=1.0, dt=0.002, kT=1.0, vel_freq=2, seed=11)
        a = {k: s[k].copy() for k in ("pos", "pos0", "vel", "frc", "frc0")}
        rng = np.random.default_rng(9)
        for step in range(5):
            pf = rng.standard_normal(3 * n) * 20 if step != 2 else None
            it.next_system(step * 0.002, box, a["pos"], a["pos0"], a["vel"], a["frc"], a["frc0"],
                           s["mass"], particle_force=pf)
        it.close()
        out[mode] = a
    for k in out["0"]:
        assert np.array_equal(out["0"][k], out["1"][k]), k
