"""Observables of the device-resident state against numpy restatements of
the reference's analysis routines on the downloaded state."""
import numpy as np
import pytest

from gpu_helpers import rsa_state

pytestmark = pytest.mark.gpu


def ao_system(psim, n=600, box=12.0, scale=4, precision=0, vel_freq=0, seed=70, skin=0.0):
    pos, rad = rsa_state(n, box, seed=seed)
    g = psim.geometry(n, box, box / scale, scale)
    s = psim.System(g, psim.make_force("AO", 1.1, kT=1.0, well_depth=0.25), gamma=1.0,
                    dt=0.002, kT=1.0, vel_freq=vel_freq, precision=precision, skin=skin)
    s.upload(pos, rad, vel=np.random.default_rng(seed).standard_normal(3 * n))
    return s, g


def min_image(d, L):
    # pbcDist (utilities.cpp:79-104): |d| > L/2 -> |d| - L
    a = np.abs(d)
    return np.where(a > L / 2.0, a - L, a)


@pytest.mark.parametrize("precision", [0, 1])
def test_temperature_displacement_and_potential(psim, precision):
    s, g = ao_system(psim, precision=precision)
    s.step(25)
    st = s.download()
    n = g.n_particles
    v = st["vel"]
    assert s.temperature() == pytest.approx(np.sum(v * v) / 3.0 / n, rel=1e-12)
    d = st["pos"] - st["pos0"]
    assert s.mean_displacement() == pytest.approx(np.sum(d * d) / n, rel=1e-12)
    # particle::calculatePotential in FP32, averaged (analysisOutput.cpp:117-123)
    f32 = np.float32
    dx = (st["pos"] - st["pos0"]).reshape(-1, 3).astype(f32)
    df = (st["frc"] - st["frc0"]).reshape(-1, 3).astype(f32)
    f0 = st["frc0"].reshape(-1, 3)
    dr = np.sqrt(np.sum(dx * dx, axis=1, dtype=f32))
    dfn = np.sqrt(np.sum(df * df, axis=1, dtype=f32))
    f0n = np.sqrt(np.sum(f0 * f0, axis=1).astype(f32))
    pot = -(f0n * dr + f32(0.5) * dfn * dr)
    assert s.potential() == pytest.approx(np.mean(pot.astype(np.float64)), rel=1e-5, abs=1e-9)
    s.close()


def test_tracked_displacement_counts_every_wrap(psim):
    s, g = ao_system(psim, n=400, box=9.0, scale=3, precision=1)
    L = g.box_size
    s.step(2)
    s.track_start()
    start = s.download()["pos"].copy()
    prev, unwrapped = start.copy(), start.copy()
    for _ in range(40):
        s.step(5)   # a particle moves far less than L/2 in 5 steps
        cur = s.download()["pos"]
        d = cur - prev
        d -= L * np.round(d / L)
        unwrapped += d
        prev = cur
    ref = np.mean(np.sum(((unwrapped - start) ** 2).reshape(-1, 3), axis=1))
    assert np.any(np.abs(unwrapped - prev) > L / 2)   # some particle did cross the box
    assert s.tracked_displacement() == pytest.approx(ref, rel=1e-9)
    s.close()


@pytest.mark.parametrize("skin", [0.0, 0.4])
def test_interactions_and_rdf_match_all_pairs(psim, skin):
    s, g = ao_system(psim, n=700, box=12.0, scale=4, precision=1, skin=skin)
    s.step(10)
    hi, cse, srt = s.download_cells()
    pos = s.download()["pos"].reshape(-1, 3)
    L = g.box_size
    d = min_image(pos[:, None, :] - pos[None, :, :], L)
    r = np.sqrt(np.sum(d * d, axis=2))
    np.fill_diagonal(r, np.inf)
    coor, tot = s.interactions(1.2)
    assert np.array_equal(coor, np.sum(r < 1.2, axis=1))
    assert tot == int(np.sum(r < 1.2))
    rmin, rmax, nb = 0.8, 3.0, 44
    gr = s.rdf(rmin, rmax, nb)
    hist, edges = np.histogram(r[np.isfinite(r)], bins=nb, range=(rmin, rmax))
    n = g.n_particles
    rho = n / L ** 3
    shell = 4.0 / 3.0 * np.pi * (edges[1:] ** 3 - edges[:-1] ** 3)
    assert np.allclose(gr, hist / (n * rho * shell), rtol=1e-12)
    s.close()


def test_clusters_match_connected_components(psim):
    sp = pytest.importorskip("scipy.sparse")
    csgraph = pytest.importorskip("scipy.sparse.csgraph")
    n, box, scale = 1500, 14.0, 4   # phi ~ 0.29: many contacts closer than 1.2
    s, g = ao_system(psim, n=n, box=box, scale=scale, precision=1, seed=72)
    s.step(5)
    pos = s.download()["pos"].reshape(-1, 3)
    d = min_image(pos[:, None, :] - pos[None, :, :], box)
    r = np.sqrt(np.sum(d * d, axis=2))
    np.fill_diagonal(r, np.inf)
    ncomp, lab = csgraph.connected_components(sp.csr_matrix(r < 1.2), directed=False)
    root, groups, avg = s.clusters(1.2, 4)
    # the same partition, each cluster named by its smallest original index
    first = {}
    for i in range(n):
        first.setdefault(lab[i], i)
    assert np.array_equal(root, np.array([first[lab[i]] for i in range(n)]))
    big = [np.flatnonzero(lab == c) for c in range(ncomp) if np.sum(lab == c) > 4]
    big.sort(key=lambda m: m[0])
    assert len(groups) == len(big) and all(np.array_equal(a, b) for a, b in zip(groups, big))
    assert avg == (sum(len(m) for m in big) // len(big) if big else 0)
    s.close()


# ------------------------------------------------------------ energy, virial

def _pair_u_f(kind, p, r, size):
    """u(r) (zero at the cutoff) and fNet(r) of the plugin force laws
    (AOPotential.cpp:90-99, LJPotential.cpp:96-109, Calibration.cpp:75-81)."""
    rc = p["cutoff"]
    if kind == "AO":
        from oracle import port
        c1, c2 = port.ao_coeffs(p["kT"], p["well_depth"], rc)
        u = 36 / 37 * (r ** -37 - rc ** -37) + c1 * np.log(rc / r) + 0.5 * c2 * (rc * rc - r * r)
        f = -(36 * r ** -38 + c1 / r + c2 * r)
    elif kind == "LJ":
        n, e, lam, y = p["lj_num"], p["kT"] * p["well_depth"], p["debye_length"], p["yukawa_strength"]
        L, Lc = (size / r) ** n, (size / rc) ** n
        u = e * (4 * (L * L - L) - 4 * (Lc * Lc - Lc)
                 + y * lam * (np.exp(-r / lam) / r - np.exp(-rc / lam) / rc))
        f = -e * ((2 * L - 1) * 4 * n * L / r + y * np.exp(-r / lam) * (lam + r) / r ** 2)
    else:
        u = r ** -36 - rc ** -36
        f = -36 * r ** -37
    return u, f


ENERGY_CASES = {
    "AO": (dict(kind="AO", cutoff=1.1, kT=1.0, well_depth=0.25), 12.0, 4),
    "LJ6": (dict(kind="LJ", cutoff=2.5, kT=1.5, well_depth=1 / 1.5, lj_num=6,
                 yukawa_strength=0.0, debye_length=0.5), 15.0, 6),
    "LJ18Y": (dict(kind="LJ", cutoff=2.5, kT=1.0, well_depth=3.0, lj_num=18,
                   yukawa_strength=8.0, debye_length=0.5), 15.0, 6),
    "CAL": (dict(kind="CAL", cutoff=1.1, kT=1.0), 12.0, 4),
}


def _energy_system(psim, case, n, seed, precision=0):
    p, box, scale = ENERGY_CASES[case]
    args = {k: v for k, v in p.items() if k != "kind"}
    force = psim.make_force(p["kind"], **args)
    pos, rad = rsa_state(n, box, seed=seed)
    g = psim.geometry(n, box, box / scale, scale)
    s = psim.System(g, force, precision=precision)
    s.upload(pos, rad)
    return s, g, pos, rad, force


@pytest.mark.parametrize("case", list(ENERGY_CASES))
def test_energy_and_virial_match_pair_sums(psim, case):
    n = 700
    s, g, pos, rad, force = _energy_system(psim, case, n, seed=31)
    u, w = s.energy()
    p = ENERGY_CASES[case][0]
    x = pos.reshape(-1, 3)
    i, j = np.triu_indices(n, 1)
    d = min_image(x[j] - x[i], g.box_size)
    r = np.sqrt(np.sum(d * d, axis=1))
    m = r < p["cutoff"]
    uu, ff = _pair_u_f(p["kind"], p, r[m], rad[i][m] + rad[j][m])
    assert u == pytest.approx(np.sum(uu) / n, rel=1e-12, abs=1e-14)
    assert w == pytest.approx(np.sum(-ff * r[m]) / n, rel=1e-12, abs=1e-14)
    s.close()


@pytest.mark.parametrize("case", ["AO", "LJ18Y"])
def test_energy_gradient_is_the_reference_force(psim, oracle_port, case):
    # u(r) is pinned to the reference's force law: -dU/dx_i (central
    # differences of the GPU energy) equals the oracle's force on i
    n = 500
    s, g, pos, rad, force = _energy_system(psim, case, n, seed=32)
    og = oracle_port.geom(n, g.box_size, g.cell_size, g.cell_scale)
    hi, cse, srt = oracle_port.build_cells(og, pos, rad)
    F, err = oracle_port.forces(og, oracle_port.force_from_params(force.as_dict()), srt, hi, cse)
    assert err == 0
    h = 1e-6
    worst = 0.0
    for i in (0, 17, 123, 499):
        for k in range(3):
            e = np.zeros_like(pos)
            e[3 * i + k] = h
            s.upload(pos + e, rad)
            up = s.energy()[0] * n
            s.upload(pos - e, rad)
            dn = s.energy()[0] * n
            fd = -(up - dn) / (2 * h)
            worst = max(worst, abs(fd - F[3 * i + k]) / max(1.0, abs(F[3 * i + k])))
    # central differences at h = 1e-6: truncation ~h^2 F''' and rounding of
    # the energy sum, both well under 1e-4 of the force here
    assert worst < 1e-4
    s.close()
