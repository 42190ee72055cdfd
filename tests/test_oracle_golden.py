"""The oracle restatement against golden vectors produced by the reference
itself (tests/golden/make_golden.py).  CPU only."""
import numpy as np
import pytest

from conftest import settings_of

KEYS = ("y", "coeff0", "coeff1", "coeff2", "coeff3", "sig1", "sig2", "corr", "dev", "goy2",
        "goy3", "hn", "gn")


def _geom(port, golden):
    n, box, cs, scale = golden["cellsA_geom"]
    return port.geom(n, box, cs, scale)


def _force_from_settings(port, plugin, s):
    if plugin == "Cal":
        return port.make_force(port.CAL, s["cutOff"])
    if plugin == "AO":
        return port.make_force(port.AO, s["cutOff"], kT=s["kT"], well_depth=s["wellDepth"])
    return port.make_force(port.LJ, s["cutOff"], kT=s["kT"], well_depth=s["wellDepth"],
                           lj_num=s["ljNum"], yuk_str=s["yukawaStrength"],
                           debye_length=s["debyeLength"])


PLUGIN_OF = {"AO": "AO", "AOq": "AO", "LJ6": "LJ", "LJ18": "LJ", "YUK": "LJ", "CAL": "Cal"}


def test_cells_bit_exact(oracle_port, golden):
    g = _geom(oracle_port, golden)
    hi, cse, srt = oracle_port.build_cells(g, golden["cellsA_pos"], golden["cellsA_radius"])
    assert np.array_equal(hi, golden["cellsA_hash_index"])
    assert np.array_equal(cse, golden["cellsA_cse"])
    assert np.array_equal(srt, golden["cellsA_sorted"])


@pytest.mark.parametrize("key", sorted(PLUGIN_OF))
def test_forces_bit_exact(oracle_port, golden, key):
    g = _geom(oracle_port, golden)
    s = settings_of(golden, "forceA_%s_settings" % key)
    f = _force_from_settings(oracle_port, PLUGIN_OF[key], s)
    out, err = oracle_port.forces(g, f, golden["cellsA_sorted"], golden["cellsA_hash_index"],
                                  golden["cellsA_cse"])
    assert err == 0
    # same pair order inside each cell as the stable-sorted fixture: bit-exact
    assert np.array_equal(out, golden["forceA_%s" % key])


@pytest.mark.parametrize("gamma", [1.0, 0.5, 0.01, 0.049, 2.0])
def test_vgb_coefficients_bit_exact(oracle_port, golden, gamma):
    c = oracle_port.vgb_coeffs(gamma, 0.001, 1.0).as_dict()
    ref = golden["vgb_%g" % gamma]
    assert np.array_equal(np.array([c[k] for k in KEYS]), ref)


def test_vgb_known_answers(oracle_port):
    # values the reference prints for gamma=1, dt=1e-3 (brownianIntegrator.cpp:87-98)
    c = oracle_port.vgb_coeffs(1.0, 0.001, 1.0)
    assert abs(c.sig1 - 0.000026) < 5e-7
    assert abs(c.corr - 0.5) < 1e-6
    assert abs(c.dev - 0.866025) < 1e-6
    assert abs(c.coeff0 - 0.999000) < 1e-6
    assert abs(c.coeff1 - 0.999500) < 1e-6
    assert abs(c.coeff2 - 0.000083) < 1e-6
    assert abs(c.coeff3 - 0.499833) < 1e-6


def test_low_gamma_branch_keeps_high_coeff0(oracle_port):
    # setupLow does not set coEff0 (brownianIntegrator.cpp:68-74, :135-166)
    lo = oracle_port.vgb_coeffs(0.01, 0.001, 1.0)
    assert lo.coeff0 == np.exp(-0.01 * 0.001)
    hi = oracle_port.vgb_coeffs(0.05, 0.001, 1.0)
    assert hi.coeff1 == (1.0 - np.exp(-0.05 * 0.001)) / (0.05 * 0.001)


def test_ao_contact_value(oracle_port):
    # AO potential U(r) = a1 (1 + a2 r + a3 r^3) (AOPotential.cpp:50-52) has the
    # contact value U(1) = -kT wd (rc + 0.5)/(rc - 1), exactly -16 kT wd at rc = 1.1.
    # The plugin's attraction c1/r + c2 r is (dU/dr)/r: the force along the
    # unit vector carries an extra 1/r (AOPotential.cpp:96-99).
    kT, wd, rc = 1.0, 0.25, 1.1
    c1, c2 = oracle_port.ao_coeffs(kT, wd, rc)
    a2, a3 = -3.0 / (2.0 * rc), 1.0 / (2.0 * rc ** 3)
    a1 = -c1 / a2
    assert abs(c2 - (-3.0 * a1 * a3)) < 1e-12 * abs(c2)
    u1 = a1 * (1.0 + a2 + a3)
    assert abs(u1 - (-kT * wd * (rc + 0.5) / (rc - 1.0))) < 1e-12 * 16
    assert abs(u1 - (-16.0 * kT * wd)) < 1e-12 * 16
    r = 1.05
    dudr = a1 * (a2 + 3.0 * a3 * r * r)
    assert abs((c1 / r + c2 * r) - (-dudr / r)) < 1e-12 * abs(dudr)


@pytest.mark.parametrize("tag", ["AO", "LJ"])
def test_trajectory_bit_exact(oracle_port, golden, tag):
    n, box, cs, scale = golden["cellsA_geom"]
    g = oracle_port.geom(n, box, cs, scale)
    s = settings_of(golden, "traj%s_settings" % tag)
    steps, vel_freq = golden["traj%s_meta" % tag]
    f = _force_from_settings(oracle_port, tag, s)
    c = oracle_port.vgb_coeffs(s["gamma"], s["timeStep"], s["kT"])
    st = oracle_port.State(golden["cellsA_pos"], golden["cellsA_radius"],
                           vel=golden["traj%s_vel0" % tag])
    err, *_ = oracle_port.run(g, f, c, s["timeStep"], st, int(steps), golden["traj%s_noise" % tag],
                              vel_freq=int(vel_freq))
    assert err == 0
    assert np.array_equal(st.pos, golden["traj%s_pos" % tag])
    assert np.array_equal(st.pos0, golden["traj%s_pos0" % tag])
    assert np.array_equal(st.vel, golden["traj%s_vel" % tag])
    # forces: the reference's in-cell order is unspecified, so the sums may
    # differ in the last bits
    for k in ("frc", "frc0"):
        ref = golden["traj%s_%s" % (tag, k)]
        assert np.max(np.abs(getattr(st, k) - ref)) <= 1e-12 * np.max(np.abs(ref))


@pytest.mark.parametrize("seed", [90210, 180420, 7])
def test_reference_rng(oracle_port, golden, seed):
    assert np.array_equal(oracle_port.fastrandom_draws(seed, 256), golden["rng_%d" % seed])


def test_overlap_error_code(oracle_port, golden):
    g = oracle_port.geom(2, 12, 3, 4)
    pos = np.array([1.0, 1.0, 1.0, 1.5, 1.0, 1.0])  # r = 0.5 < 0.8 * 1.0
    hi, cse, srt = oracle_port.build_cells(g, pos, np.full(2, 0.5))
    _, err = oracle_port.forces(g, oracle_port.make_force(oracle_port.AO, 1.1, well_depth=1.0),
                                srt, hi, cse)
    assert err == 7704
