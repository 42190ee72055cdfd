"""The kinetic temperature of an aggregating AO gel (phi 0.30, 6 kT contact
attraction at q = 0.08, the 2^23-particle stress workload's parameters at
20,000 particles).  While the colloids fall into their wells the released
energy outpaces the gamma = 1 friction and the kinetic temperature
(getTemperature, analysisGeneral.cpp:26-43) rises to ~3.2 kT by t = 1.  The
oracle -- the reference's own method -- reads the same, at every time step
tried (the rise does not shrink with dt, so it is not a discretisation
error of the velocity reconstruction, brownianIntegrator.cpp:298-356), and a
purely repulsive control stays at kT."""
import math
import os

import numpy as np
import pytest

from oracle import port
from proteinsim2015_gb300 import init

pytestmark = pytest.mark.gpu

N, PHI, Q, A = 20000, 0.30, 0.08, 6.0


def _gel():
    box = init.box_for_phi(N, 0.5, PHI)
    rc = 1.0 + Q
    wd = A * Q / (1.5 + Q)
    scale = int(box // rc)
    pos = init.rsa_native(N, box, 1.0, seed=11).reshape(-1)
    vel = init.maxwell(N, 1.0, seed=11).reshape(-1)
    return box, rc, wd, scale, pos, np.full(N, 0.5), vel


def _gpu_T(psim, precision, dt, wd, skin=0.0):
    box, rc, _, _, pos, rad, vel = _gel()
    scale = int(box // (rc + skin))          # cellSize >= cutOff + skin
    g = psim.geometry(N, box, box / scale, scale)
    s = psim.System(g, psim.make_force("AO", rc, kT=1.0, well_depth=wd), gamma=1.0, dt=dt,
                    kT=1.0, vel_freq=0, seed=5, precision=precision, skin=skin)
    s.upload(pos, rad, vel=vel)
    s.step(int(round(1.0 / dt)))
    T = s.temperature()
    s.close()
    return T


@pytest.fixture(scope="module")
def oracle_T():
    port.set_threads(os.cpu_count() or 1)
    box, rc, wd, scale, pos, rad, vel = _gel()
    dt = 1e-3
    st = port.State(pos, rad, vel=vel)
    err, *_ = port.run(port.geom(N, box, box / scale, scale),
                       port.make_force(port.AO, rc, kT=1.0, well_depth=wd),
                       port.vgb_coeffs(1.0, dt, 1.0), dt, st, 1000, None, vel_freq=0)
    assert err == 0
    return float(np.sum(st.vel ** 2) / 3.0 / N)


def test_gel_heats_as_the_reference_does(psim, oracle_T):
    wd = _gel()[2]
    assert oracle_T > 2.5
    t64 = _gpu_T(psim, psim.PRECISION_FP64, 1e-3, wd)
    tmx = _gpu_T(psim, psim.PRECISION_MIXED, 1e-3, wd, skin=0.3)
    for T in (t64, tmx):
        assert abs(T - oracle_T) < 0.1 * oracle_T


def test_gel_heating_does_not_shrink_with_dt(psim):
    wd = _gel()[2]
    t_coarse = _gpu_T(psim, psim.PRECISION_MIXED, 1e-3, wd)
    t_fine = _gpu_T(psim, psim.PRECISION_MIXED, 2.5e-4, wd)
    assert t_fine > 2.5 and abs(t_fine - t_coarse) < 0.1 * t_fine


def test_repulsive_control_stays_at_kT(psim):
    # the same packing with (almost) no attraction: no energy is released
    T = _gpu_T(psim, psim.PRECISION_MIXED, 1e-3, 1e-9)
    assert abs(T - 1.0) < 0.03
