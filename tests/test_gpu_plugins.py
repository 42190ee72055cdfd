"""The plugin device entry on the GPU: every force pass of a system (and of
the force drop-in) runs through the plugin's psim_force_launch, the
library's force templates instantiated with the plugin's own __device__
functor.  The three reference plugins give the library's own forces bit for
bit; a fourth plugin written outside the library is checked against the
oracle; a C++ host builds PSim::system from the reference's own
settings.cfg."""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT
from gpu_helpers import FORCE_TOL_FP64, FORCE_TOL_MIXED, TRAJ_TOL, rel_norm, rel_per_particle
from plugin_helpers import (YUKAWA_SETTINGS, build_host, build_yukawa, settings_text,
                            write_bin, yukawa_oracle_force)
from proteinsim2015_gb300 import init

pytestmark = pytest.mark.gpu

SETTINGS_NPZ = os.path.join(ROOT, "tests", "golden", "reference_settings.npz")

PLUGIN_CASES = {   # plugin -> (settings, n, box, scale)
    "AOPotential": ({"kT": 1.0, "wellDepth": 0.25, "cutOff": 1.1}, 4000, 21.0, 7),
    "LennardJones": ({"kT": 1.5, "wellDepth": 1 / 1.5, "ljNum": 6, "yukawaStrength": 0.0,
                      "cutOff": 2.5}, 6000, 25.0, 8),
    "Calibration": ({"cutOff": 1.1}, 4000, 21.0, 7),
}


def _plugin(psim, name, settings):
    return psim.ForcePlugin(os.path.join(psim.PLUGIN_DIR, name + ".so"),
                            settings_text(dict(settings, force=name)))


@pytest.mark.parametrize("name", list(PLUGIN_CASES))
def test_plugin_entry_gives_library_forces(psim, name):
    settings, n, box, scale = PLUGIN_CASES[name]
    plug = _plugin(psim, name, settings)
    g = psim.geometry(n, box, box / scale, scale)
    pos, rad = init.rsa(n, box, 1.0, seed=12).reshape(-1), np.full(n, 0.5)
    hi, cse, srt = psim.cells_build(g, pos, rad)
    for prec in (psim.PRECISION_FP64, psim.PRECISION_MIXED):
        lib_f = psim.force_evaluate(plug.params, g, srt, hi, cse, precision=prec)
        plug_f = psim.force_evaluate(plug, g, srt, hi, cse, precision=prec)
        assert np.array_equal(lib_f, plug_f), prec


@pytest.mark.parametrize("name", ["AOPotential", "LennardJones"])
@pytest.mark.parametrize("precision", [0, 1])
def test_system_steps_through_plugin_entry(psim, name, precision):
    settings, n, box, scale = PLUGIN_CASES[name]
    plug = _plugin(psim, name, settings)
    g = psim.geometry(n, box, box / scale, scale)
    pos, rad = init.rsa(n, box, 1.0, seed=13).reshape(-1), np.full(n, 0.5)
    vel = init.maxwell(n, settings.get("kT", 1.0), seed=13).reshape(-1)
    out = []
    for force in (plug.params, plug):   # the library's functor, then the plugin's entry
        s = psim.System(g, force, gamma=1.0, dt=0.001, kT=settings.get("kT", 1.0), vel_freq=4,
                        seed=77, precision=precision, skin="auto")
        s.upload(pos, rad, vel=vel)
        s.step(40)
        out.append((s.download(), s.forces(), s.list_builds()))
        s.close()
    (a, fa, la), (b, fb, lb) = out
    for k in ("pos", "pos0", "vel", "frc"):
        assert np.array_equal(a[k], b[k]), k
    assert np.array_equal(fa, fb) and la == lb


@pytest.fixture(scope="module")
def yukawa(psim, tmp_path_factory):
    so = build_yukawa(tmp_path_factory.mktemp("yukawa"))
    if so is None:
        pytest.skip("nvcc is not available")
    return psim.ForcePlugin(so, settings_text(YUKAWA_SETTINGS))


def test_out_of_tree_plugin_system_forces_match_oracle(psim, oracle_port, yukawa):
    n, box, scale = 4000, 24.0, 6                  # phi 0.15, cells of 4 >= 3 + skin
    pos, rad = init.rsa(n, box, 1.0, seed=14).reshape(-1), np.full(n, 0.5)
    g = psim.geometry(n, box, box / scale, scale)
    og = oracle_port.geom(n, box, box / scale, scale)
    f = yukawa_oracle_force(oracle_port)
    hi, cse, srt = oracle_port.build_cells(og, pos, rad)
    want, err = oracle_port.forces(og, f, srt, hi, cse)
    assert err == 0
    scale_i = oracle_port.force_scale(og, f, srt, hi, cse)
    s64 = psim.System(g, yukawa, precision=psim.PRECISION_FP64)
    s64.upload(pos, rad)
    assert rel_per_particle(s64.forces(), want, scale_i) <= FORCE_TOL_FP64
    s64.close()
    smx = psim.System(g, yukawa, precision=psim.PRECISION_MIXED, skin="auto")
    assert smx.skin > 0                            # the pair-list pass of the plugin
    smx.upload(pos, rad)
    assert rel_norm(smx.forces(), want) <= FORCE_TOL_MIXED
    smx.close()
    # the drop-in through the plugin's entry
    assert rel_per_particle(psim.force_evaluate(yukawa, g, srt, hi, cse), want,
                            scale_i) <= FORCE_TOL_FP64


def test_out_of_tree_plugin_trajectory_matches_oracle(psim, oracle_port, yukawa):
    n, box, scale, steps, dt = 4000, 24.0, 6, 20, 0.001
    pos, rad = init.rsa(n, box, 1.0, seed=15).reshape(-1), np.full(n, 0.5)
    rng = np.random.default_rng(15)
    vel = rng.standard_normal(3 * n)
    noise = rng.standard_normal(steps * n * 6)
    g = psim.geometry(n, box, box / scale, scale)
    s = psim.System(g, yukawa, gamma=1.0, dt=dt, kT=1.0, vel_freq=0,
                    precision=psim.PRECISION_FP64, noise_mode=psim.NOISE_INJECTED)
    s.upload(pos, rad, vel=vel)
    s.set_noise(noise, steps)
    s.step(steps)
    out = s.download()
    s.close()
    st = oracle_port.State(pos, rad, vel=vel)
    err, *_ = oracle_port.run(oracle_port.geom(n, box, box / scale, scale),
                              yukawa_oracle_force(oracle_port),
                              oracle_port.vgb_coeffs(1.0, dt, 1.0), dt, st, steps, noise,
                              vel_freq=0)
    assert err == 0
    assert np.max(np.abs(out["pos"] - st.pos)) <= TRAJ_TOL


def test_cpp_system_from_reference_settings_cfg(psim, oracle_port, tmp_path):
    # The reference's own ClusteredUI/settings.cfg: 2500 LJ(18) + Yukawa
    # particles at conc 0.05, scale 5 -> L = 25, cellSize 5 as the reference
    # derives them; PSim::system loads the plugin it names (LJ), builds the
    # grid and steps on the GPU.
    d = np.load(SETTINGS_NPZ)
    text = str(d["text_reference_settings_cfg"])
    n, box, cell, scale = d["ints_reference_settings_cfg"].tolist()
    cfg_path = tmp_path / "settings.cfg"
    cfg_path.write_text(text)
    pos = init.rsa(n, box, 1.0, seed=16).reshape(-1)
    host = build_host(psim, tmp_path)
    r = subprocess.run([host, "system", str(cfg_path), psim.PLUGIN_DIR, "0",
                        write_bin(tmp_path / "pos.bin", pos), str(tmp_path / "f.bin"),
                        str(tmp_path / "p.bin"), "0.01"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert r.stdout.split() == [str(box), str(cell), str(scale), str(n)]
    got = np.fromfile(str(tmp_path / "f.bin"))
    og = oracle_port.geom(n, box, cell, scale)
    f = oracle_port.force_from_params(psim.load_force(psim.Config(text)).as_dict())
    hi, cse, srt = oracle_port.build_cells(og, pos, np.full(n, 0.5))
    want, err = oracle_port.forces(og, f, srt, hi, cse)
    assert err == 0
    assert rel_per_particle(got, want, oracle_port.force_scale(og, f, srt, hi, cse)) <= FORCE_TOL_FP64
    after = np.fromfile(str(tmp_path / "p.bin"))
    assert np.all((after >= 0) & (after < box)) and not np.array_equal(after, pos)
