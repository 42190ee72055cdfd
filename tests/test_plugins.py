"""The plugin contract on the CPU: each GB300 plugin exports the reference's
factory getForce(config*) and a device entry; a host built from the
reference's own sources loads it and runs it through the IForce vtable
(IForce.h:35, defaultForceManager.cpp:55-65, runSim.cpp:35-61); its CPU
getAcceleration matches the oracle; a plugin written outside the library
builds against the plugin header alone; settings.cfg gives the box the
reference derives (system.cpp:28-65)."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT
from gpu_helpers import FORCE_TOL_FP64, rel_per_particle
from plugin_helpers import (YUKAWA_SETTINGS, build_host, build_yukawa, settings_text,
                            write_bin, yukawa_oracle_force)
from proteinsim2015_gb300 import init

SETTINGS_NPZ = os.path.join(ROOT, "tests", "golden", "reference_settings.npz")

CASES = {   # plugin -> (settings, box, scale): states at the reference's integer boxes
    "AOPotential": ({"kT": 1.0, "wellDepth": 4.0, "cutOff": 1.1}, 21, 7),
    "LennardJones": ({"kT": 1.5, "wellDepth": 1 / 1.5, "ljNum": 6, "yukawaStrength": 0.0,
                      "cutOff": 2.5}, 24, 8),
    "Calibration": ({"cutOff": 1.1}, 21, 7),
}


@pytest.fixture(scope="module")
def host(psim, tmp_path_factory):
    return build_host(psim, tmp_path_factory.mktemp("host"))


def _state(n, box, seed=3):
    return init.rsa(n, box, 1.0, seed=seed).reshape(-1), np.full(n, 0.5)


@pytest.mark.parametrize("name", ["AOPotential", "LennardJones", "Calibration"])
def test_plugin_exports_factory_and_device_entry(psim, name):
    lib = C.CDLL(os.path.join(psim.PLUGIN_DIR, name + ".so"))
    for sym in ("getForce", "psim_plugin_abi", "psim_plugin_device_params", "psim_force_launch",
                "psim_plugin_params"):
        assert hasattr(lib, sym), sym
    assert lib.psim_plugin_abi() == 2
    plug = psim.ForcePlugin(os.path.join(psim.PLUGIN_DIR, name + ".so"))
    assert plug.launch and plug.params.cutoff > 0


@pytest.mark.parametrize("name", ["AOPotential", "LennardJones", "Calibration"])
def test_reference_host_runs_gb300_plugin(psim, name):
    # the reference's own config, IForce vtable and defaultForceManager, built
    # from its sources, drive the GB300 plugin against its own plugin
    from oracle import ref
    if not ref.available():
        pytest.skip("the reference is rebuilt only where its sources are")
    settings, box, scale = CASES[name]
    n = 4000
    pos, rad = _state(n, box)
    cs = box // scale
    hi, cse, srt = ref.build_cells(n, box, cs, scale, pos, rad)
    key = {"AOPotential": "AO", "LennardJones": "LJ", "Calibration": "Cal"}[name]
    want = ref.forces(key, settings, n, box, cs, scale, srt, hi, cse)
    got, rc = ref.foreign_forces(os.path.join(psim.PLUGIN_DIR, name + ".so"), settings, n, box,
                                 cs, scale, srt, hi, cse)
    assert rc == 0
    assert np.max(np.abs(got - want)) <= 1e-12 * np.max(np.abs(want))


def _cpu_forces(host, plugin_dir, text, n, box, scale, pos, rad, tmp_path, oracle_port):
    cfgp = tmp_path / "settings.cfg"
    cfgp.write_text(text)
    g = oracle_port.geom(n, box, box // scale, scale)
    hi, cse, srt = oracle_port.build_cells(g, pos, rad)
    out = tmp_path / "force.bin"
    r = subprocess.run([host, "cpu_forces", str(cfgp), plugin_dir, str(n), str(box),
                        str(box // scale), str(scale), write_bin(tmp_path / "s.bin", srt),
                        write_bin(tmp_path / "h.bin", hi), write_bin(tmp_path / "c.bin", cse),
                        str(out)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return np.fromfile(str(out)), (g, hi, cse, srt), r.stdout.strip()


@pytest.mark.parametrize("name", ["AOPotential", "LennardJones", "Calibration"])
def test_plugin_cpu_entry_matches_oracle(psim, host, oracle_port, tmp_path, name):
    settings, box, scale = CASES[name]
    n = 3000
    pos, rad = _state(n, box, seed=9)
    text = settings_text(dict(settings, force=name))
    got, (g, hi, cse, srt), pname = _cpu_forces(host, psim.PLUGIN_DIR, text, n, box, scale, pos,
                                                rad, tmp_path, oracle_port)
    assert pname == name
    f = oracle_port.force_from_params(psim.load_force(psim.Config(text)).as_dict())
    want, err = oracle_port.forces(g, f, srt, hi, cse)
    assert err == 0
    assert rel_per_particle(got, want, oracle_port.force_scale(g, f, srt, hi, cse)) <= FORCE_TOL_FP64


def test_out_of_tree_plugin_builds_and_matches_oracle(psim, host, oracle_port, tmp_path):
    # a fourth potential, written outside the library against its plugin
    # header only, built by the plugin recipe; no rebuild of the library
    so = build_yukawa(tmp_path / "plugins")
    if so is None:
        pytest.skip("nvcc is not available")
    lib = C.CDLL(so)
    assert hasattr(lib, "getForce") and hasattr(lib, "psim_force_launch")
    n, box, scale = 3000, 21, 7
    pos, rad = _state(n, box, seed=4)
    got, (g, hi, cse, srt), pname = _cpu_forces(host, os.path.dirname(so),
                                                settings_text(YUKAWA_SETTINGS), n, box, scale,
                                                pos, rad, tmp_path, oracle_port)
    assert pname == "Yukawa"
    f = yukawa_oracle_force(oracle_port)
    want, err = oracle_port.forces(g, f, srt, hi, cse)
    assert err == 0
    assert rel_per_particle(got, want, oracle_port.force_scale(g, f, srt, hi, cse)) <= FORCE_TOL_FP64


def test_settings_give_the_reference_box(psim, host, tmp_path):
    # the reference's own ClusteredUI/settings.cfg among them: (nParticles,
    # boxSize, cellSize, cellScale) and the concentration as its
    # setSystemConstants derives them, from the C++ host and the Python mirror
    d = np.load(SETTINGS_NPZ)
    keys = [f[5:] for f in d.files if f.startswith("text_")]
    assert "reference_settings_cfg" in keys
    for k in keys:
        text = str(d["text_" + k])
        p = tmp_path / ("%s.cfg" % k)
        p.write_text(text)
        out = subprocess.check_output([host, "constants", str(p)], text=True).split()
        assert [int(v) for v in out[:4]] == d["ints_" + k].tolist(), k
        assert float(out[4]) == float(d["conc_" + k]), k
        st, geom = psim.system_constants(psim.Config(text))
        assert [st["nParticles"], st["boxSize"], st["cellSize"], st["cellScale"]] == \
            d["ints_" + k].tolist(), k
        assert st["concentration"] == float(d["conc_" + k])
        assert geom.box_size == st["boxSize"] and geom.cell_size == st["cellSize"]
