"""The C-ABI library and the plugin shims: they load and export what the
headers declare; host-side logic that needs no GPU.  CPU only."""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "psim_gb300.h")


def declared_symbols():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(psim_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(psim):
    syms = declared_symbols()
    assert len(syms) >= 25
    missing = [s for s in syms if not hasattr(psim.lib(), s)]
    assert not missing, missing
    out = subprocess.run(["nm", "-D", "--defined-only", psim.LIB_PATH], capture_output=True,
                         text=True).stdout
    exported = set(re.findall(r" T (psim_[a-z0-9_]+)", out))
    assert set(syms) <= exported


def test_abi_version_and_no_device_is_reported(psim):
    assert psim.lib().psim_abi_version() == 4
    if psim.device_count() == 0:
        g = psim.geometry(4, 12, 3, 4)
        with pytest.raises(psim.PsimError) as e:
            psim.cells_build(g, np.random.rand(12) * 12, np.full(4, 0.5))
        assert e.value.code == psim.ERR_NO_DEVICE


@pytest.mark.parametrize("name", ["AOPotential", "LennardJones", "Calibration"])
def test_plugin_exports_factory(psim, name):
    path = os.path.join(psim.PLUGIN_DIR, name + ".so")
    lib = C.CDLL(path)
    assert hasattr(lib, "getForce") and hasattr(lib, "psim_plugin_params")


def test_plugin_defaults_match_reference_constructors(psim):
    # AOPotential.cpp:40-47, LJPotential.cpp:31-55, Calibration.cpp:33-36
    ao = psim.load_force(psim.Config("force = AOPotential\n")).as_dict()
    assert (ao["kind"], ao["well_depth"], ao["cutoff"], ao["kT"]) == ("AO", 0.261, 1.1, 1.0)
    lj = psim.load_force(psim.Config("force = LennardJones\n")).as_dict()
    assert (lj["kind"], lj["well_depth"], lj["yukawa_strength"], lj["lj_num"], lj["cutoff"],
            lj["debye_length"]) == ("LJ", 10.0, 8.0, 18, 2.5, 0.5)
    cal = psim.load_force(psim.Config("force = Calibration\n")).as_dict()
    assert (cal["kind"], cal["cutoff"]) == ("CAL", 1.1)


def test_settings_parse_like_reference(psim):
    # values with trailing ';' parse as their leading number (stod), '#' at column 0
    text = "# comment\nkT = 1.5\nwellDepth = 10;\nljNum = 6;\ncutOff = 2.5\n"
    lj = psim.load_force(psim.Config("force = LennardJones\n" + text)).as_dict()
    assert (lj["kT"], lj["well_depth"], lj["lj_num"]) == (1.5, 10.0, 6)
    p = psim.force_params_from_settings("LennardJones", text).as_dict()
    assert (p["kT"], p["well_depth"], p["lj_num"]) == (1.5, 10.0, 6)
    with pytest.raises(psim.PsimError) as e:
        psim.force_params_from_settings("NoSuchForce", text)
    assert e.value.code == psim.ERR_LOAD
    with pytest.raises(psim.PsimError) as e:
        psim.load_force(psim.Config("force = NoSuchForce\n"))
    assert e.value.code == psim.ERR_LOAD


def test_vgb_coefficients_match_oracle(psim, oracle_port):
    for gamma in (1.0, 0.5, 0.01, 2.0):
        a = psim.vgb_coefficients(gamma, 0.001, 1.0).as_dict()
        b = oracle_port.vgb_coeffs(gamma, 0.001, 1.0).as_dict()
        assert a == b


def test_ao_coefficients_match_oracle(psim, oracle_port):
    assert psim.ao_coefficients(1.0, 0.25, 1.1) == oracle_port.ao_coeffs(1.0, 0.25, 1.1)


def test_cpp_header_and_plugin_loader(tmp_path, psim):
    # A C++ host program that loads a plugin the reference's way
    # (dlopen "./<force>.so", dlsym getForce) and reads the parameters of its
    # device entry.
    src = tmp_path / "host.cpp"
    src.write_text(r'''
#include "psim_gb300.hpp"
#include <cstdio>
int main(int argc, char** argv) {
    PSim::config cfg = PSim::config::fromText("force = LennardJones\nljNum = 6\nwellDepth = 2\n");
    PSim::IForce* f = PSim::loadForces(&cfg, argv[1]);
    psim_force_params p = PSim::requireDevice(f).params;
    std::printf("%s %d %d %.3f\n", f->getName().c_str(), p.kind, p.lj_num, p.well_depth);
    try { PSim::config bad = PSim::config::fromText("force = Nope\n"); PSim::loadForces(&bad, argv[1]); }
    catch (const std::exception& e) { std::printf("caught\n"); }
    return 0;
}
''')
    exe = tmp_path / "host"
    subprocess.check_call(["g++", "-std=c++17", "-I", os.path.join(ROOT, "include"), str(src),
                           "-o", str(exe), "-ldl", "-L", os.path.dirname(psim.LIB_PATH),
                           "-Wl,-rpath," + os.path.dirname(psim.LIB_PATH), "-lpsim_gb300"])
    out = subprocess.check_output([str(exe), psim.PLUGIN_DIR], text=True).split("\n")
    assert out[0] == "LennardJones 2 6 2.000"
    assert out[1] == "caught"


def test_geometry_validation_needs_no_gpu(psim):
    # cellScale < 3 would make the 27-cell stencil visit a cell twice
    g = psim.geometry(4, 12, 6, 2)
    with pytest.raises(psim.PsimError) as e:
        psim.cells_build(g, np.random.rand(12) * 12, np.full(4, 0.5))
    assert e.value.code == psim.ERR_INPUT
    g = psim.geometry(4, 12, 3, 4)
    f = psim.make_force("LJ", 3.5, lj_num=6)
    with pytest.raises(psim.PsimError) as e:  # cellSize below the cutoff
        psim.force_evaluate(f, g, np.zeros(16), np.zeros(8, np.int32), np.zeros(128, np.uint32))
    assert e.value.code == psim.ERR_INPUT


def test_output_arrays_must_be_writeable(psim):
    # the device may write a caller's output array in place: a read-only one
    # is refused on the host, before any call
    ro = np.zeros(12)
    ro.flags.writeable = False
    with pytest.raises(psim.PsimError) as e:
        psim._out(ro, np.float64, 12)
    assert e.value.code == psim.ERR_INPUT
    ok = np.zeros(12)
    assert psim._out(ok, np.float64, 12) is not None


def test_force_list_settings_need_no_gpu(psim):
    # the drop-in pair list's skin and counters are host state: settable and
    # readable without a device; a NaN skin is refused
    psim.set_force_list_skin(0.25)
    psim.set_force_list_skin(0.0)
    with pytest.raises(psim.PsimError) as e:
        psim.set_force_list_skin(float("nan"))
    assert e.value.code == psim.ERR_INPUT
    calls, builds = psim.force_list_stats()
    assert calls >= 0 and 0 <= builds <= max(calls, 0)
