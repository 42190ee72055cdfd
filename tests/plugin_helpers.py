"""Shared set-up for the plugin tests: the C++ test host, the out-of-tree
Yukawa plugin, and the oracle's view of that plugin."""
import os
import shutil
import subprocess

import numpy as np

from conftest import ROOT

HOST_SRC = os.path.join(ROOT, "tests", "plugins", "plugin_host.cpp")
YUKAWA_SRC = os.path.join(ROOT, "tests", "plugins", "yukawa_plugin.cu")
YUKAWA_SETTINGS = {"force": "Yukawa", "yukawaAmplitude": 10.0, "kappa": 4.0, "sigma": 1.0,
                   "cutOff": 3.0}


def settings_text(d):
    return "".join("%s = %r\n" % (k, v) if not isinstance(v, str) else "%s = %s\n" % (k, v)
                   for k, v in d.items())


def build_host(psim, out_dir):
    exe = os.path.join(str(out_dir), "plugin_host")
    libdir = os.path.dirname(psim.LIB_PATH)
    subprocess.check_call(["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"),
                           HOST_SRC, "-o", exe, "-ldl", "-L", libdir, "-Wl,-rpath," + libdir,
                           "-lpsim_gb300"])
    return exe


def build_yukawa(out_dir):
    """The out-of-tree plugin, built by the library's plugin recipe into
    out_dir/Yukawa.so (None when nvcc is absent)."""
    from proteinsim2015_gb300 import build
    if not (shutil.which("nvcc") or os.path.exists("/usr/local/cuda/bin/nvcc")):
        return None
    return build.build_force_plugin(YUKAWA_SRC, out=os.path.join(str(out_dir), "Yukawa.so"),
                                    include_dirs=[build.CSRC])


def yukawa_oracle_force(port, d=YUKAWA_SETTINGS):
    """The plugin's force as the LennardJones plugin's Yukawa term with ljNum
    0 (LJPotential.cpp:96-109): kT wellDepth yukawaStrength = A kappa
    e^{kappa sigma}, debyeLength = 1/kappa."""
    amp = d["yukawaAmplitude"] * d["kappa"] * np.exp(d["kappa"] * d["sigma"])
    return port.make_force(port.LJ, d["cutOff"], kT=1.0, well_depth=1.0, yuk_str=amp,
                           debye_length=1.0 / d["kappa"], lj_num=0)


def write_bin(path, a):
    np.ascontiguousarray(a).tofile(str(path))
    return str(path)
