"""Build recipe for libpsim_gb300.so (sm_103a) and the force-plugin shims.

Translation units are compiled in parallel with one -gencode each:
  psim_exact.cu  --fmad=false (FP64 update and plain force form keep the
                 reference's two-rounding a*b+c)
  psim_mixed.cu  FP32 pair math (contraction allowed)
  psim_cells.cu  integer counting sort and layout conversions
  psim_api.cu    host side of the C ABI
  psim_noalloc.cu  the cell-list build on a static device scratch array
The CUDA runtime is linked statically, so the library needs only the driver.
Output goes next to this file (git-ignored) and is what the package loads.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
ROOT = os.path.dirname(HERE)
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libpsim_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = {
    "psim_exact.cu": ["--fmad=false"],
    "psim_mixed.cu": [],
    "psim_cells.cu": [],
    "psim_api.cu": [],
    "psim_noalloc.cu": [],
    # host and device evaluate the RSA trials with the same IEEE operations
    "psim_init.cu": ["--fmad=false", "-Xcompiler", "-ffp-contract=off"],
    "psim_observe.cu": [],
    "psim_adjoint.cu": ["--fmad=false"],
}


def nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.isabs(c) and os.path.exists(c) or not os.path.isabs(c)):
            return c
    return "nvcc"


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src, extra, verbose):
    obj = os.path.join(OUT_DIR, src.replace(".cu", ".o"))
    headers = [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith(".cuh")]
    deps = [os.path.join(CSRC, src)] + headers + [
        os.path.join(ROOT, "include", "psim_gb300.h"), __file__]
    if not _stale(obj, deps):
        return obj
    # -ffp-contract=off: the host compiler on Arm contracts a*b+c into FMA by
    # default, which would move the host-computed vGB coefficients by an ulp
    cmd = [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
           "-Xcompiler", "-fno-fast-math", "-Xcompiler", "-ffp-contract=off",
           "--expt-relaxed-constexpr", *extra,
           "-c", os.path.join(CSRC, src), "-o", obj + ".tmp"]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, r.stdout, r.stderr))
    if verbose and r.stderr:
        sys.stderr.write(r.stderr)
    os.replace(obj + ".tmp", obj)
    return obj


def build(verbose=False, force=False):
    """Compile every translation unit and link libpsim_gb300.so; returns its path."""
    os.makedirs(OUT_DIR, exist_ok=True)
    if force:
        for f in os.listdir(OUT_DIR):
            os.unlink(os.path.join(OUT_DIR, f))
    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda kv: _compile(kv[0], kv[1], verbose), SOURCES.items()))
    if _stale(LIB, objs):
        tmp = LIB + ".tmp%d" % os.getpid()
        cmd = [nvcc(), *ARCH, "-shared", "-cudart", "static", "-o", tmp, *objs]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
        os.replace(tmp, LIB)
    build_plugins()
    return LIB


PLUGINS = ["AOPotential", "LennardJones", "Calibration"]
# the names the reference's own settings.cfg files use for the same plugins
ALIASES = {"AO": "AOPotential", "LJ": "LennardJones", "Cal": "Calibration"}


def build_plugins():
    """The drop-in force plugins: AOPotential.so, LennardJones.so and
    Calibration.so, each exporting the reference's getForce(config*) factory
    (host C++ only; the device functors live in libpsim_gb300.so)."""
    src = os.path.join(CSRC, "plugins", "psim_plugin.cpp")
    hdr = os.path.join(ROOT, "include", "psim_gb300.hpp")
    for name in PLUGINS:
        out = os.path.join(HERE, "plugins", name + ".so")
        if not _stale(out, [src, hdr, os.path.join(ROOT, "include", "psim_gb300.h")]):
            continue
        os.makedirs(os.path.dirname(out), exist_ok=True)
        cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-ffp-contract=off",
               "-I", os.path.join(ROOT, "include"),
               "-DPSIM_PLUGIN_NAME=\"%s\"" % name, src, "-o", out + ".tmp"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("plugin build failed for %s:\n%s" % (name, r.stderr))
        os.replace(out + ".tmp", out)
    for alias, name in ALIASES.items():
        link = os.path.join(HERE, "plugins", alias + ".so")
        if not os.path.lexists(link):
            os.symlink(name + ".so", link)


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
