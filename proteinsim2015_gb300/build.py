"""Build recipe for libpsim_gb300.so (sm_103a) and the force-plugin shims.

Translation units are compiled in parallel with one -gencode each:
  psim_exact.cu  --fmad=false (FP64 update and plain force form keep the
                 reference's two-rounding a*b+c)
  psim_mixed.cu  FP32 pair math (contraction allowed)
  psim_cells.cu  integer counting sort and layout conversions
  psim_api.cu    host side of the C ABI
  psim_noalloc.cu  the cell-list build on a static device scratch array
and the three force plugins (csrc/plugins/*.cu, each compiled twice, see
build_force_plugin).  The CUDA runtime is linked statically, so the library
and the plugins need only the driver.
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


def _compile_any(src, extra, obj, verbose):
    """nvcc -c src -> obj (skipped when obj is newer than src, the library's
    headers and this recipe)."""
    headers = [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith(".cuh")]
    deps = [src] + headers + [os.path.join(ROOT, "include", h)
                              for h in ("psim_gb300.h", "psim_gb300.hpp")] + [__file__]
    if not _stale(obj, deps):
        return obj
    # -ffp-contract=off: the host compiler on Arm contracts a*b+c into FMA by
    # default, which would move the host-computed vGB coefficients by an ulp
    cmd = [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
           "-Xcompiler", "-fno-fast-math", "-Xcompiler", "-ffp-contract=off",
           "--expt-relaxed-constexpr", *extra,
           "-c", src, "-o", obj + ".tmp"]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, r.stdout, r.stderr))
    if verbose and r.stderr:
        sys.stderr.write(r.stderr)
    os.replace(obj + ".tmp", obj)
    return obj


def _link(objs, out):
    if not _stale(out, objs):
        return out
    os.makedirs(os.path.dirname(out), exist_ok=True)
    tmp = out + ".tmp%d" % os.getpid()
    cmd = [nvcc(), *ARCH, "-shared", "-cudart", "static", "-o", tmp, *objs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link of %s failed:\n%s\n%s" % (out, r.stdout, r.stderr))
    os.replace(tmp, out)
    return out


# The force plugins built with the library: the reference's three plugins,
# each exporting getForce(config*) and the device entry psim_force_launch.
PLUGINS = ["AOPotential", "LennardJones", "Calibration"]
PLUGIN_DIR = os.path.join(HERE, "plugins")
# the names the reference's own settings.cfg files use for the same plugins
ALIASES = {"AO": "AOPotential", "LJ": "LennardJones", "Cal": "Calibration"}


def _plugin_jobs(src, obj_dir, verbose=False, include_dirs=()):
    """The two compiles of a plugin source (psim_plugin.cuh): part 1, the
    plain FP64 pass, without FMA contraction; part 2, the mixed passes and
    the host entries."""
    base = os.path.splitext(os.path.basename(src))[0]
    inc = [x for d in include_dirs for x in ("-I", d)]
    return [
        (src, ["-DPSIM_PLUGIN_PART=1", "--fmad=false", *inc],
         os.path.join(obj_dir, base + ".part1.o"), verbose),
        (src, ["-DPSIM_PLUGIN_PART=2", *inc], os.path.join(obj_dir, base + ".part2.o"), verbose),
    ]


def build_force_plugin(src, out=None, include_dirs=(), verbose=False):
    """Compile a force plugin source into a shared object (default: the
    source's name + .so beside it) and return its path.  The source includes
    proteinsim2015_gb300/csrc/psim_plugin.cuh and ends with
    PSIM_FORCE_PLUGIN(Class); it needs nothing else of the library."""
    src = os.path.abspath(src)
    out = out or os.path.splitext(src)[0] + ".so"
    obj_dir = os.path.join(os.path.dirname(os.path.abspath(out)), "_build")
    os.makedirs(obj_dir, exist_ok=True)
    objs = [_compile_any(*j) for j in _plugin_jobs(src, obj_dir, verbose, include_dirs)]
    return _link(objs, out)


def build(verbose=False, force=False):
    """Compile every translation unit, link libpsim_gb300.so and the force
    plugins; returns the library's path."""
    os.makedirs(OUT_DIR, exist_ok=True)
    if force:
        for f in os.listdir(OUT_DIR):
            os.unlink(os.path.join(OUT_DIR, f))
    jobs = [(os.path.join(CSRC, src), extra, os.path.join(OUT_DIR, src.replace(".cu", ".o")),
             verbose) for src, extra in SOURCES.items()]
    for name in PLUGINS:
        jobs += _plugin_jobs(os.path.join(CSRC, "plugins", name + ".cu"), OUT_DIR, verbose)
    with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        objs = list(ex.map(lambda j: _compile_any(*j), jobs))
    _link(objs[:len(SOURCES)], LIB)
    for k, name in enumerate(PLUGINS):
        i = len(SOURCES) + 2 * k
        _link(objs[i:i + 2], os.path.join(PLUGIN_DIR, name + ".so"))
    for alias, name in ALIASES.items():
        link = os.path.join(PLUGIN_DIR, alias + ".so")
        if not os.path.lexists(link):
            os.symlink(name + ".so", link)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
