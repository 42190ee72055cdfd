"""ctypes binding of the reference rebuilt from its own sources (oracle/_ref).

TEST INFRASTRUCTURE ONLY.  Available only where the reference tree exists
(oracle/build_ref.sh); callers must check ``available()``.  The reference
terminates its process on physical errors (exit 7703/7704/7705), so error
paths are exercised in a child process (``run_in_child``).
"""
import ctypes as C
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
LIB = os.path.join(REF_DIR, "libpsimref.so")
RNG_LIB = os.path.join(REF_DIR, "libpsimref_rng.so")
REFERENCE = os.environ.get("PSIM_REFERENCE", "/root/reference")


def build():
    if not os.path.isdir(os.path.join(REFERENCE, "ClusteredCore", "src")):
        return False
    subprocess.check_call(["sh", os.path.join(HERE, "build_ref.sh")],
                          stdout=subprocess.DEVNULL)
    return True


def available():
    return os.path.exists(LIB) and os.path.exists(RNG_LIB)


_lib = None
_rng = None


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(LIB)
        P = C.c_void_p
        _lib.psimref_build_cells.argtypes = [C.c_int] * 4 + [P] * 5 + [C.c_int]
        _lib.psimref_forces.argtypes = [C.c_char_p, C.c_char_p] + [C.c_int] * 4 + [P] * 4 + [C.c_int]
        _lib.psimref_vgb_coeffs.argtypes = [C.c_char_p, P]
        _lib.psimref_run.argtypes = ([C.c_char_p, C.c_char_p] + [C.c_int] * 5 + [P] * 12
                                     + [C.c_int])
        _lib.psimref_foreign_forces.argtypes = ([C.c_char_p, C.c_char_p] + [C.c_int] * 4 +
                                                [P] * 4 + [C.c_int])
        _lib.psimref_analysis.argtypes = [C.c_int] * 4 + [P] * 7 + [C.c_double] + [P] * 4 + [
            C.c_char_p]
        _lib.psimref_system_constants.argtypes = [C.c_char_p] + [C.POINTER(C.c_int)] * 4 + [
            C.POINTER(C.c_double)]
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


def write_settings(settings):
    """Write a settings.cfg (``key = value`` lines, as config.cpp:27-56 reads)."""
    fd, path = tempfile.mkstemp(prefix="psimref_", suffix=".cfg")
    with os.fdopen(fd, "w") as fh:
        for k, v in settings.items():
            fh.write("%s = %s\n" % (k, v))
    return path


def foreign_forces(plugin_path, settings, n, box, cell_size, scale, sorted_, hi, cse,
                   threads=1):
    """The reference's defaultForceManager::getAcceleration on a plugin it
    dlopens by path (runSim.cpp:35-61), e.g. a GB300 plugin; (force, status)."""
    path = write_settings(settings)
    try:
        out = np.zeros(3 * n)
        rc = lib().psimref_foreign_forces(plugin_path.encode(), path.encode(), n, int(box),
                                          int(cell_size), scale, _p(sorted_), _p(hi), _p(cse),
                                          _p(out), threads)
        return out, rc
    finally:
        os.unlink(path)


def analysis(n, box, cell_size, scale, pos, pos0, vel, frc, frc0, radius, mass,
             current_time, out_prefix):
    """The reference's analysis of a state (see psimref_analysis): returns
    (coordination numbers, cluster of each particle (-1: none), number of
    clusters, [temperature, mean displacement, <EAP>]) and writes
    out_prefix.txt / .xyz with writeSystem / writeSystemXYZ."""
    f = lambda a: np.ascontiguousarray(a, np.float64)
    coor = np.zeros(n, np.int32)
    clu = np.zeros(n, np.int32)
    nc = C.c_int()
    stats = np.zeros(3)
    lib().psimref_analysis(n, int(box), int(cell_size), scale, _p(f(pos)), _p(f(pos0)),
                           _p(f(vel)), _p(f(frc)), _p(f(frc0)), _p(f(radius)), _p(f(mass)),
                           float(current_time), _p(coor), _p(clu), C.byref(nc), _p(stats),
                           out_prefix.encode())
    return coor, clu, nc.value, stats


def system_constants(settings_path):
    """The reference's setSystemConstants on a settings.cfg file: (nParticles,
    boxSize, cellSize, cellScale, concentration)."""
    v = [C.c_int() for _ in range(4)]
    c = C.c_double()
    lib().psimref_system_constants(settings_path.encode(), *[C.byref(x) for x in v], C.byref(c))
    return tuple(x.value for x in v) + (c.value,)


def build_cells(n, box, cell_size, scale, pos, radius, threads=1):
    pos = np.ascontiguousarray(pos, np.float64).reshape(-1)
    radius = np.ascontiguousarray(radius, np.float64)
    hi = np.empty(2 * n, np.int32)
    cse = np.empty(2 * scale ** 3, np.uint32)
    srt = np.empty(4 * n, np.float64)
    lib().psimref_build_cells(n, int(box), int(cell_size), scale, _p(pos), _p(radius),
                              _p(hi), _p(cse), _p(srt), threads)
    return hi, cse, srt


def forces(plugin, settings, n, box, cell_size, scale, sorted_, hi, cse, threads=1):
    path = write_settings(settings)
    try:
        out = np.zeros(3 * n)
        rc = lib().psimref_forces(plugin.encode(), path.encode(), n, int(box), int(cell_size),
                                  scale, _p(np.ascontiguousarray(sorted_, np.float64)),
                                  _p(np.ascontiguousarray(hi, np.int32)),
                                  _p(np.ascontiguousarray(cse, np.uint32)), _p(out), threads)
        assert rc == 0, rc
        return out
    finally:
        os.unlink(path)


VGB_KEYS = ("y", "coeff0", "coeff1", "coeff2", "coeff3", "sig1", "sig2", "corr", "dev",
            "goy2", "goy3", "hn", "gn")


def vgb_coeffs(settings):
    path = write_settings(settings)
    try:
        out = np.zeros(13)
        lib().psimref_vgb_coeffs(path.encode(), _p(out))
        return dict(zip(VGB_KEYS, out.tolist()))
    finally:
        os.unlink(path)


def run(plugin, settings, n, box, cell_size, scale, n_steps, noise, pos, pos0, vel, frc,
        frc0, radius, mass, threads=1):
    """Run the reference hot loop (system::run) n_steps; state arrays are
    updated in place.  Returns (hash_index, cell_start_end, sorted, last_force)."""
    path = write_settings(settings)
    try:
        hi = np.empty(2 * n, np.int32)
        cse = np.empty(2 * scale ** 3, np.uint32)
        srt = np.empty(4 * n)
        lf = np.empty(3 * n)
        noise = np.ascontiguousarray(noise, np.float64).reshape(-1)
        rc = lib().psimref_run(plugin.encode(), path.encode(), n, int(box), int(cell_size), scale,
                               n_steps, _p(noise), _p(pos), _p(pos0), _p(vel), _p(frc),
                               _p(frc0), _p(radius), _p(mass), _p(hi), _p(cse), _p(srt),
                               _p(lf), threads)
        assert rc == 0, rc
        return hi, cse, srt, lf
    finally:
        os.unlink(path)


def rng_draws(seed, count):
    global _rng
    if _rng is None:
        _rng = C.CDLL(RNG_LIB)
        _rng.psimref_rng_draw.argtypes = [C.c_int, C.c_int, C.c_void_p]
    out = np.zeros(count)
    _rng.psimref_rng_draw(seed, count, _p(out))
    return out


def run_in_child(code):
    """Run python ``code`` (with oracle.ref importable) in a child process;
    returns its exit status (the reference exits on physical errors)."""
    env = dict(os.environ)
    env["PYTHONPATH"] = os.path.dirname(HERE) + os.pathsep + env.get("PYTHONPATH", "")
    p = subprocess.run([sys.executable, "-c", code], env=env, stdout=subprocess.DEVNULL,
                       stderr=subprocess.DEVNULL, timeout=120)
    return p.returncode
