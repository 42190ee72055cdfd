"""ctypes binding of the oracle restatement (psim_oracle.c).

TEST INFRASTRUCTURE ONLY -- the checker and the CPU "port" baseline.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libpsim_oracle.so")

AO, LJ, CAL, AO_YUK = 1, 2, 3, 4


def build(force=False):
    """Compile psim_oracle.c and psim_tangent.c (no FMA contraction, so x86
    and Arm agree)."""
    srcs = [os.path.join(HERE, f) for f in ("psim_oracle.c", "psim_tangent.c")]
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(
            [os.path.getmtime(f) for f in srcs] + [os.path.getmtime(os.path.join(HERE,
                                                                            "psim_oracle.h"))]):
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    tmp = LIB + ".tmp%d" % os.getpid()
    subprocess.check_call(["gcc", "-O2", "-std=gnu99", "-fopenmp", "-fPIC", "-shared",
                           "-ffp-contract=off", "-fno-fast-math", "-Wall",
                           *srcs, "-o", tmp, "-lm"])
    os.replace(tmp, LIB)
    return LIB


class Geom(C.Structure):
    _fields_ = [("n", C.c_int), ("box", C.c_double), ("cell_size", C.c_double),
                ("scale", C.c_int)]


class Force(C.Structure):
    _fields_ = [("kind", C.c_int), ("cutoff", C.c_double), ("ao_c1", C.c_double),
                ("ao_c2", C.c_double), ("kT", C.c_double), ("well_depth", C.c_double),
                ("yuk_str", C.c_double), ("debye_length", C.c_double),
                ("lj_num", C.c_int), ("cutoff2", C.c_double)]


class Vgb(C.Structure):
    _fields_ = [(k, C.c_double) for k in (
        "y", "coeff0", "coeff1", "coeff2", "coeff3", "sig1", "sig2", "corr", "dev",
        "goy2", "goy3", "hn", "gn")]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class AdjParams(C.Structure):
    """oracle_adj_params: the fields of psim_adjoint_params."""
    _fields_ = [("kT", C.c_double), ("ao_well_depth", C.c_double), ("ao_cutoff", C.c_double),
                ("yuk_amplitude", C.c_double), ("yuk_length", C.c_double),
                ("yuk_cutoff", C.c_double), ("ao_range", C.c_double),
                ("lj_epsilon", C.c_double), ("lj_sigma", C.c_double), ("lj_cutoff", C.c_double),
                ("lj_n", C.c_int32)]


class FastRandom(C.Structure):
    _fields_ = [("istack", C.c_int32 * 58), ("jrand", C.c_int32), ("init", C.c_int32),
                ("deviate_available", C.c_int32), ("stored_deviate", C.c_float)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(build())
        P = C.c_void_p
        _lib.oracle_hash.argtypes = [C.POINTER(Geom), P, P]
        _lib.oracle_sort.argtypes = [C.POINTER(Geom), P]
        _lib.oracle_reorder.argtypes = [C.POINTER(Geom), P, P, P, P, P]
        _lib.oracle_build_cells.argtypes = [C.POINTER(Geom), P, P, P, P, P]
        _lib.oracle_forces.argtypes = [C.POINTER(Geom), C.POINTER(Force), P, P, P, P]
        _lib.oracle_forces.restype = C.c_int
        _lib.oracle_force_scale.argtypes = [C.POINTER(Geom), C.POINTER(Force), P, P, P, P]
        _lib.oracle_vgb_coeffs.argtypes = [C.c_double, C.c_double, C.c_double, C.POINTER(Vgb)]
        _lib.oracle_push_force.argtypes = [C.c_int, P, P, P]
        _lib.oracle_vgb_step.argtypes = [C.POINTER(Geom), C.POINTER(Vgb), C.c_double, C.c_int,
                                         C.c_int, P, P, P, P, P, P, P, P, P]
        _lib.oracle_vgb_step.restype = C.c_int
        _lib.oracle_run.argtypes = [C.POINTER(Geom), C.POINTER(Force), C.POINTER(Vgb),
                                    C.c_double, C.c_int, C.c_int, C.c_int,
                                    C.POINTER(C.c_int), P, C.c_int] + [P] * 13
        _lib.oracle_run.restype = C.c_int
        _lib.oracle_ao_coeffs.argtypes = [C.c_double, C.c_double, C.c_double,
                                          C.POINTER(C.c_double), C.POINTER(C.c_double)]
        _lib.oracle_set_threads.argtypes = [C.c_int]
        _lib.oracle_get_threads.restype = C.c_int
        _lib.oracle_fastrandom_init.argtypes = [C.POINTER(FastRandom)]
        _lib.oracle_fastrandom_g250.argtypes = [C.POINTER(FastRandom), C.c_int]
        _lib.oracle_fastrandom_g250.restype = C.c_double
        _lib.oracle_fastrandom_fill.argtypes = [C.POINTER(FastRandom), C.c_int, C.c_int, C.c_int,
                                                C.c_int, P]
        _lib.oracle_adjoint_tangent.argtypes = ([C.c_int, C.c_double, C.POINTER(AdjParams),
                                                 C.POINTER(Vgb), C.c_double, C.c_double,
                                                 C.c_int, C.c_int, C.c_double, C.c_double,
                                                 C.c_int, C.c_double] + [P] * 7)
        _lib.oracle_adjoint_tangent.restype = C.c_int
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


def set_threads(n):
    lib().oracle_set_threads(int(n))


def get_threads():
    return lib().oracle_get_threads()


def ao_coeffs(kT, well_depth, cutoff):
    c1, c2 = C.c_double(), C.c_double()
    lib().oracle_ao_coeffs(kT, well_depth, cutoff, C.byref(c1), C.byref(c2))
    return c1.value, c2.value


def make_force(kind, cutoff, kT=1.0, well_depth=0.0, yuk_str=0.0, debye_length=0.5,
               lj_num=18, cutoff2=0.0):
    f = Force(kind=kind, cutoff=cutoff, kT=kT, well_depth=well_depth, yuk_str=yuk_str,
              debye_length=debye_length, lj_num=lj_num, cutoff2=cutoff2)
    if kind in (AO, AO_YUK):
        f.ao_c1, f.ao_c2 = ao_coeffs(kT, well_depth, cutoff)
    return f


def force_from_params(p):
    """oracle Force from ``proteinsim2015_gb300.ForceParams.as_dict()``: for the
    AO + LJ(n) composite the AO part uses well_depth/cutoff and the LJ part
    well_depth2/cutoff2."""
    kind = {"AO": AO, "LJ": LJ, "CAL": CAL, "AO_YUK": AO_YUK}[p["kind"]]
    kT = p.get("kT", 1.0)
    if kind == AO_YUK:
        f = make_force(kind, p["cutoff"], kT=kT, well_depth=p["well_depth2"],
                       yuk_str=p.get("yukawa_strength", 0.0),
                       debye_length=p.get("debye_length", 0.5), lj_num=p.get("lj_num", 0),
                       cutoff2=p["cutoff2"])
        f.ao_c1, f.ao_c2 = ao_coeffs(kT, p["well_depth"], p["cutoff"])
        return f
    return make_force(kind, p["cutoff"], kT=kT, well_depth=p.get("well_depth", 0.0),
                      yuk_str=p.get("yukawa_strength", 0.0),
                      debye_length=p.get("debye_length", 0.5), lj_num=p.get("lj_num", 18))


def geom(n, box, cell_size, scale):
    return Geom(n=int(n), box=float(box), cell_size=float(cell_size), scale=int(scale))


def build_cells(g, pos, radius):
    n = g.n
    pos = np.ascontiguousarray(pos, np.float64)
    radius = np.ascontiguousarray(radius, np.float64)
    hi = np.empty(2 * n, np.int32)
    cse = np.empty(2 * g.scale ** 3, np.uint32)
    sorted_ = np.empty(4 * n, np.float64)
    lib().oracle_build_cells(C.byref(g), _p(pos), _p(radius), _p(hi), _p(cse), _p(sorted_))
    return hi, cse, sorted_


def forces(g, f, sorted_, hi, cse):
    out = np.zeros(3 * g.n, np.float64)
    err = lib().oracle_forces(C.byref(g), C.byref(f), _p(sorted_), _p(hi), _p(cse), _p(out))
    return out, err


def force_scale(g, f, sorted_, hi, cse):
    out = np.zeros(g.n, np.float64)
    lib().oracle_force_scale(C.byref(g), C.byref(f), _p(sorted_), _p(hi), _p(cse), _p(out))
    return out


def vgb_coeffs(gamma, dt, kT):
    c = Vgb()
    lib().oracle_vgb_coeffs(gamma, dt, kT, C.byref(c))
    return c


class State:
    """Particle state in the reference's original order (AoS xyz)."""

    def __init__(self, pos, radius, mass=None, vel=None, pos0=None, frc=None, frc0=None):
        n = len(radius)
        self.n = n
        self.pos = np.ascontiguousarray(pos, np.float64).reshape(-1).copy()
        self.radius = np.ascontiguousarray(radius, np.float64).copy()
        self.mass = np.ones(n) if mass is None else np.ascontiguousarray(mass, np.float64).copy()
        z = lambda a: np.zeros(3 * n) if a is None else np.ascontiguousarray(a, np.float64).reshape(-1).copy()
        self.vel, self.pos0, self.frc, self.frc0 = z(vel), z(pos0), z(frc), z(frc0)
        self.mem = np.zeros(3 * n)
        self.mem_corr = np.zeros(3 * n)
        self.vel_counter = 0
        self.step = 0

    def copy(self):
        s = State.__new__(State)
        s.__dict__ = {k: (v.copy() if isinstance(v, np.ndarray) else v)
                      for k, v in self.__dict__.items()}
        return s


def run(g, f, c, dt, state, n_steps, noise, vel_freq=1000, cells=None):
    """Advance ``state`` n_steps through the reference hot loop; returns
    (err, hash_index, cell_start_end, sorted, last_force).  ``noise`` holds
    whole steps of n*6 Gaussians (reused cyclically when shorter than
    n_steps), or None for the oracle's own counter-based generator.  ``cells`` (hash_index, cse, sorted) continues from a
    previous call's cell list instead of rebuilding it."""
    n = g.n
    if noise is None:   # counter-based Gaussians generated inside the oracle
        noise_steps = 0
    else:
        noise = np.ascontiguousarray(noise, np.float64).reshape(-1)
        noise_steps = noise.size // (n * 6) if n else 1
        assert noise_steps >= 1
    if cells is None:
        hi, cse, sorted_ = build_cells(g, state.pos, state.radius)
    else:
        hi, cse, sorted_ = cells
    force = np.zeros(3 * n)
    vc = C.c_int(state.vel_counter)
    err = lib().oracle_run(C.byref(g), C.byref(f), C.byref(c), dt, state.step, n_steps,
                           vel_freq, C.byref(vc), _p(noise), noise_steps, _p(state.pos),
                           _p(state.pos0),
                           _p(state.vel), _p(state.frc), _p(state.frc0), _p(state.radius),
                           _p(state.mass), _p(state.mem), _p(state.mem_corr), _p(hi),
                           _p(cse), _p(sorted_), _p(force))
    state.vel_counter = vc.value
    state.step += n_steps
    return err, hi, cse, sorted_, force


def fastrandom_draws(seed, count):
    r = FastRandom()
    lib().oracle_fastrandom_init(C.byref(r))
    return np.array([lib().oracle_fastrandom_g250(C.byref(r), seed) for _ in range(count)])


class ReferenceNoise:
    """The reference's own noise stream: one fastRandom generator per particle,
    seeded seed*(i+1) as brownianIntegrator does (valid while that product
    fits an int, e.g. N = 4000 at seed 90210).  ``take(k)`` returns the next k
    steps in the injected-noise layout (k*n*6 doubles); the first call's first
    step is firstStep's three draws."""

    def __init__(self, n, seed=90210):
        assert seed * n < 2 ** 31, "seed*(i+1) overflows an int: the reference stream breaks"
        self.n, self.seed, self.first = int(n), int(seed), 1
        self.gens = (FastRandom * self.n)()
        for g in self.gens:
            lib().oracle_fastrandom_init(C.byref(g))

    def take(self, n_steps):
        out = np.empty(int(n_steps) * self.n * 6)
        lib().oracle_fastrandom_fill(self.gens, self.n, self.seed, self.first, int(n_steps),
                                     _p(out))
        self.first = 0
        return out


def adjoint_tangent(box, params, gamma, dt, kT, mass, n_steps, sample_every, r_min, r_max,
                    n_bins, sigma, pos0, vel0, noise, g_target):
    """(loss, g_mean, grad[6]) of the differentiable trajectory by FP64
    forward-mode tangents (psim_tangent.c); params: an object with the fields
    of psim_adjoint_params; noise: n_steps*n*6 draws in the injected layout."""
    n = len(pos0) // 3
    p = AdjParams(**{k: getattr(params, k) for k, _ in AdjParams._fields_})
    c = vgb_coeffs(gamma, dt, kT)
    g = np.empty(n_bins)
    grad = np.empty(6)
    loss = np.zeros(1)
    f = lambda a: None if a is None else np.ascontiguousarray(a, np.float64)
    rc = lib().oracle_adjoint_tangent(n, float(box), C.byref(p), C.byref(c), dt, mass, n_steps,
                                      sample_every, r_min, r_max, n_bins, sigma, _p(f(pos0)),
                                      _p(f(vel0)), _p(f(noise)), _p(f(g_target)), _p(loss),
                                      _p(g), _p(grad))
    assert rc == 0, rc
    return float(loss[0]), g, grad
