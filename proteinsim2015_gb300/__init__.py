"""GB300-native ProteinSim2015 Langevin step.

The hot path of the reference's ``system::run`` -- the hashed cell-list
rebuild, pair forces through the IForce plugins and the van Gunsteren-
Berendsen integrator -- runs as hand-written sm_103a CUDA kernels in
``libpsim_gb300.so``; this module is a thin ctypes binding of its C ABI
(``include/psim_gb300.h``) with the reference's names:

    Config                  settings.cfg reader          (config.h)
    load_force / load_plugin "./<force>.so" + getForce   (runSim.cpp:29-79)
    cells_build             hash/sort/clear/reorder      (systemHandling.cpp:33-85)
    force_evaluate          defaultForceManager::getAcceleration
    vgb_coefficients        brownianIntegrator set-up
    Integrator.next_system  brownianIntegrator::nextSystem
    System                  device-resident system::run loop

There is no CPU fallback: importing works anywhere, but every compute call
needs the native library and a CUDA device and raises ``PsimError``
otherwise.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libpsim_gb300.so")
PLUGIN_DIR = os.path.join(HERE, "plugins")
# PSIM_FORCE_ABI of include/psim_gb300.h: the device entry a plugin exports
FORCE_ABI = 2

OK = 0
ERR_LOAD = 100
ERR_INIT = 7701
ERR_CELL_BOUNDS = 7702
ERR_PARTICLE_BOUNDS = 7703
ERR_OVERLAP = 7704
ERR_NAN_FORCE = 7705
ERR_INPUT = 7706
ERR_CUDA = 7790
ERR_NO_DEVICE = 7791

FORCE_AO, FORCE_LJ, FORCE_CALIBRATION, FORCE_AO_YUKAWA, FORCE_PLUGIN = 1, 2, 3, 4, 5
PRECISION_FP64, PRECISION_MIXED = 0, 1
NOISE_PHILOX, NOISE_INJECTED = 0, 1

KIND_NAMES = {FORCE_AO: "AO", FORCE_LJ: "LJ", FORCE_CALIBRATION: "CAL", FORCE_AO_YUKAWA: "AO_YUK",
              FORCE_PLUGIN: "PLUGIN"}


class PsimError(RuntimeError):
    def __init__(self, code, msg=""):
        super().__init__("psim error %d: %s" % (code, msg))
        self.code = code


class ForceParams(C.Structure):
    _fields_ = [("kind", C.c_int32), ("lj_num", C.c_int32), ("kT", C.c_double),
                ("cutoff", C.c_double), ("well_depth", C.c_double),
                ("yukawa_strength", C.c_double), ("debye_length", C.c_double),
                ("cutoff2", C.c_double), ("well_depth2", C.c_double),
                ("user", C.c_double * 8)]

    def as_dict(self):
        d = {k: getattr(self, k) for k, _ in self._fields_}
        d["kind"] = KIND_NAMES[self.kind]
        d["user"] = list(self.user)
        return d

    def max_cutoff(self):
        return max(self.cutoff, self.cutoff2) if self.kind == FORCE_AO_YUKAWA else self.cutoff


class Geometry(C.Structure):
    _fields_ = [("n_particles", C.c_int32), ("cell_scale", C.c_int32),
                ("box_size", C.c_double), ("cell_size", C.c_double)]


class VgbCoeffs(C.Structure):
    _fields_ = [(k, C.c_double) for k in (
        "y", "coeff0", "coeff1", "coeff2", "coeff3", "sig1", "sig2", "corr", "dev",
        "goy2", "goy3", "hn", "gn")]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class IntegratorConfig(C.Structure):
    _fields_ = [("gamma", C.c_double), ("dt", C.c_double), ("kT", C.c_double),
                ("vel_freq", C.c_int32), ("seed", C.c_int32)]


class SystemConfig(C.Structure):
    _fields_ = [("geom", Geometry), ("integ", IntegratorConfig), ("force", ForceParams),
                ("precision", C.c_int32), ("noise_mode", C.c_int32), ("device", C.c_int32),
                ("skin", C.c_double), ("force_launch", C.c_void_p)]


class Replica(C.Structure):
    _fields_ = [("geom", Geometry), ("force", ForceParams), ("seed", C.c_int32)]


_lib = None


def lib():
    """The native library; raises PsimError when it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise PsimError(ERR_LOAD, "%s is missing: run __graft_entry__.build()" % LIB_PATH)
        L = C.CDLL(LIB_PATH)
        P = C.c_void_p
        sigs = {
            "psim_abi_version": ([], C.c_int),
            "psim_last_error_string": ([], C.c_char_p),
            "psim_device_count": ([], C.c_int),
            "psim_force_params_from_settings": ([C.c_char_p, C.c_char_p, C.POINTER(ForceParams)], C.c_int),
            "psim_ao_coefficients": ([C.c_double] * 3 + [C.POINTER(C.c_double)] * 2, C.c_int),
            "psim_cells_build": ([C.POINTER(Geometry), P, P, P, P, P], C.c_int),
            "psim_cells_build_noalloc": ([C.POINTER(Geometry), P, P, P, P, P, P], C.c_int),
            "psim_force_evaluate": ([C.POINTER(ForceParams), C.POINTER(Geometry), C.c_int32, P, P, P, P], C.c_int),
            "psim_force_evaluate_plugin": ([P, C.POINTER(ForceParams), C.POINTER(Geometry), C.c_int32, P, P, P, P], C.c_int),
            "psim_force_set_list_skin": ([C.c_double], C.c_int),
            "psim_force_list_stats": ([C.POINTER(C.c_int64), C.POINTER(C.c_int64)], C.c_int),
            "psim_vgb_coefficients": ([C.c_double] * 3 + [C.POINTER(VgbCoeffs)], C.c_int),
            "psim_integrator_create": ([C.POINTER(IntegratorConfig), C.c_int32], P),
            "psim_integrator_destroy": ([P], None),
            "psim_integrator_next_system": ([P, C.c_double, C.c_double, C.c_int32] + [P] * 8, C.c_int),
            "psim_init_rsa": ([C.c_int32, C.c_double, C.c_double, C.c_uint64, C.c_int64, P],
                              C.c_int),
            "psim_init_rsa_device": ([C.c_int32, C.c_double, C.c_double, C.c_uint64, C.c_int64,
                                      P, C.c_int32], C.c_int),
            "psim_system_create": ([C.POINTER(SystemConfig)], P),
            "psim_batch_create": ([C.POINTER(Replica), C.c_int32, C.POINTER(IntegratorConfig),
                                   C.c_int32, C.c_int32, C.c_int32], P),
            "psim_batch_create_list": ([C.POINTER(Replica), C.c_int32, C.POINTER(IntegratorConfig),
                                        C.c_int32, C.c_int32, C.c_int32, C.c_double], P),
            "psim_system_destroy": ([P], None),
            "psim_system_upload": ([P] * 8, C.c_int),
            "psim_system_set_noise": ([P, P, C.c_int32, C.c_int32], C.c_int),
            "psim_system_step": ([P, C.c_int32], C.c_int),
            "psim_system_step_async": ([P, C.c_int32], C.c_int),
            "psim_system_sync": ([P], C.c_int),
            "psim_system_download": ([P] * 6, C.c_int),
            "psim_system_download_cells": ([P] * 4, C.c_int),
            "psim_system_snapshot_async": ([P, P], C.c_int),
            "psim_system_snapshot_wait": ([P], C.c_int),
            "psim_system_get_step": ([P, C.POINTER(C.c_int64), C.POINTER(C.c_int32)], C.c_int),
            "psim_system_stream": ([P], P),
            "psim_system_list_builds": ([P, C.POINTER(C.c_int32)], C.c_int),
            "psim_system_temperature": ([P, C.POINTER(C.c_double)], C.c_int),
            "psim_system_mean_displacement": ([P, C.POINTER(C.c_double)], C.c_int),
            "psim_system_potential": ([P, C.POINTER(C.c_double)], C.c_int),
            "psim_system_track_start": ([P], C.c_int),
            "psim_system_tracked_displacement": ([P, C.POINTER(C.c_double)], C.c_int),
            "psim_system_interactions": ([P, C.c_double, P, C.POINTER(C.c_int64)], C.c_int),
            "psim_philox_noise": ([C.c_uint32, C.c_int32, C.c_int64, C.c_int32, P, C.c_int32], C.c_int),
            "psim_system_set_list_lanes": ([P, C.c_int32], C.c_int),
            "psim_system_energy": ([P, C.POINTER(C.c_double), C.POINTER(C.c_double)], C.c_int),
            "psim_system_rdf": ([P, C.c_double, C.c_double, C.c_int32, P], C.c_int),
            "psim_system_clusters": ([P, C.c_double, C.c_int32, P, C.POINTER(C.c_int32),
                                      C.POINTER(C.c_int32)], C.c_int),
            "psim_system_forces": ([P, P], C.c_int),
            "psim_system_profile": ([P, C.c_int32, P], C.c_int),
            "psim_system_launches_per_step": ([P], C.c_int),
            "psim_system_launches_per_rebuild": ([P], C.c_int),
            "psim_system_cell_occupancy": ([P, C.POINTER(C.c_int32), C.POINTER(C.c_double)], C.c_int),
            "psim_system_time_steps": ([P, C.c_int32, C.POINTER(C.c_double)], C.c_int),
            "psim_system_pair_count": ([P, C.c_double, C.POINTER(C.c_double)], C.c_int),
            "psim_measure_fp32_peak": ([C.c_int32, C.POINTER(C.c_double)], C.c_int),
            "psim_measure_host_link": ([C.c_int32] + [C.POINTER(C.c_double)] * 3, C.c_int),
        }
        for name, (args, res) in sigs.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        _lib = L
    return _lib


def _check(rc):
    if rc != OK:
        raise PsimError(rc, lib().psim_last_error_string().decode(errors="replace"))


def _raise_last(code):
    msg = lib().psim_last_error_string().decode(errors="replace")
    if "no CUDA device" in msg:
        code = ERR_NO_DEVICE
    raise PsimError(code, msg)


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _f64(a, n=None):
    a = np.ascontiguousarray(a, dtype=np.float64).reshape(-1)
    if n is not None and a.size != n:
        raise ValueError("expected %d values, got %d" % (n, a.size))
    return a


def device_count():
    return lib().psim_device_count()


def philox_noise(seed, n, first_step, n_steps, device=0):
    """The Philox Gaussians a system or the adjoint draws for particles
    0..n-1 at steps first_step .. first_step + n_steps - 1, in the injected
    layout (n_steps * n * 6), computed on the GPU: a CPU checker replays a
    Philox run with them."""
    out = np.empty(int(n_steps) * int(n) * 6)
    _check(lib().psim_philox_noise(int(seed) & 0xffffffff, int(n), int(first_step), int(n_steps),
                                   _p(out), int(device)))
    return out


def measure_host_link(device=0):
    """Measured host-link bandwidth (GB/s) of the device with SM loads and
    stores on pinned host memory: {"read", "write", "both"}."""
    r, w, b = C.c_double(), C.c_double(), C.c_double()
    _check(lib().psim_measure_host_link(device, C.byref(r), C.byref(w), C.byref(b)))
    return {"read": r.value, "write": w.value, "both": b.value}


def measure_fp32_peak(device=0):
    """Measured FP32 FMA throughput (TFLOP/s) of the device."""
    v = C.c_double()
    _check(lib().psim_measure_fp32_peak(device, C.byref(v)))
    return v.value


# ---------------------------------------------------------------- settings

class Config:
    """settings.cfg: ``key = value`` lines, '#' in column 0 is a comment
    (ClusteredCore/src/utilities/config.cpp:27-56)."""

    def __init__(self, text="", path=None):
        if path is not None:
            with open(path) as fh:
                text = fh.read()
        self.text = text
        self.options = {}
        for line in text.splitlines():
            if not line or line[0] == "#":
                continue
            key, _, val = line.partition("=")
            self.options[key.strip()] = val.strip()

    @staticmethod
    def _lead(v, conv):
        import re
        m = re.match(r"\s*[-+]?(\d+\.?\d*([eE][-+]?\d+)?|\.\d+([eE][-+]?\d+)?)", v)
        if not m:
            raise ValueError("not a number: %r" % v)
        return conv(float(m.group(0))) if conv is int else conv(m.group(0))

    def get(self, key, default):
        if key not in self.options:
            return default
        v = self.options[key]
        if isinstance(default, bool):
            return bool(int(self._lead(v, int)))
        if isinstance(default, int):
            return int(self._lead(v, float))
        if isinstance(default, float):
            return self._lead(v, float)
        return v


def system_constants(cfg):
    """system::setSystemConstants (system.cpp:28-65): the run constants of a
    settings.cfg (a Config).  The box holds nParticles spheres of ``radius``
    at volume fraction ``conc``, cut to a whole number of integer cells:
    L = int(cbrt(vP / conc)), cellSize = L // scale, L = cellSize * scale; the
    concentration is that of the quantised box.  A ``boxSize`` key (never read
    by the reference) gives a real-valued box cut into ``scale`` cells.
    Returns (state dict, Geometry)."""
    import math
    n = cfg.get("nParticles", 1000)
    conc = cfg.get("conc", 0.01)
    scale = cfg.get("scale", 4)
    r = cfg.get("radius", 0.5)
    vp = n * (4.0 / 3.0) * math.atan(1.0) * 4.0 * r * r * r
    if "boxSize" in cfg.options:
        box = cfg.get("boxSize", 0.0)
        cell = box / scale
        st = {"boxSize": int(box), "cellSize": int(cell), "concentration": vp / box ** 3}
    else:
        ibox = int(np.cbrt(vp / conc))      # libm cbrt, truncated as the (int) cast
        cell_i = ibox // scale if scale else 0
        box = float(cell_i * scale)
        cell = float(cell_i)
        st = {"boxSize": cell_i * scale, "cellSize": cell_i,
              "concentration": vp / math.pow(box, 3.0)}
    dt = cfg.get("timeStep", 0.001)
    st.update(nParticles=n, cellScale=scale, dTime=dt, seed=cfg.get("seed", 90210),
              temp=cfg.get("kT", 1.0), outputFreq=cfg.get("outputFreq", int(1.0 / dt)),
              radius=r, mass=cfg.get("mass", 1.0))
    return st, geometry(n, box, cell, scale)


def force_params_from_settings(plugin, text):
    p = ForceParams()
    _check(lib().psim_force_params_from_settings(plugin.encode(), text.encode(), C.byref(p)))
    return p


def load_force(cfg, plugin_dir=PLUGIN_DIR):
    """runSim.cpp:29-79: open ``<plugin_dir>/<force>.so`` named by the
    ``force`` key and take the parameters its factory builds from the same
    settings (the plugin itself: load_plugin)."""
    return load_plugin(cfg, plugin_dir).params


class ForcePlugin:
    """A force plugin shared object: the reference factory getForce(config*)
    plus the GB300 device entry psim_force_launch, whose force passes run the
    plugin's own __device__ pair functor.  ``params`` are the parameters its
    factory builds from the settings text; System and force_evaluate take
    the plugin in place of a ForceParams and run it through its entry."""

    def __init__(self, path, settings_text=""):
        if not os.path.exists(path):
            raise PsimError(ERR_LOAD, "cannot load force library %s" % path)
        self.path = path
        self.lib = C.CDLL(path)
        for sym in ("getForce", "psim_plugin_abi", "psim_plugin_params", "psim_force_launch"):
            if not hasattr(self.lib, sym):
                raise PsimError(ERR_LOAD, "could not find symbol %s in %s" % (sym, path))
        if self.lib.psim_plugin_abi() != FORCE_ABI:
            raise PsimError(ERR_LOAD, "%s was built for another device-entry ABI" % path)
        fn = self.lib.psim_plugin_params
        fn.argtypes = [C.c_char_p, C.POINTER(ForceParams)]
        fn.restype = C.c_int
        self.params = ForceParams()
        _check(fn(settings_text.encode(), C.byref(self.params)))
        self.launch = C.cast(self.lib.psim_force_launch, C.c_void_p).value

    def as_dict(self):
        return self.params.as_dict()

    def max_cutoff(self):
        return self.params.max_cutoff()


def load_plugin(cfg, plugin_dir=PLUGIN_DIR):
    """runSim.cpp:29-79: the plugin ``<plugin_dir>/<force>.so`` named by the
    ``force`` key, with the parameters its factory builds from cfg."""
    return ForcePlugin(os.path.join(plugin_dir, cfg.get("force", "") + ".so"), cfg.text)


def _force_of(force):
    """(parameters, device entry or None) of a ForceParams or ForcePlugin."""
    if isinstance(force, ForcePlugin):
        return force.params, force.launch
    return force, None


def make_force(kind, cutoff, kT=1.0, well_depth=0.0, yukawa_strength=0.0, debye_length=0.5,
               lj_num=18, cutoff2=0.0, well_depth2=0.0):
    kinds = {"AO": FORCE_AO, "LJ": FORCE_LJ, "CAL": FORCE_CALIBRATION, "AO_YUK": FORCE_AO_YUKAWA}
    return ForceParams(kind=kinds.get(kind, kind), lj_num=lj_num, kT=kT, cutoff=cutoff,
                       well_depth=well_depth, yukawa_strength=yukawa_strength,
                       debye_length=debye_length, cutoff2=cutoff2, well_depth2=well_depth2)


def geometry(n, box, cell_size, scale):
    return Geometry(n_particles=int(n), cell_scale=int(scale), box_size=float(box),
                    cell_size=float(cell_size))


def ao_coefficients(kT, well_depth, cutoff):
    c1, c2 = C.c_double(), C.c_double()
    _check(lib().psim_ao_coefficients(kT, well_depth, cutoff, C.byref(c1), C.byref(c2)))
    return c1.value, c2.value


# ---------------------------------------------------------------- drop-ins

def _out(arr, dtype, size):
    """A caller's output array (which the device may write in place), checked,
    or a new one."""
    if arr is None:
        return np.empty(size, dtype)
    if (arr.dtype != dtype or not arr.flags.c_contiguous or not arr.flags.writeable
            or arr.size != size):
        raise PsimError(ERR_INPUT, "output array must be writeable contiguous %s[%d]"
                        % (np.dtype(dtype), size))
    return arr.reshape(-1)


def cells_build(geom, pos, radius, out=None):
    """hashParticles + sortParticles + clearCells + reorderParticles on the GPU.
    Returns (particle_hash_index[2n] int32, cell_start_end[2 s^3] uint32,
    sorted_particles[4n] float64), written into `out` (the same three arrays)
    when given."""
    n = geom.n_particles
    pos = _f64(pos, 3 * n)
    radius = _f64(radius, n)
    o = out if out is not None else (None, None, None)
    hi = _out(o[0], np.int32, 2 * n)
    cse = _out(o[1], np.uint32, 2 * geom.cell_scale ** 3)
    srt = _out(o[2], np.float64, 4 * n)
    _check(lib().psim_cells_build(C.byref(geom), _p(pos), _p(radius), _p(hi), _p(cse), _p(srt)))
    return hi, cse, srt


def force_evaluate(params, geom, sorted_particles, hash_index, cell_start_end,
                   precision=PRECISION_FP64, out=None):
    """defaultForceManager::getAcceleration on the reference's arrays; returns
    particle_force[3n] in original order (written into `out` when given).
    params: a ForceParams, or a ForcePlugin (run through its device entry)."""
    n = geom.n_particles
    srt = _f64(sorted_particles, 4 * n)
    hi = np.ascontiguousarray(hash_index, np.int32).reshape(-1)
    cse = np.ascontiguousarray(cell_start_end, np.uint32).reshape(-1)
    out = _out(out, np.float64, 3 * n)
    fp, launch = _force_of(params)
    if launch:
        _check(lib().psim_force_evaluate_plugin(launch, C.byref(fp), C.byref(geom), precision,
                                                _p(srt), _p(hi), _p(cse), _p(out)))
    else:
        _check(lib().psim_force_evaluate(C.byref(fp), C.byref(geom), precision, _p(srt),
                                         _p(hi), _p(cse), _p(out)))
    return out


def set_force_list_skin(skin=-1.0):
    """The pair-list skin of force_evaluate's mixed precision: the list is kept
    across calls while no particle has moved skin/2 since its build.  < 0:
    automatic (the smaller of 0.4 and cellSize - cutOff, if at least 0.1);
    0 (the library's default): a list of each call's own pairs, built every
    call, so each call stands alone."""
    _check(lib().psim_force_set_list_skin(float(skin)))


def force_list_stats():
    """(mixed-precision force_evaluate calls, pair lists they built)."""
    calls, builds = C.c_int64(0), C.c_int64(0)
    _check(lib().psim_force_list_stats(C.byref(calls), C.byref(builds)))
    return calls.value, builds.value


def vgb_coefficients(gamma, dt, kT):
    c = VgbCoeffs()
    _check(lib().psim_vgb_coefficients(gamma, dt, kT, C.byref(c)))
    return c


class Integrator:
    """brownianIntegrator: noise memory and velocity counter on the device."""

    def __init__(self, n, gamma=0.5, dt=0.001, kT=1.0, vel_freq=1000, seed=90210):
        cfg = IntegratorConfig(gamma=gamma, dt=dt, kT=kT, vel_freq=vel_freq, seed=seed)
        self.n = n
        self._h = lib().psim_integrator_create(C.byref(cfg), n)
        if not self._h:
            _raise_last(ERR_INPUT)

    def next_system(self, current_time, box, pos, pos0, vel, frc, frc0, mass, noise=None,
                    particle_force=None):
        """pushParticleForce (if particle_force is given) + nextSystem; the
        float64 arrays are updated in place."""
        for a in (pos, pos0, vel, frc, frc0):   # updated in place, possibly by the device
            if (a.dtype != np.float64 or not a.flags.c_contiguous or not a.flags.writeable
                    or a.size != 3 * self.n):
                raise PsimError(ERR_INPUT, "state arrays must be writeable contiguous "
                                "float64[%d]" % (3 * self.n))
        mode = NOISE_INJECTED if noise is not None else NOISE_PHILOX
        nz = _f64(noise, 6 * self.n) if noise is not None else None
        pf = _f64(particle_force, 3 * self.n) if particle_force is not None else None
        mass = _f64(mass, self.n)
        _check(lib().psim_integrator_next_system(self._h, current_time, box, mode, _p(nz), _p(pf),
                                                 _p(pos), _p(pos0), _p(vel), _p(frc), _p(frc0),
                                                 _p(mass)))

    def close(self):
        if self._h:
            lib().psim_integrator_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def auto_skin(geom, force, preferred=0.4, smallest=0.1):
    """A pair-list skin the cell size allows: min(preferred, cellSize - cutOff),
    or 0 (no list) when that is below `smallest`."""
    room = geom.cell_size - force.max_cutoff()
    skin = min(preferred, room * (1.0 - 1e-9))
    return skin if skin >= smallest else 0.0


class System:
    """The device-resident hot loop of system::run (system.cpp:187-206)."""

    def __init__(self, geom, force, gamma=1.0, dt=0.001, kT=1.0, vel_freq=1000, seed=90210,
                 precision=PRECISION_MIXED, noise_mode=NOISE_PHILOX, device=0, skin=0.0):
        """force: a ForceParams, or a ForcePlugin whose device entry runs every
        force pass.  skin: Verlet pair-list skin of the mixed form (0: walk the
        27 cells every step; "auto": the largest of 0.4 and cellSize - cutOff
        that the cell size allows, if at least 0.1)."""
        if skin == "auto":
            skin = auto_skin(geom, force) if precision == PRECISION_MIXED else 0.0
        fp, launch = _force_of(force)
        self._plugin = force if launch else None   # keeps the plugin library loaded
        self.cfg = SystemConfig(geom=geom,
                                integ=IntegratorConfig(gamma=gamma, dt=dt, kT=kT,
                                                       vel_freq=vel_freq, seed=seed),
                                force=fp, precision=precision, noise_mode=noise_mode,
                                device=device, skin=float(skin), force_launch=launch)
        self.skin = float(skin)
        self.n = geom.n_particles
        self.ncell = geom.cell_scale ** 3
        self._h = lib().psim_system_create(C.byref(self.cfg))
        if not self._h:
            _raise_last(ERR_INPUT)

    def upload(self, pos, radius, mass=None, vel=None, pos0=None, frc=None, frc0=None):
        n = self.n
        args = [_f64(pos, 3 * n), None if pos0 is None else _f64(pos0, 3 * n),
                None if vel is None else _f64(vel, 3 * n),
                None if frc is None else _f64(frc, 3 * n),
                None if frc0 is None else _f64(frc0, 3 * n), _f64(radius, n),
                None if mass is None else _f64(mass, n)]
        self._keep = args
        _check(lib().psim_system_upload(self._h, *[_p(a) for a in args]))

    def set_noise(self, noise, n_steps, first_step=0):
        nz = _f64(noise, n_steps * self.n * 6)
        _check(lib().psim_system_set_noise(self._h, _p(nz), n_steps, first_step))

    def step(self, n_steps=1):
        _check(lib().psim_system_step(self._h, n_steps))

    def step_async(self, n_steps=1):
        _check(lib().psim_system_step_async(self._h, n_steps))

    def sync(self):
        _check(lib().psim_system_sync(self._h))

    def download(self):
        n = self.n
        out = {k: np.empty(3 * n) for k in ("pos", "pos0", "vel", "frc", "frc0")}
        _check(lib().psim_system_download(self._h, *[_p(out[k]) for k in
                                                     ("pos", "pos0", "vel", "frc", "frc0")]))
        return out

    def download_cells(self):
        hi = np.empty(2 * self.n, np.int32)
        cse = np.empty(2 * self.ncell, np.uint32)
        srt = np.empty(4 * self.n)
        _check(lib().psim_system_download_cells(self._h, _p(hi), _p(cse), _p(srt)))
        return hi, cse, srt

    def snapshot_async(self, host_pos):
        assert host_pos.dtype == np.float64 and host_pos.size == 3 * self.n
        _check(lib().psim_system_snapshot_async(self._h, _p(host_pos)))

    def snapshot_wait(self):
        _check(lib().psim_system_snapshot_wait(self._h))

    def get_step(self):
        s, v = C.c_int64(), C.c_int32()
        _check(lib().psim_system_get_step(self._h, C.byref(s), C.byref(v)))
        return s.value, v.value

    def forces(self):
        """The force on every particle at the current state (3n, original
        order), from the force pass the next step runs."""
        out = np.empty(3 * self.n)
        _check(lib().psim_system_forces(self._h, _p(out)))
        return out

    def _scalar(self, fn):
        v = C.c_double()
        _check(fn(self._h, C.byref(v)))
        return v.value

    def temperature(self):
        """sum v^2 / 3N of the last velocity step (getTemperature)."""
        return self._scalar(lib().psim_system_temperature)

    def mean_displacement(self):
        """mean |x - x0|^2 (meanDisplacement)."""
        return self._scalar(lib().psim_system_mean_displacement)

    def potential(self):
        """<EAP>: calculatePotential averaged over the particles."""
        return self._scalar(lib().psim_system_potential)

    def track_start(self):
        _check(lib().psim_system_track_start(self._h))

    def tracked_displacement(self):
        """mean squared unwrapped displacement since track_start()."""
        return self._scalar(lib().psim_system_tracked_displacement)

    def interactions(self, r_contact=1.2):
        """Coordination numbers (original order) and their sum (updateInteractions)."""
        coor = np.empty(self.n, dtype=np.int32)
        tot = C.c_int64()
        _check(lib().psim_system_interactions(self._h, r_contact, _p(coor), C.byref(tot)))
        return coor, tot.value

    def clusters(self, r_contact=1.2, min_size=4):
        """findClusters + writeClusters: (root of every particle -- the smallest
        original index of its cluster --, the clusters of more than min_size
        particles as sorted index arrays in root order, their integer mean size)."""
        root = np.empty(self.n, dtype=np.int32)
        nc, avg = C.c_int32(), C.c_int32()
        _check(lib().psim_system_clusters(self._h, r_contact, int(min_size), _p(root),
                                          C.byref(nc), C.byref(avg)))
        order = np.argsort(root, kind="stable")
        bounds = np.flatnonzero(np.diff(root[order])) + 1
        groups = [g for g in np.split(order, bounds) if len(g) > min_size]
        assert len(groups) == nc.value
        return root, groups, avg.value

    def rdf(self, r_min, r_max, n_bins):
        g = np.empty(int(n_bins))
        _check(lib().psim_system_rdf(self._h, r_min, r_max, int(n_bins), _p(g)))
        return g

    def energy(self):
        """(potential energy per particle, virial per particle) of the current
        state in FP64: u(r) is the integral of the plugin's force law, zero at
        the cutoff; the virial is sum r_ij . f_ij / N."""
        u, w = C.c_double(), C.c_double()
        _check(lib().psim_system_energy(self._h, C.byref(u), C.byref(w)))
        return u.value, w.value

    def set_list_lanes(self, lanes):
        """Threads per particle (1, 2 or 4) of the pair-list force pass."""
        _check(lib().psim_system_set_list_lanes(self._h, int(lanes)))

    def list_builds(self):
        b = C.c_int32()
        _check(lib().psim_system_list_builds(self._h, C.byref(b)))
        return b.value

    def stream(self):
        return lib().psim_system_stream(self._h)

    def profile(self, n_steps):
        out = np.zeros(4)
        _check(lib().psim_system_profile(self._h, n_steps, _p(out)))
        return {"force_ms": out[0], "integrate_ms": out[1], "rebuild_ms": out[2],
                "total_ms": out[3]}

    def launches_per_step(self):
        return lib().psim_system_launches_per_step(self._h)

    def launches_per_rebuild(self):
        return lib().psim_system_launches_per_rebuild(self._h)

    def cell_occupancy(self):
        m, a = C.c_int32(), C.c_double()
        _check(lib().psim_system_cell_occupancy(self._h, C.byref(m), C.byref(a)))
        return m.value, a.value

    def time_steps(self, n_steps):
        """Device time (ms) of n_steps, CUDA events on the step stream."""
        ms = C.c_double()
        _check(lib().psim_system_time_steps(self._h, n_steps, C.byref(ms)))
        return ms.value

    def pair_count(self, cutoff):
        v = C.c_double()
        _check(lib().psim_system_pair_count(self._h, cutoff, C.byref(v)))
        return v.value

    def close(self):
        if getattr(self, "_h", None):
            lib().psim_system_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Batch(System):
    """Independent replicas stepped together, one launch per phase.  Each
    replica is (geometry, force params, seed); arrays are the replicas'
    arrays concatenated in replica order.  Every System method applies.  A
    skin > 0 gives the mixed form a pair list (every replica's cellSize >=
    its cutOff + skin)."""

    def __init__(self, replicas, gamma=1.0, dt=0.001, kT=1.0, vel_freq=1000,
                 precision=PRECISION_MIXED, noise_mode=NOISE_PHILOX, device=0, skin=0.0):
        arr = (Replica * len(replicas))()
        for k, (g, f, seed) in enumerate(replicas):
            arr[k] = Replica(geom=g, force=f, seed=int(seed))
        self._reps = arr
        self.integ = IntegratorConfig(gamma=gamma, dt=dt, kT=kT, vel_freq=vel_freq, seed=0)
        self.sizes = [g.n_particles for g, _, _ in replicas]
        self.offsets = np.concatenate([[0], np.cumsum(self.sizes)]).astype(int)
        self.n = int(self.offsets[-1])
        self.ncell = sum(g.cell_scale ** 3 for g, _, _ in replicas)
        self.skin = float(skin)
        self._h = lib().psim_batch_create_list(arr, len(replicas), C.byref(self.integ), precision,
                                               noise_mode, device, self.skin)
        if not self._h:
            _raise_last(ERR_INPUT)

    def split(self, a, width=3):
        """A concatenated per-particle array cut into the replicas' arrays."""
        return [a[width * self.offsets[k]:width * self.offsets[k + 1]]
                for k in range(len(self.sizes))]
