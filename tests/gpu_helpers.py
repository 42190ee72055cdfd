"""Shared set-up for the GPU parity tests: seeded states and comparisons."""
import numpy as np

from oracle import port
from proteinsim2015_gb300 import init

FORCE_TOL_FP64 = 1e-12   # per-particle |dF| / sum_j |f_ij| (plain form)
FORCE_TOL_MIXED = 1e-5   # ||dF||_2 / ||F||_2 over all particles (mixed form)
TRAJ_TOL = 1e-9          # positions after 100 steps with identical injected noise


def rsa_state(n, box, seed):
    return init.rsa(n, box, 1.0, seed=seed).reshape(-1), np.full(n, 0.5)


def lattice_state(cells, lattice, jitter, seed):
    p = init.fcc(cells, lattice)
    rng = np.random.default_rng(seed)
    p = p + rng.uniform(-jitter, jitter, p.shape)
    box = cells * lattice
    p = np.mod(p, box)
    return p.reshape(-1), np.full(len(p), 0.5), box


def oracle_force(kind_params, geom, pos, radius):
    g = port.geom(geom.n_particles, geom.box_size, geom.cell_size, geom.cell_scale)
    f = port.force_from_params(kind_params)
    hi, cse, srt = port.build_cells(g, pos, radius)
    out, err = port.forces(g, f, srt, hi, cse)
    scale = port.force_scale(g, f, srt, hi, cse)
    return hi, cse, srt, out, err, scale


def rel_per_particle(a, b, scale):
    d = np.abs(a - b).reshape(-1, 3).max(1)
    s = np.maximum(scale, 1e-300)
    return np.max(np.where(scale > 0, d / s, d))


def rel_norm(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)
