"""Seeded initial states (host-side set-up, not on the hot path).

The reference's own initialiser (ClusteredCore/src/system/systemInit.cpp:31-267:
uniform mt19937 placement, an O(N^2) overlap fix, Maxwell velocities) cannot
build the dense or large systems, so states are made here: random sequential
addition (RSA), FCC lattices, and Maxwell-Boltzmann velocities normalised per
axis like maxwellVelocityInit (systemInit.cpp:162-267).
"""
import math

import numpy as np


def box_for_phi(n, radius, phi):
    """Edge of the cubic box holding n spheres of ``radius`` at volume fraction phi."""
    return (n * (4.0 / 3.0) * math.pi * radius ** 3 / phi) ** (1.0 / 3.0)


def reference_box(n, radius, conc, scale):
    """The reference's integer box quantisation (system.cpp:57-64): returns
    (boxSize, cellSize, actual concentration)."""
    vp = n * (4.0 / 3.0) * math.atan(1.0) * 4.0 * radius ** 3
    box = int(math.pow(vp / conc, 1.0 / 3.0))
    cell = box // scale
    box = cell * scale
    return box, cell, vp / float(box) ** 3


def rsa_native(n, box, min_sep=1.0, seed=90210, max_trials=0, device=None):
    """Random sequential addition in the native library (O(1) per trial): the
    same construction as rsa() with its own random stream.  device: a GPU
    that evaluates the trials in parallel chunks (the same result); None
    picks GPU 0 for n >= 2^17 when one is present, else the host."""
    import proteinsim2015_gb300 as psim
    out = np.empty(3 * int(n))
    if device is None and int(n) >= (1 << 17) and psim.device_count() > 0:
        device = 0
    if device is not None:
        rc = psim.lib().psim_init_rsa_device(int(n), float(box), float(min_sep),
                                             int(seed) & (2 ** 64 - 1), int(max_trials),
                                             out.ctypes.data, int(device))
    else:
        rc = psim.lib().psim_init_rsa(int(n), float(box), float(min_sep),
                                      int(seed) & (2 ** 64 - 1), int(max_trials), out.ctypes.data)
    if rc != 0:
        raise psim.PsimError(rc, psim.lib().psim_last_error_string().decode())
    return out.reshape(-1, 3)


def rsa(n, box, min_sep=1.0, seed=90210, max_tries=200):
    """Random sequential addition of n points in a periodic cube with minimum
    separation ``min_sep`` (a cell grid keeps each trial O(1))."""
    rng = np.random.default_rng(seed)
    ncell = max(1, int(box // min_sep))
    cs = box / ncell
    grid = {}
    pos = np.empty((n, 3))
    sep2 = min_sep * min_sep
    for i in range(n):
        for _ in range(max_tries * 50):
            p = rng.random(3) * box
            c = np.floor(p / cs).astype(int) % ncell
            ok = True
            for dx in (-1, 0, 1):
                for dy in (-1, 0, 1):
                    for dz in (-1, 0, 1):
                        key = ((c[0] + dx) % ncell, (c[1] + dy) % ncell, (c[2] + dz) % ncell)
                        for j in grid.get(key, ()):
                            d = pos[j] - p
                            d -= box * np.round(d / box)
                            if d @ d < sep2:
                                ok = False
                                break
                        if not ok:
                            break
                    if not ok:
                        break
                if not ok:
                    break
            if ok:
                pos[i] = p
                grid.setdefault(tuple(c), []).append(i)
                break
        else:
            raise RuntimeError("RSA could not place particle %d" % i)
    return pos


def fcc(cells, lattice):
    """FCC lattice of 4*cells^3 points with cubic cell edge ``lattice``."""
    base = np.array([[0, 0, 0], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]])
    g = np.stack(np.meshgrid(np.arange(cells), np.arange(cells), np.arange(cells),
                             indexing="ij"), -1).reshape(-1, 3)
    pts = (g[:, None, :] + base[None, :, :]).reshape(-1, 3) + 0.25
    return pts * lattice


def maxwell(n, kT, seed=90210, mass=1.0):
    """Maxwell-Boltzmann velocities, each axis shifted to zero mean and scaled
    to variance kT/m as maxwellVelocityInit does per axis."""
    rng = np.random.default_rng(seed + 1)
    v = rng.standard_normal((n, 3))
    if n > 1:
        v -= v.mean(0)
        v *= math.sqrt(kT / mass) / v.std(0)
    return v
