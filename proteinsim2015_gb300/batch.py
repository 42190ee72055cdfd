"""Batches of independent AO replicas: the seeded replica set of the
batched-replica workload, their initial states, and the cell-size autotuner.

A replica is (geometry, force parameters, Philox seed) as ``Batch`` takes it.
The workload draws, per replica, N ~ U[500, 20000], a volume fraction
phi ~ U[0.05, 0.35], a contact attraction A ~ U[1, 6] kT and a polymer/colloid
size ratio q ~ U[0.05, 0.2]; the AOPotential plugin then has cutOff = 1 + q and
wellDepth = A q / (1.5 + q), so that U(1) = -kT wellDepth (rc + 1/2)/(rc - 1)
= -A kT (AOPotential.cpp:50-55).  States are seeded random sequential addition
with minimum separation 1 (diameter 1) and Maxwell-Boltzmann velocities.

The autotuner picks each replica's cell size: the grid is the finest one with
cellSize >= f * cutOff, and f is chosen per size bucket (particles per cell of
the finest grid) from a few candidates by timing sub-batches of that bucket's
replicas on the GPU.
"""
import math
import os
from concurrent.futures import ThreadPoolExecutor

import numpy as np

from . import init as _init


def ao_params(psim, contact_kT, q, kT=1.0):
    rc = 1.0 + q
    return psim.make_force("AO", rc, kT=kT, well_depth=contact_kT * q / (1.5 + q))


def geometry_for(psim, n, box, cutoff, factor=1.0, skin=0.0):
    """The finest grid with cellSize >= factor * cutoff and >= cutoff + skin
    (at least 3 cells a side)."""
    scale = max(3, int(math.floor(box / max(factor * cutoff, cutoff + skin))))
    return psim.geometry(n, box, box / scale, scale)


def c2_draws(n_reps=512, seed=2015):
    """The replica parameters of the batched workload: a list of dicts."""
    rng = np.random.default_rng(seed)
    out = []
    for r in range(n_reps):
        n = int(rng.integers(500, 20001))
        phi = float(rng.uniform(0.05, 0.35))
        a = float(rng.uniform(1.0, 6.0))
        q = float(rng.uniform(0.05, 0.2))
        box = (n * math.pi / 6.0 / phi) ** (1.0 / 3.0)
        out.append(dict(n=n, phi=phi, contact_kT=a, q=q, box=box, seed=int(seed * 1000 + r)))
    return out


def replicas(psim, draws, factors=None, skin=0.0):
    """(geometry, force, seed) per draw; factors: cell-size factor per replica;
    skin: the pair-list skin the grids must allow."""
    reps = []
    for k, d in enumerate(draws):
        f = ao_params(psim, d["contact_kT"], d["q"])
        fac = 1.0 if factors is None else factors[k]
        reps.append((geometry_for(psim, d["n"], d["box"], f.cutoff, fac, skin), f, d["seed"]))
    return reps


def states(draws, threads=None):
    """Seeded RSA positions (min separation 1) and Maxwell velocities at kT = 1,
    concatenated in replica order; the replicas are set up in parallel."""
    threads = threads or os.cpu_count() or 1

    def one(d):
        p = _init.rsa_native(d["n"], d["box"], 1.0, seed=d["seed"])
        v = _init.maxwell(d["n"], 1.0, seed=d["seed"] + 1)
        return p.reshape(-1), np.asarray(v).reshape(-1)

    with ThreadPoolExecutor(max_workers=threads) as ex:
        res = list(ex.map(one, draws))
    return np.concatenate([r[0] for r in res]), np.concatenate([r[1] for r in res])


def size_bucket(d, cutoff, edges=(0.5, 1.0, 2.0)):
    """Bucket of a replica by particles per cell of its finest grid."""
    scale = max(3, int(math.floor(d["box"] / cutoff)))
    occ = d["n"] / float(scale ** 3)
    return int(np.searchsorted(edges, occ))


def autotune(psim, draws, candidates=(1.0, 1.25, 1.5, 2.0), per_bucket=24, steps=40,
             dt=0.001, device=0, seed=7):
    """Cell-size factor per size bucket, from timed sub-batches (the cell
    walk; the pair-list pass's threads per particle: tune_lanes).

    For each bucket, up to ``per_bucket`` of its replicas (drawn with ``seed``)
    are batched at every candidate factor, warmed up, and timed over ``steps``
    steps; the factor with the highest particle-steps/s wins.  Returns
    (factor per replica, {bucket: (factor, {factor: rate})})."""
    rng = np.random.default_rng(seed)
    buckets = {}
    for k, d in enumerate(draws):
        b = size_bucket(d, 1.0 + d["q"])
        buckets.setdefault(b, []).append(k)
    report, best = {}, {}
    for b, members in sorted(buckets.items()):
        pick = sorted(rng.choice(members, size=min(per_bucket, len(members)), replace=False))
        sub = [draws[k] for k in pick]
        pos, vel = states(sub)
        rates = {}
        for fac in candidates:
            reps = replicas(psim, sub, [fac] * len(sub))
            bt = psim.Batch(reps, gamma=1.0, dt=dt, kT=1.0, vel_freq=0,
                            precision=psim.PRECISION_MIXED, device=device)
            bt.upload(pos, np.full(bt.n, 0.5), vel=vel)
            bt.step(3)
            ms = bt.time_steps(steps)
            rates[fac] = bt.n * steps / (ms * 1e-3)
            bt.close()
        best[b] = max(rates, key=rates.get)
        report[b] = (best[b], rates)
    factors = [best[size_bucket(d, 1.0 + d["q"])] for d in draws]
    return factors, report


def tune_lanes(system, candidates=(1, 2, 4), steps=100, warmup=5):
    """Threads per particle of a system's pair-list force pass (a System or
    Batch with a skin): each candidate is timed over ``steps`` steps of the
    live system (after ``warmup`` steps that capture its graphs), the fastest
    is kept set.  The steps advance the state, as warm-up steps do.  Returns
    (lanes, {lanes: particle-steps/s})."""
    rates = {}
    for lanes in candidates:
        system.set_list_lanes(lanes)
        system.step(warmup)
        ms = system.time_steps(steps)
        rates[lanes] = system.n * steps / (ms * 1e-3)
    best = max(rates, key=rates.get)
    system.set_list_lanes(best)
    return best, rates
