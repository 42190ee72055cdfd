"""Host side of the batched-replica workload: the seeded draws, the replica
geometries and the autotuner's size buckets (no GPU)."""
import math

import numpy as np

import proteinsim2015_gb300 as psim
from proteinsim2015_gb300 import batch


def test_c2_draws_are_seeded_and_in_range():
    a, b = batch.c2_draws(64, seed=5), batch.c2_draws(64, seed=5)
    assert a == b
    assert a != batch.c2_draws(64, seed=6)
    for d in a:
        assert 500 <= d["n"] <= 20000
        assert 0.05 <= d["phi"] <= 0.35 and 1.0 <= d["contact_kT"] <= 6.0
        assert 0.05 <= d["q"] <= 0.2
        assert math.isclose(d["n"] * math.pi / 6 / d["box"] ** 3, d["phi"], rel_tol=1e-12)


def test_replica_grids_respect_the_cutoff_and_contact_attraction():
    draws = batch.c2_draws(32, seed=9)
    for fac in (1.0, 1.5):
        for (g, f, seed), d in zip(batch.replicas(psim, draws, [fac] * 32), draws):
            assert g.cell_scale >= 3
            assert g.cell_size >= fac * f.cutoff - 1e-12 or g.cell_scale == 3
            assert math.isclose(g.cell_size * g.cell_scale, d["box"], rel_tol=1e-12)
            # U(1) = -kT wd (rc + 1/2) / (rc - 1) is the drawn contact attraction
            u1 = -f.kT * f.well_depth * (f.cutoff + 0.5) / (f.cutoff - 1.0)
            assert math.isclose(u1, -d["contact_kT"], rel_tol=1e-12)
            assert seed == d["seed"]


def test_size_buckets_follow_cell_occupancy():
    d = dict(n=1000, box=20.0)
    occ = 1000 / (int(20.0 // 1.1) ** 3)
    assert batch.size_bucket(d, 1.1) == int(np.searchsorted((0.5, 1.0, 2.0), occ))
