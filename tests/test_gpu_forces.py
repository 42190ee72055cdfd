"""Force pass on the GPU: plain FP64 form against the reference within 1e-12
(per particle, relative to sum_j |f_ij|); mixed form within 1e-5 (norm)."""
import numpy as np
import pytest

from conftest import settings_of
from gpu_helpers import (FORCE_TOL_FP64, FORCE_TOL_MIXED, lattice_state, oracle_force,
                         rel_norm, rel_per_particle, rsa_state)
from oracle import port

pytestmark = pytest.mark.gpu
PLUGIN_OF = {"AO": "AOPotential", "AOq": "AOPotential", "LJ6": "LennardJones",
             "LJ18": "LennardJones", "YUK": "LennardJones", "CAL": "Calibration"}


def params_from_golden(psim, golden, key):
    s = settings_of(golden, "forceA_%s_settings" % key)
    text = "".join("%s = %r\n" % kv for kv in s.items())
    return psim.force_params_from_settings(PLUGIN_OF[key], text)


@pytest.mark.parametrize("key", sorted(PLUGIN_OF))
@pytest.mark.parametrize("precision", [0, 1])
def test_forces_match_reference_golden(psim, golden, key, precision, force_pass):
    n, box, cs, scale = (int(v) for v in golden["cellsA_geom"])
    g = psim.geometry(n, box, cs, scale)
    p = params_from_golden(psim, golden, key)
    f = psim.force_evaluate(p, g, golden["cellsA_sorted"], golden["cellsA_hash_index"],
                            golden["cellsA_cse"], precision=precision)
    ref = golden["forceA_%s" % key]
    _, _, _, _, _, scale_ = oracle_force(p.as_dict(), g, golden["cellsA_pos"],
                                         golden["cellsA_radius"])
    if precision == 0:
        assert rel_per_particle(f, ref, scale_) <= FORCE_TOL_FP64
    else:
        assert rel_norm(f, ref) <= FORCE_TOL_MIXED


@pytest.mark.parametrize("precision", [0, 1])
def test_lj_dense_liquid_matches_oracle(psim, precision, force_pass):
    # rho = 0.8 LJ (the 2^20 benchmark's density), a jittered FCC block
    pos, rad, box = lattice_state(8, (4 / 0.8) ** (1 / 3), 0.08, seed=4)
    n = len(rad)
    scale = int(box // 2.5)
    g = psim.geometry(n, box, box / scale, scale)
    p = psim.make_force("LJ", 2.5, kT=1.5, well_depth=1 / 1.5, lj_num=6, yukawa_strength=0.0)
    hi, cse, srt, ref, err, sc = oracle_force(p.as_dict(), g, pos, rad)
    assert err == 0
    f = psim.force_evaluate(p, g, srt, hi, cse, precision=precision)
    if precision == 0:
        assert rel_per_particle(f, ref, sc) <= FORCE_TOL_FP64
    else:
        assert rel_norm(f, ref) <= FORCE_TOL_MIXED


@pytest.mark.parametrize("precision", [0, 1])
def test_ao_yukawa_composite_matches_oracle(psim, precision, force_pass):
    pos, rad = rsa_state(3000, 26.0, seed=9)
    n = len(rad)
    g = psim.geometry(n, 26.0, 26.0 / 8, 8)
    p = psim.make_force("AO_YUK", 1.1, kT=1.0, well_depth=0.1875, cutoff2=3.0, well_depth2=1.0,
                        yukawa_strength=2183.93, debye_length=0.25, lj_num=0)
    hi, cse, srt, ref, err, sc = oracle_force(p.as_dict(), g, pos, rad)
    assert err == 0
    f = psim.force_evaluate(p, g, srt, hi, cse, precision=precision)
    if precision == 0:
        assert rel_per_particle(f, ref, sc) <= FORCE_TOL_FP64
    else:
        assert rel_norm(f, ref) <= FORCE_TOL_MIXED


def test_overlap_is_reported_as_7704(psim):
    g = psim.geometry(2, 12.0, 3.0, 4)
    pos = np.array([1.0, 1.0, 1.0, 1.5, 1.0, 1.0])
    hi, cse, srt = psim.cells_build(g, pos, np.full(2, 0.5))
    for prec in (0, 1):
        with pytest.raises(psim.PsimError) as e:
            psim.force_evaluate(psim.make_force("AO", 1.1, well_depth=1.0), g, srt, hi, cse, prec)
        assert e.value.code == psim.ERR_OVERLAP


def test_empty_and_single_particle(psim):
    g = psim.geometry(1, 12.0, 3.0, 4)
    hi, cse, srt = psim.cells_build(g, np.array([5.0, 5.0, 5.0]), np.full(1, 0.5))
    f = psim.force_evaluate(psim.make_force("AO", 1.1, well_depth=1.0), g, srt, hi, cse)
    assert np.array_equal(f, np.zeros(3))


@pytest.mark.parametrize("precision", [0, 1])
def test_sparse_grid_with_empty_cells(psim, precision, force_pass):
    # 0.5 particles per cell: most rows cross empty cells, whose sentinel
    # start must not break the contiguous row walk
    n, box, scale = 500, 30.0, 10
    pos, rad = rsa_state(n, box, seed=12)
    g = psim.geometry(n, box, box / scale, scale)
    p = psim.make_force("AO", 1.1, kT=1.0, well_depth=2.0)
    hi, cse, srt, ref, err, sc = oracle_force(p.as_dict(), g, pos, rad)
    assert err == 0 and np.sum(cse == 0xFFFFFFFF) > 0
    f = psim.force_evaluate(p, g, srt, hi, cse, precision=precision)
    if precision == 0:
        assert rel_per_particle(f, ref, sc) <= FORCE_TOL_FP64
    else:
        assert rel_norm(f, ref) <= FORCE_TOL_MIXED


def test_malformed_cell_list_is_refused(psim):
    n, box, scale = 300, 12.0, 4
    pos, rad = rsa_state(n, box, seed=13)
    g = psim.geometry(n, box, box / scale, scale)
    hi, cse, srt = psim.cells_build(g, pos, rad)
    p = psim.make_force("AO", 1.1, well_depth=1.0)
    bad_tag = hi.copy()
    bad_tag[1] = n + 5                        # an original index beyond n
    bad_end = cse.copy()
    k = int(np.flatnonzero(cse[0::2] != 0xFFFFFFFF)[0])
    bad_end[2 * k + 1] = n + 100              # a cell range beyond the list
    bad_start = cse.copy()
    nz = np.flatnonzero(cse[0::2] != 0xFFFFFFFF)
    bad_start[2 * nz[3]] += 1                 # a start off the counting-sort layout
    bad_start[2 * nz[3] + 1] += 1
    for h, c in ((bad_tag, cse), (hi, bad_end), (hi, bad_start)):
        with pytest.raises(psim.PsimError) as e:
            psim.force_evaluate(p, g, srt, h, c)
        assert e.value.code == psim.ERR_INPUT


@pytest.mark.parametrize("system", ["lj_dense", "ao_sparse"])
def test_walk_choice_keeps_the_fp64_sums(psim, monkeypatch, system):
    # PSIM_FORCE_WALK picks the mixed form's 27-cell walk (the staged or the
    # direct one: the same pair terms, summed in another cadence, within the
    # mixed tolerance); the FP64 form always takes the staged walk in the
    # reference's order, so its forces do not move by a bit, through the
    # drop-in and a system
    if system == "lj_dense":   # ~32 particles per cell
        pos, rad, box = lattice_state(8, (4 / 0.8) ** (1 / 3), 0.08, seed=52)
        n, scale = len(rad), 4
        p = psim.make_force("LJ", 2.5, kT=1.5, well_depth=1 / 1.5, lj_num=6,
                            yukawa_strength=0.0)
    else:                      # ~0.3 particles per cell
        n, box, scale = 3000, 30.0, 25
        pos, rad = rsa_state(n, box, seed=53)
        p = psim.make_force("AO", 1.1, kT=1.0, well_depth=0.25)
    g = psim.geometry(n, box, box / scale, scale)
    hi, cse, srt = psim.cells_build(g, pos, rad)
    out = {}
    for walk in ("staged", "direct"):
        monkeypatch.setenv("PSIM_FORCE_WALK", walk)
        f64 = psim.force_evaluate(p, g, srt, hi, cse, precision=psim.PRECISION_FP64)
        s = psim.System(g, p, precision=psim.PRECISION_FP64)
        s.upload(pos, rad)
        fs = s.forces()
        s.close()
        s = psim.System(g, p, precision=psim.PRECISION_MIXED)
        s.upload(pos, rad)
        fm = s.forces()
        s.close()
        out[walk] = (f64, fs, fm)
    assert np.array_equal(out["staged"][0], out["direct"][0])
    assert np.array_equal(out["staged"][1], out["direct"][1])
    assert rel_norm(out["direct"][2], out["direct"][1]) < FORCE_TOL_MIXED
    assert rel_norm(out["staged"][2], out["direct"][1]) < FORCE_TOL_MIXED
