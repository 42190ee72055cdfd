"""psim_force_evaluate's mixed precision keeps its pair list across calls: a
list of the pairs within cutOff + skin, reused while no particle has moved
skin/2 since its build.  Every call's forces are those of its own positions
(against the plain FP64 form on the same cell list), the list is rebuilt when
a particle moves further or another system comes in, and a particle that
wraps around the box between calls keeps its pairs."""
import numpy as np
import pytest

from gpu_helpers import FORCE_TOL_MIXED, lattice_state, rel_norm

pytestmark = pytest.mark.gpu

KT = 1.5


@pytest.fixture
def skin_reset(psim):
    psim.set_force_list_skin(-1.0)
    yield
    psim.set_force_list_skin(0.0)   # the library's default: each call stands alone


def liquid(psim, seed=60):
    # rho ~0.69 LJ (fcc 1.8), 2048 particles in a 14.4 box: 5^3 cells of 2.88,
    # room for a 0.38 skin over cutOff 2.5
    pos, rad, box = lattice_state(8, 1.8, 0.1, seed=seed)
    n = len(rad)
    g = psim.geometry(n, box, box / 5, 5)
    p = psim.make_force("LJ", 2.5, kT=KT, well_depth=1 / KT, lj_num=6, yukawa_strength=0.0)
    return g, p, pos, rad, box


def both(psim, g, p, pos, rad):
    hi, cse, srt = psim.cells_build(g, pos, rad)
    mixed = psim.force_evaluate(p, g, srt, hi, cse, precision=psim.PRECISION_MIXED)
    fp64 = psim.force_evaluate(p, g, srt, hi, cse, precision=psim.PRECISION_FP64)
    return mixed, fp64


def builds(psim):
    return psim.force_list_stats()[1]


def test_kept_list_follows_each_calls_positions(psim, skin_reset):
    g, p, pos, rad, box = liquid(psim)
    rng = np.random.default_rng(61)
    # one particle just inside the low x face, walking out of it: it wraps to
    # the high face on the second call
    pos = pos.copy()
    pos[0] = 0.004
    b0 = builds(psim)
    for k in range(6):
        mixed, fp64 = both(psim, g, p, pos, rad)
        assert rel_norm(mixed, fp64) <= FORCE_TOL_MIXED, k
        # up to 0.01 per axis per call: 0.1 at most after 6 calls, under skin/2
        pos = np.mod(pos + rng.uniform(-0.01, 0.01, pos.shape), box)
        pos[0] = np.mod(0.004 - 0.005 * (k + 1), box)
    assert builds(psim) - b0 == 1
    assert pos[0] > box - 0.03   # it did wrap


def test_kept_list_matches_fresh_lists(psim, skin_reset):
    g, p, pos, rad, box = liquid(psim, seed=62)
    rng = np.random.default_rng(63)
    hi, cse, srt = psim.cells_build(g, pos, rad)
    psim.force_evaluate(p, g, srt, hi, cse, precision=psim.PRECISION_MIXED)
    pos = np.mod(pos + rng.uniform(-0.03, 0.03, pos.shape), box)
    hi, cse, srt = psim.cells_build(g, pos, rad)
    b0 = builds(psim)
    kept = psim.force_evaluate(p, g, srt, hi, cse, precision=psim.PRECISION_MIXED)
    assert builds(psim) == b0
    psim.set_force_list_skin(0.0)
    fresh = psim.force_evaluate(p, g, srt, hi, cse, precision=psim.PRECISION_MIXED)
    assert builds(psim) == b0 + 1
    # the same pair terms summed in another order
    assert rel_norm(kept, fresh) < 1e-6


def test_large_move_rebuilds(psim, skin_reset):
    g, p, pos, rad, box = liquid(psim, seed=64)
    both(psim, g, p, pos, rad)
    b0 = builds(psim)
    pos = pos.copy()
    pos[3 * 17] = np.mod(pos[3 * 17] + 0.25, box)   # more than skin/2 = 0.19
    mixed, fp64 = both(psim, g, p, pos, rad)
    assert builds(psim) == b0 + 1
    assert rel_norm(mixed, fp64) <= FORCE_TOL_MIXED


def test_other_system_rebuilds(psim, skin_reset):
    a = liquid(psim, seed=65)
    b = liquid(psim, seed=66)
    for k in range(4):
        g, p, pos, rad, _ = (a, b)[k % 2]
        b0 = builds(psim)
        mixed, fp64 = both(psim, g, p, pos, rad)
        assert builds(psim) == b0 + 1, k
        assert rel_norm(mixed, fp64) <= FORCE_TOL_MIXED, k


def test_radius_change_is_seen(psim, skin_reset):
    g, p, pos, rad, box = liquid(psim, seed=67)
    both(psim, g, p, pos, rad)
    b0 = builds(psim)
    # one radius for all: compact records, which hold no radius -- a new
    # radius is a new list
    mixed, fp64 = both(psim, g, p, pos, rad * 0.9)
    assert builds(psim) == b0 + 1
    assert rel_norm(mixed, fp64) <= FORCE_TOL_MIXED
    # unequal radii: full records, rebuilt once, then kept as the radii change
    rad3 = np.random.default_rng(71).uniform(0.42, 0.5, len(rad))
    mixed, fp64 = both(psim, g, p, pos, rad3)
    assert builds(psim) == b0 + 2
    assert rel_norm(mixed, fp64) <= FORCE_TOL_MIXED
    mixed, fp64 = both(psim, g, p, pos, rad3 * 0.98)
    assert builds(psim) == b0 + 2
    assert rel_norm(mixed, fp64) <= FORCE_TOL_MIXED


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("radii", ["one", "unequal"])
def test_in_place_and_copied_arrays_agree(psim, skin_reset, monkeypatch, precision, radii):
    # the device reading the caller's arrays in place, or copies of them:
    # the same forces, bit for bit
    g, p, pos, rad, box = liquid(psim, seed=72)
    if radii == "unequal":
        rad = np.random.default_rng(73).uniform(0.42, 0.5, len(rad))
    hi, cse, srt = psim.cells_build(g, pos, rad)
    out = []
    for mode in ("0", "1"):
        monkeypatch.setenv("PSIM_DROPIN_COPIES", mode)
        psim.set_force_list_skin(0.0)   # a fresh list each call: the same summation order
        out.append(psim.force_evaluate(p, g, srt, hi, cse, precision=precision))
    assert np.array_equal(out[0], out[1])


def test_no_skin_builds_every_call(psim, skin_reset):
    g, p, pos, rad, box = liquid(psim, seed=68)
    psim.set_force_list_skin(0.0)
    b0 = builds(psim)
    for _ in range(3):
        mixed, fp64 = both(psim, g, p, pos, rad)
        assert rel_norm(mixed, fp64) <= FORCE_TOL_MIXED
    assert builds(psim) == b0 + 3


def test_skin_is_clamped_to_the_cells_room(psim, skin_reset):
    # a skin larger than cellSize - cutOff is cut to that room: still correct
    g, p, pos, rad, box = liquid(psim, seed=69)
    psim.set_force_list_skin(5.0)
    rng = np.random.default_rng(70)
    for _ in range(3):
        mixed, fp64 = both(psim, g, p, pos, rad)
        assert rel_norm(mixed, fp64) <= FORCE_TOL_MIXED
        pos = np.mod(pos + rng.uniform(-0.02, 0.02, pos.shape), box)


def test_host_link_probe(psim):
    # the denominators of the drop-ins' end-to-end roofline: finite, positive,
    # and both directions at once no slower than either alone
    link = psim.measure_host_link(0)
    assert all(v > 1.0 for v in link.values())
    assert link["both"] >= 0.9 * min(link["read"], link["write"])
