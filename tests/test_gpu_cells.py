"""Cell-list rebuild on the GPU against the reference's golden vectors and the
oracle: hashes, cellStartEnd and sorted particles bit-exact."""
import numpy as np
import pytest

from gpu_helpers import rsa_state
from oracle import port

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True, params=["direct", "copies"])
def host_access(request, monkeypatch):
    """Both drop-in paths: the device on the caller's arrays in place (a device
    with pageable host memory access), or copies in and out."""
    monkeypatch.setenv("PSIM_DROPIN_COPIES", "1" if request.param == "copies" else "0")
    return request.param


def test_cells_match_reference_golden(psim, golden):
    n, box, cs, scale = (int(v) for v in golden["cellsA_geom"])
    hi, cse, srt = psim.cells_build(psim.geometry(n, box, cs, scale), golden["cellsA_pos"],
                                    golden["cellsA_radius"])
    assert np.array_equal(hi, golden["cellsA_hash_index"])
    assert np.array_equal(cse, golden["cellsA_cse"])
    assert np.array_equal(srt, golden["cellsA_sorted"])


@pytest.mark.parametrize("n,box,scale,seed", [
    (4000, 21.0, 7, 1),          # the reference-constructible AO box
    (20000, 41.53, 13, 2),       # real-valued box
    (50000, 60.0, 24, 3),        # small cells (0.4 per cell on average)
])
def test_cells_match_oracle(psim, n, box, scale, seed):
    rng = np.random.default_rng(seed)
    pos = rng.uniform(0, box, 3 * n)
    rad = np.full(n, 0.5)
    g = psim.geometry(n, box, box / scale, scale)
    hi, cse, srt = psim.cells_build(g, pos, rad)
    og = port.geom(n, box, box / scale, scale)
    ohi, ocse, osrt = port.build_cells(og, pos, rad)
    assert np.array_equal(hi, ohi)
    assert np.array_equal(cse, ocse)
    assert np.array_equal(srt, osrt)


def test_cells_edge_cases(psim):
    box, scale = 12.0, 4
    g = psim.geometry(0, box, 3.0, scale)
    hi, cse, srt = psim.cells_build(g, np.zeros(0), np.zeros(0))
    assert hi.size == 0 and np.all(cse == 0xFFFFFFFF)
    # exact cell boundaries, the origin, just below L, and a crowded cell
    pts = [0.0, 0.0, 0.0, 3.0, 3.0, 3.0, 6.0, 9.0, 11.999999999999998,
           np.nextafter(3.0, 0.0), 3.0, 0.0] + [1.0, 1.0, 1.0] * 5
    pos = np.array(pts)
    n = len(pos) // 3
    g = psim.geometry(n, box, 3.0, scale)
    hi, cse, srt = psim.cells_build(g, pos, np.full(n, 0.5))
    ohi, ocse, osrt = port.build_cells(port.geom(n, box, 3.0, scale), pos, np.full(n, 0.5))
    assert np.array_equal(hi, ohi) and np.array_equal(cse, ocse) and np.array_equal(srt, osrt)


def test_cells_outside_grid_is_reported(psim):
    g = psim.geometry(2, 12.0, 3.0, 4)
    with pytest.raises(psim.PsimError) as e:
        psim.cells_build(g, np.array([1.0, 1.0, 1.0, 12.5, 1.0, 1.0]), np.full(2, 0.5))
    assert e.value.code == psim.ERR_CELL_BOUNDS
