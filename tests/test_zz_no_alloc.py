"""psim_cells_build_noalloc: the cell-list build for callers that cannot
allocate device memory themselves (they hand in their own device buffers and
the build's scratch lives in a static device array of the library).

The test plays such a caller: PyTorch owns the device buffers, the entry point
is called through the C ABI with their addresses, and its output must equal
psim_cells_build's (bit for bit: integer work and copies) on two calls in a
row -- the second call reuses the static scratch left by the first.  This
file is collected last so that a run stopping at the first failure has
already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _case(n, box, scale, seed):
    rng = np.random.default_rng(seed)
    pos = rng.uniform(0.0, box, 3 * n)
    rad = np.full(n, 0.5)
    return pos, rad


def _noalloc_rc(psim, torch, geom, pos, rad, stream=None):
    """Call the entry point on device buffers PyTorch owns; returns the status
    and the three outputs as host arrays."""
    n, ncell = geom.n_particles, geom.cell_scale ** 3
    dev = torch.device("cuda:0")
    d_pos = torch.from_numpy(pos).to(dev)
    d_rad = torch.from_numpy(rad).to(dev)
    d_hi = torch.empty(2 * n, dtype=torch.int32, device=dev)
    d_cse = torch.empty(2 * ncell, dtype=torch.int32, device=dev)
    d_srt = torch.empty(4 * n, dtype=torch.float64, device=dev)
    assert d_srt.data_ptr() % 32 == 0
    torch.cuda.synchronize()
    st = None if stream is None else C.c_void_p(stream.cuda_stream)
    rc = psim.lib().psim_cells_build_noalloc(
        C.byref(geom), C.c_void_p(d_pos.data_ptr()), C.c_void_p(d_rad.data_ptr()),
        C.c_void_p(d_hi.data_ptr()), C.c_void_p(d_cse.data_ptr()),
        C.c_void_p(d_srt.data_ptr()), st)
    torch.cuda.synchronize()
    return rc, (d_hi.cpu().numpy(), d_cse.cpu().numpy().view(np.uint32), d_srt.cpu().numpy())


def _noalloc(psim, torch, geom, pos, rad, stream=None):
    rc, out = _noalloc_rc(psim, torch, geom, pos, rad, stream)
    assert rc == 0, psim.lib().psim_last_error_string()
    return out


@pytest.mark.parametrize("n,box,scale", [(4000, 21.0, 7), (20000, 41.53, 13)])
def test_noalloc_matches_cells_build_twice(psim, n, box, scale):
    torch = pytest.importorskip("torch")
    g = psim.geometry(n, box, box / scale, scale)
    for seed in (1, 2):  # two calls in a row on the shared static scratch
        pos, rad = _case(n, box, scale, seed)
        ref = psim.cells_build(g, pos, rad)
        got = _noalloc(psim, torch, g, pos, rad)
        for a, b in zip(got, ref):
            assert np.array_equal(a, b)


def test_noalloc_on_a_side_stream(psim):
    # the work is queued on the caller's stream, not the default one
    torch = pytest.importorskip("torch")
    n, box, scale = 4000, 21.0, 7
    g = psim.geometry(n, box, box / scale, scale)
    side = torch.cuda.Stream()
    for seed in (3, 4):
        pos, rad = _case(n, box, scale, seed)
        ref = psim.cells_build(g, pos, rad)
        got = _noalloc(psim, torch, g, pos, rad, stream=side)
        for a, b in zip(got, ref):
            assert np.array_equal(a, b)


def test_noalloc_reports_a_particle_outside_the_grid(psim):
    # a position beyond the box hashes outside the grid: the kernel clamps the
    # cell it writes and raises the 7702 bit, as psim_cells_build does; a
    # clean call afterwards is unaffected by the flagged one
    torch = pytest.importorskip("torch")
    g = psim.geometry(2, 12.0, 3.0, 4)
    pos = np.array([1.0, 1.0, 1.0, 12.5, 1.0, 1.0])
    rc, _ = _noalloc_rc(psim, torch, g, pos, np.full(2, 0.5))
    assert rc == psim.ERR_CELL_BOUNDS
    pos[3] = 11.5
    got = _noalloc(psim, torch, g, pos, np.full(2, 0.5))
    ref = psim.cells_build(g, pos, np.full(2, 0.5))
    for a, b in zip(got, ref):
        assert np.array_equal(a, b)


def test_noalloc_refuses_oversized_problem(psim):
    # 2^20 particles need ~80 MB of scratch, beyond the 32 MiB array.  Every
    # buffer is NULL: the size check refuses first, and were the checks ever
    # reordered the NULL-buffer check would refuse on the host, so no kernel
    # can be handed an address it does not own.
    n = 1 << 20
    g = psim.geometry(n, 100.0, 100.0 / 40, 40)
    rc = psim.lib().psim_cells_build_noalloc(C.byref(g), None, None, None, None, None, None)
    assert rc == psim.ERR_INPUT
    assert b"static scratch" in psim.lib().psim_last_error_string()
