"""The differentiable trajectory: its forward against the system's plain FP64
form, and its adjoint gradients against central finite differences."""
import math
import time

import numpy as np
import pytest

from gpu_helpers import rsa_state

pytestmark = pytest.mark.gpu


def setup(psim, n=300, phi=0.18, seed=90):
    box = (n * math.pi / 6.0 / phi) ** (1.0 / 3.0)
    scale = max(3, int(box // 3.1))         # cells of >= 3.1: the Yukawa cutoff and g(r) reach
    pos, rad = rsa_state(n, box, seed=seed)
    vel = np.random.default_rng(seed).standard_normal(3 * n)
    return psim.geometry(n, box, box / scale, scale), pos, vel


def test_forward_matches_system_fp64(psim):
    from proteinsim2015_gb300 import adjoint as adj
    g, pos, vel = setup(psim)
    n = g.n_particles
    p, _ = adj.plugin_params(3.0, 0.1, 10.0, 4.0)
    steps = 30
    a = adj.Adjoint(g, steps, dt=0.001, seed=4242, checkpoint_every=8, sample_every=5)
    _, x = a.forward(p, pos, vel, final=True)
    a.close()
    f = psim.make_force("AO_YUK", p.ao_cutoff, kT=1.0, well_depth=p.ao_well_depth,
                        cutoff2=p.yuk_cutoff, well_depth2=1.0, yukawa_strength=p.yuk_amplitude,
                        debye_length=p.yuk_length, lj_num=0)
    s = psim.System(g, f, gamma=1.0, dt=0.001, kT=1.0, vel_freq=1000, seed=4242,
                    precision=psim.PRECISION_FP64)
    s.upload(pos, np.full(n, 0.5), vel=vel)
    s.step(steps)
    ref = s.download()["pos"]
    s.close()
    d = x - ref
    d -= g.box_size * np.round(d / g.box_size)   # the adjoint keeps positions unwrapped
    assert np.max(np.abs(d)) < 1e-9


def test_gradient_matches_central_differences(psim):
    from proteinsim2015_gb300 import adjoint as adj
    g, pos, vel = setup(psim, seed=91)
    a = adj.Adjoint(g, 40, dt=0.001, seed=7, checkpoint_every=16, sample_every=4, n_bins=60)
    p, _ = adj.plugin_params(3.0, 0.1, 10.0, 4.0)
    pt, _ = adj.plugin_params(3.3, 0.1, 9.0, 4.2)
    target = a.forward(pt, pos, vel)
    loss, gm, grad, gpos = a.gradient(p, pos, target, vel, wrt_pos=True)
    assert loss > 0 and np.all(np.isfinite(grad)) and np.all(np.isfinite(gpos))
    assert loss == pytest.approx(float(np.sum((gm - target) ** 2)), rel=1e-12)

    def loss_at(q, x=pos):
        return float(np.sum((a.forward(q, x, vel) - target) ** 2))

    # smooth parameters: AO strength, Yukawa amplitude and length
    for k, name in ((0, "ao_well_depth"), (2, "yuk_amplitude"), (3, "yuk_length")):
        h = 1e-5 * getattr(p, name)
        qp, qm = adj.AdjointParams.from_buffer_copy(p), adj.AdjointParams.from_buffer_copy(p)
        setattr(qp, name, getattr(p, name) + h)
        setattr(qm, name, getattr(p, name) - h)
        fd = (loss_at(qp) - loss_at(qm)) / (2 * h)
        assert grad[k] == pytest.approx(fd, rel=1e-4, abs=1e-9 * abs(loss) / h), name
    # a few initial coordinates
    rng = np.random.default_rng(3)
    for idx in rng.choice(3 * g.n_particles, 4, replace=False):
        h = 1e-6
        xp, xm = pos.copy(), pos.copy()
        xp[idx] += h
        xm[idx] -= h
        fd = (loss_at(p, xp) - loss_at(p, xm)) / (2 * h)
        assert gpos[idx] == pytest.approx(fd, rel=1e-4, abs=1e-7 * np.max(np.abs(gpos))), idx
    a.close()


def test_torch_function_and_cost(psim):
    torch = pytest.importorskip("torch")
    from proteinsim2015_gb300 import adjoint as adj
    g, pos, vel = setup(psim, n=600, phi=0.15, seed=92)
    a = adj.Adjoint(g, 100, dt=0.001, seed=11, checkpoint_every=25, sample_every=10)
    pt, _ = adj.plugin_params(3.3, 0.1, 9.0, 4.2)
    target = a.forward(pt, pos, vel)
    F = adj.trajectory_loss_function()
    theta = torch.tensor([3.0, 0.1, 10.0, 4.0], dtype=torch.float64, requires_grad=True)
    loss = F.apply(theta, a, pos, vel, target)
    loss.backward()
    p, J = adj.plugin_params(3.0, 0.1, 10.0, 4.0)
    _, _, grad, _ = a.gradient(p, pos, target, vel)
    assert np.allclose(theta.grad.numpy(), (J.T @ grad)[:4], rtol=1e-12)
    t0 = time.perf_counter()
    a.forward(p, pos, vel)
    t1 = time.perf_counter()
    a.gradient(p, pos, target, vel)
    t2 = time.perf_counter()
    print("adjoint cost / forward:", (t2 - t1) / (t1 - t0))
    a.close()


def _lj_params(adj, **kw):
    d = dict(lj_epsilon=0.3, lj_sigma=1.0, lj_n=6, lj_cutoff=2.0)
    d.update(kw)
    return adj.plugin_params(3.0, 0.1, 10.0, 4.0, **d)


def test_gradient_matches_forward_mode_tangent(psim, oracle_port):
    # the FP64 reverse sweep on the GPU against FP64 forward-mode tangents on
    # the CPU (oracle/psim_tangent.c), on the same trajectory: the GPU's own
    # Philox draws replayed; all six plugin parameters, the LJ(n) term on
    from proteinsim2015_gb300 import adjoint as adj
    g, pos, vel = setup(psim, seed=93)
    n, T, every, nb, seed = g.n_particles, 40, 4, 60, 19
    a = adj.Adjoint(g, T, dt=0.001, seed=seed, checkpoint_every=16, sample_every=every, n_bins=nb)
    p, _ = _lj_params(adj)
    pt, _ = _lj_params(adj, lj_epsilon=0.33, lj_sigma=1.03)
    target = a.forward(pt, pos, vel)
    loss, gm, grad, _ = a.gradient(p, pos, target, vel)
    a.close()
    noise = psim.philox_noise(seed, n, 0, T)
    tl, tg, tgrad = oracle_port.adjoint_tangent(g.box_size, p, 1.0, 0.001, 1.0, 1.0, T, every,
                                                0.8, 3.0, nb, (3.0 - 0.8) / nb, pos, vel, noise,
                                                target)
    assert loss == pytest.approx(tl, rel=1e-9)
    assert np.allclose(gm, tg, rtol=1e-9, atol=1e-12)
    for k, name in enumerate(adj.GRAD_NAMES):
        assert grad[k] == pytest.approx(tgrad[k], rel=1e-6, abs=1e-9 * max(abs(tgrad))), name


def test_gradient_matches_central_differences_at_4096(psim):
    # N = 4096, 200 steps: every parameter, q (the AO coefficients' range,
    # the cutoff held) and the LJ epsilon and sigma included.  The pair
    # forces jump at their cutoffs (the reference's AO soft core is cut at
    # 1 + q), so the loss is only piecewise smooth: a step of 1e-7 relative
    # keeps the +h and -h runs from differing by a pair crossing a cutoff,
    # which at 1e-5 happens about twice per evaluation at this size.  Each
    # forward run's smoothed g(r) is summed with atomics, so its loss carries
    # ~1e-13 relative rounding noise; against the loss change of a 1e-7 step
    # that bounds the agreement near 1e-4 (the exact comparison is the
    # forward-mode tangent above).
    from proteinsim2015_gb300 import adjoint as adj
    g, pos, vel = setup(psim, n=4096, phi=0.15, seed=94)
    a = adj.Adjoint(g, 200, dt=0.001, seed=23, checkpoint_every=50, sample_every=10, n_bins=100)
    p, _ = _lj_params(adj)
    pt, _ = _lj_params(adj, lj_epsilon=0.33, lj_sigma=1.03)
    pt.ao_well_depth *= 1.1
    target = a.forward(pt, pos, vel)
    loss, _, grad, _ = a.gradient(p, pos, target, vel)
    fds = []
    for k, name in enumerate(adj.GRAD_NAMES):
        v = getattr(p, name)
        h = 1e-7 * abs(v)
        qp, qm = adj.AdjointParams.from_buffer_copy(p), adj.AdjointParams.from_buffer_copy(p)
        setattr(qp, name, v + h)
        setattr(qm, name, v - h)
        fd = (np.sum((a.forward(qp, pos, vel) - target) ** 2) -
              np.sum((a.forward(qm, pos, vel) - target) ** 2)) / (2 * h)
        fds.append((name, grad[k], fd, h))
        print(name, grad[k], fd, abs(grad[k] - fd) / abs(fd))
    a.close()
    for name, gk, fd, h in fds:
        assert gk == pytest.approx(fd, rel=5e-4, abs=1e-12 * loss / h), name
