"""Gradients of a trajectory's smoothed g(r) loss with the noise held fixed
(psim_adjoint_* in the C ABI), and a torch.autograd.Function over them.

The differentiable workload: colloids with the AO depletion attraction of the
AOPotential plugin and the screened-Coulomb (Yukawa) repulsion
U = A e^{-kappa (r - sigma)} / r, which the LennardJones plugin gives with
ljNum = 0, debyeLength = 1/kappa and kT wellDepth yukawaStrength =
A kappa e^{kappa sigma}, optionally with the LennardJones plugin's LJ(n) term
(energy eps, contact diameter sigma_lj).  Physical parameters (AO contact
attraction in kT, q = polymer/colloid size ratio, A, kappa, eps, sigma_lj)
map to the plugin parameters here and the gradients map back by the chain
rule.
"""
import ctypes as C
import math

import numpy as np

from . import Geometry, IntegratorConfig, PsimError, _check, _p, lib


class AdjointConfig(C.Structure):
    _fields_ = [("geom", Geometry), ("integ", IntegratorConfig), ("mass", C.c_double),
                ("n_steps", C.c_int32), ("checkpoint_every", C.c_int32),
                ("sample_every", C.c_int32), ("r_min", C.c_double), ("r_max", C.c_double),
                ("n_bins", C.c_int32), ("sigma", C.c_double)]


class AdjointParams(C.Structure):
    _fields_ = [("kT", C.c_double), ("ao_well_depth", C.c_double), ("ao_cutoff", C.c_double),
                ("yuk_amplitude", C.c_double), ("yuk_length", C.c_double),
                ("yuk_cutoff", C.c_double), ("ao_range", C.c_double),
                ("lj_epsilon", C.c_double), ("lj_sigma", C.c_double), ("lj_cutoff", C.c_double),
                ("lj_n", C.c_int32)]


# the components of Adjoint.gradient's grad: the plugin parameters
GRAD_NAMES = ("ao_well_depth", "ao_range", "yuk_amplitude", "yuk_length", "lj_epsilon",
              "lj_sigma")


_SIGS = {
    "psim_adjoint_create": ([C.POINTER(AdjointConfig), C.c_int32], C.c_void_p),
    "psim_adjoint_destroy": ([C.c_void_p], None),
    "psim_adjoint_forward": ([C.c_void_p, C.POINTER(AdjointParams)] + [C.c_void_p] * 4, C.c_int),
    "psim_adjoint_gradient": ([C.c_void_p, C.POINTER(AdjointParams)] + [C.c_void_p] * 7, C.c_int),
}


def _lib():
    L = lib()
    for name, (args, res) in _SIGS.items():
        fn = getattr(L, name)
        fn.argtypes, fn.restype = args, res
    return L


def plugin_params(ao_contact_kT, q, yuk_A, kappa, kT=1.0, yuk_cutoff=3.0, sigma=1.0,
                  lj_epsilon=0.0, lj_sigma=1.0, lj_n=6, lj_cutoff=0.0):
    """(AdjointParams, d(plugin params)/d(physical params) as a 6x6 Jacobian)
    for AO attraction ao_contact_kT at size ratio q, Yukawa (A, kappa) and,
    when lj_cutoff > 0, the LennardJones plugin's LJ(n) term with energy
    lj_epsilon (= kT wellDepth) and contact diameter lj_sigma.  Rows: the
    plugin parameters of GRAD_NAMES; columns: (A_ao, q, A, kappa, eps,
    sigma_lj).  q moves the AO coefficients' range 1 + q; differentiation
    holds the cutoff distance (also 1 + q) fixed."""
    wd = ao_contact_kT * q / (1.5 + q)
    rc = 1.0 + q
    Y = yuk_A * kappa * math.exp(kappa * sigma)
    lam = 1.0 / kappa
    p = AdjointParams(kT=kT, ao_well_depth=wd, ao_cutoff=rc, yuk_amplitude=Y, yuk_length=lam,
                      yuk_cutoff=yuk_cutoff, ao_range=rc, lj_epsilon=lj_epsilon,
                      lj_sigma=lj_sigma, lj_cutoff=lj_cutoff, lj_n=lj_n)
    J = np.zeros((6, 6))
    J[0, 0] = q / (1.5 + q)
    J[0, 1] = ao_contact_kT * 1.5 / (1.5 + q) ** 2
    J[1, 1] = 1.0
    J[2, 2] = kappa * math.exp(kappa * sigma)
    J[2, 3] = yuk_A * math.exp(kappa * sigma) * (1.0 + kappa * sigma)
    J[3, 3] = -1.0 / kappa ** 2
    J[4, 4] = 1.0
    J[5, 5] = 1.0
    return p, J


class Adjoint:
    """A trajectory of n_steps from fixed initial positions/velocities and
    fixed Philox noise, its smoothed g(r), and the loss gradient."""

    def __init__(self, geom, n_steps, gamma=1.0, dt=0.001, kT=1.0, seed=90210, mass=1.0,
                 checkpoint_every=100, sample_every=10, r_min=0.8, r_max=3.0, n_bins=100,
                 sigma=None, device=0):
        dr = (r_max - r_min) / n_bins
        self.cfg = AdjointConfig(geom=geom,
                                 integ=IntegratorConfig(gamma=gamma, dt=dt, kT=kT, vel_freq=0,
                                                        seed=seed),
                                 mass=mass, n_steps=n_steps, checkpoint_every=checkpoint_every,
                                 sample_every=sample_every, r_min=r_min, r_max=r_max,
                                 n_bins=n_bins, sigma=dr if sigma is None else sigma)
        self.n = geom.n_particles
        self.n_bins = n_bins
        self.r = r_min + (np.arange(n_bins) + 0.5) * dr
        self._h = _lib().psim_adjoint_create(C.byref(self.cfg), device)
        if not self._h:
            raise PsimError(7706, lib().psim_last_error_string().decode())

    def forward(self, params, pos0, vel0=None, final=False):
        g = np.empty(self.n_bins)
        out = np.empty(3 * self.n) if final else None
        _check(_lib().psim_adjoint_forward(self._h, C.byref(params), _p(np.ascontiguousarray(pos0,
                                           dtype=np.float64)), _p(None if vel0 is None else
                                           np.ascontiguousarray(vel0, dtype=np.float64)), _p(g),
                                           _p(out)))
        return (g, out) if final else g

    def gradient(self, params, pos0, g_target, vel0=None, wrt_pos=False):
        """(loss, g_mean, dL/d(plugin parameters of GRAD_NAMES), dL/dpos0 or None)."""
        loss = np.zeros(1)
        g = np.empty(self.n_bins)
        grad = np.empty(6)
        gp = np.empty(3 * self.n) if wrt_pos else None
        _check(_lib().psim_adjoint_gradient(
            self._h, C.byref(params), _p(np.ascontiguousarray(pos0, dtype=np.float64)),
            _p(None if vel0 is None else np.ascontiguousarray(vel0, dtype=np.float64)),
            _p(np.ascontiguousarray(g_target, dtype=np.float64)), _p(loss), _p(g), _p(grad),
            _p(gp)))
        return float(loss[0]), g, grad, gp

    def close(self):
        if getattr(self, "_h", None):
            _lib().psim_adjoint_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def trajectory_loss_function():
    """A torch.autograd.Function: loss(theta) with theta = (AO contact kT, q,
    Yukawa A, kappa[, LJ epsilon, LJ sigma]) as a float64 tensor (with the
    two LJ entries, plugin_params' lj_cutoff keyword goes in `lj`); backward
    runs the adjoint."""
    import torch

    class TrajectoryLoss(torch.autograd.Function):
        @staticmethod
        def forward(ctx, theta, adj, pos0, vel0, g_target, lj=None):
            t = [float(v) for v in theta.detach().cpu()]
            kw = dict(lj or {})
            if len(t) == 6:
                kw.update(lj_epsilon=t[4], lj_sigma=t[5])
            p, J = plugin_params(*t[:4], **kw)
            loss, _, grad, _ = adj.gradient(p, pos0, g_target, vel0)
            full = J.T @ grad
            ctx.save_for_backward(torch.as_tensor(full[:len(t)], dtype=theta.dtype))
            return theta.new_tensor(loss)

        @staticmethod
        def backward(ctx, g_out):
            (grad,) = ctx.saved_tensors
            return g_out * grad.to(g_out.device), None, None, None, None, None

    return TrajectoryLoss
