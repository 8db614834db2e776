"""Differentiable exchange: material-mode forward against the oracle, adjoint gradients against finite differences.

Tolerances: forward receiver histograms rel L2 <= 1e-4 (FP32 exchange);
gradients rel <= 2e-2 against central differences of the FP32 forward with
h = 1e-3 on the parameter (FP32 rounding of the loss limits the difference
quotient); checkpoint spacing changes nothing (same arithmetic).
"""
import numpy as np
import pytest

from conftest import rel_l2
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


def _setup(n_bins=2, K=6, duration=0.06, seed=0):
    from sparrowpy_gb300.adjoint import DifferentiableExchange, as_source, per_patch_room
    from sparrowpy_gb300.brdf import hemisphere_directions
    dirs = hemisphere_directions(8)
    r = per_patch_room((2.0, 1.5, 1.0), 0.5, dirs, n_bins)
    src = np.array([0.6, 0.5, 0.7])
    rcv = np.array([[1.4, 1.0, 0.5], [0.5, 1.1, 0.9]])
    solver = DifferentiableExchange(r, dirs, as_source(src), rcv, 343.0, 1e-3, duration, K)
    rng = np.random.default_rng(seed)
    S = solver.n_slots
    alpha = rng.uniform(0.05, 0.4, (S, n_bins))
    scat = rng.uniform(0.2, 0.8, (S, n_bins))
    return solver, r, src, rcv, alpha, scat, rng


def _t(x, grad=False):
    import torch
    return torch.tensor(x, dtype=torch.float64, device="cuda", requires_grad=grad)


def test_material_forward_matches_oracle():
    from oracle.scene import scene_from_radiosity
    from sparrowpy_gb300.adjoint import material_tables
    solver, r, src, rcv, alpha, scat, _ = _setup()
    mono = solver.forward_only(_t(alpha), _t(scat)).cpu().numpy()
    sc = scene_from_radiosity(r)
    sc["brdf"] = material_tables(_t(alpha), _t(scat), solver.mirror_np, solver.gain_np, solver.n_out).cpu().numpy()
    sc["brdf_index"] = solver.slot_of_wall.astype(np.int64)
    ref = orc.solve(sc, src, rcv, 343.0, 1e-3, 0.06, 6)
    assert rel_l2(mono, ref["mono"]) < 1e-4


def test_adjoint_gradient_matches_finite_differences():
    from sparrowpy_gb300.adjoint import energy_decay_loss
    solver, r, src, rcv, alpha, scat, rng = _setup()
    target = solver.forward_only(_t(np.clip(alpha * 0.8 + 0.05, 0, 0.9)), _t(np.clip(scat * 0.7 + 0.1, 0, 1)))
    a_t, s_t = _t(alpha, True), _t(scat, True)
    loss = energy_decay_loss(solver(a_t, s_t), target)
    loss.backward()
    ga, gs = a_t.grad.cpu().numpy(), s_t.grad.cpu().numpy()

    def loss_at(a, s):
        return float(energy_decay_loss(solver.forward_only(_t(a), _t(s)), target))

    h = 1e-3
    flat = np.abs(np.concatenate([ga.ravel(), gs.ravel()]))
    picks = np.argsort(flat)[::-1][:6]  # the largest gradients (well above the FP32 noise of the quotient)
    for q in picks:
        which, k = (0, q) if q < ga.size else (1, q - ga.size)
        idx = np.unravel_index(k, ga.shape)
        ap, am, sp, sm = alpha.copy(), alpha.copy(), scat.copy(), scat.copy()
        if which == 0:
            ap[idx] += h
            am[idx] -= h
        else:
            sp[idx] += h
            sm[idx] -= h
        fd = (loss_at(ap, sp) - loss_at(am, sm)) / (2 * h)
        g = (ga if which == 0 else gs)[idx]
        assert abs(g - fd) <= 2e-2 * abs(fd), (which, idx, g, fd)


def test_adjoint_checkpoint_spacing_is_exact():
    import torch
    from sparrowpy_gb300.adjoint import DifferentiableExchange, as_source, energy_decay_loss
    from sparrowpy_gb300.brdf import hemisphere_directions
    solver, r, src, rcv, alpha, scat, _ = _setup()
    target = solver.forward_only(_t(alpha * 0.9), _t(scat))
    grads = []
    for m in (1, 2, 4):
        s2 = DifferentiableExchange(r, hemisphere_directions(8), as_source(src), rcv, 343.0, 1e-3, 0.06, 6,
                                    checkpoint_every=m)
        a_t, s_t = _t(alpha, True), _t(scat, True)
        energy_decay_loss(s2(a_t, s_t), target).backward()
        grads.append(torch.cat([a_t.grad.reshape(-1), s_t.grad.reshape(-1)]).cpu().numpy())
    np.testing.assert_allclose(grads[1], grads[0], rtol=1e-12, atol=0)
    np.testing.assert_allclose(grads[2], grads[0], rtol=1e-12, atol=0)
