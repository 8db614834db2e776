"""Differentiable exchange: material-mode forward against the oracle, adjoint gradients against FP64 references.

Tolerances:
* forward receiver histograms: rel L2 <= 1e-4 (FP32 exchange), <= 1e-10
  (FP64 exchange) against the oracle;
* the FP64 adjoint against central differences (h = 1e-4) of the oracle's
  FP64 solve (the reference's own arithmetic, RadiosityFast.py:1073-1185)
  on 64 seeded random parameters: |g - fd| <= 1e-5 |fd| + 1e-7 max|fd|
  (the differences' truncation error is O(h^2), about 1e-8 relative);
* the FP64 GPU forward's central differences equal the oracle's to the same
  bound;
* the FP32 adjoint against the FP64 adjoint on every parameter, and against
  the FP64 central differences on the 64: within 2e-3 max|g| (FP32
  rounding of the histograms, about 1e-6 relative, grows through the
  log-EDC loss);
* checkpoint spacing changes nothing (same arithmetic).
"""
import numpy as np
import pytest

from conftest import rel_l2
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


def _setup(n_bins=2, K=6, duration=0.06, seed=0, precision="fp32"):
    from sparrowpy_gb300.adjoint import DifferentiableExchange, as_source, per_patch_room
    from sparrowpy_gb300.brdf import hemisphere_directions
    dirs = hemisphere_directions(8)
    r = per_patch_room((2.0, 1.5, 1.0), 0.5, dirs, n_bins, precision=precision)
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


@pytest.mark.parametrize("precision,tol", [("fp32", 1e-4), ("fp64", 1e-10)])
def test_material_forward_matches_oracle(precision, tol):
    from oracle.scene import scene_from_radiosity
    from sparrowpy_gb300.adjoint import material_tables
    solver, r, src, rcv, alpha, scat, _ = _setup(precision=precision)
    mono = solver.forward_only(_t(alpha), _t(scat)).cpu().numpy()
    sc = scene_from_radiosity(r)
    sc["brdf"] = material_tables(_t(alpha), _t(scat), solver.mirror_np, solver.gain_np, solver.n_out).cpu().numpy()
    sc["brdf_index"] = solver.slot_of_wall.astype(np.int64)
    ref = orc.solve(sc, src, rcv, 343.0, 1e-3, 0.06, 6)
    assert rel_l2(mono, ref["mono"]) < tol


def _np_loss(mono, target, eps=1e-30):
    """energy_decay_loss (sparrowpy_gb300.adjoint) in NumPy FP64."""
    edc = np.flip(np.cumsum(np.flip(mono, -1), -1), -1)
    edc_t = np.flip(np.cumsum(np.flip(target, -1), -1), -1)
    return float(np.sum((np.log(edc + eps) - np.log(edc_t + eps)) ** 2))


def _oracle_loss_fn(solver, r, src, rcv, target_np):
    """Loss of the oracle's FP64 solve for given materials (bake once, then source, exchange, collection)."""
    from oracle.scene import scene_from_radiosity
    from sparrowpy_gb300.adjoint import material_tables
    sc = scene_from_radiosity(r)
    sc["brdf_index"] = solver.slot_of_wall.astype(np.int64)
    bk = orc.bake(sc)

    def loss(alpha, scat):
        sc["brdf"] = material_tables(_t(alpha), _t(scat), solver.mirror_np, solver.gain_np, solver.n_out).cpu().numpy()
        e0dir, d0, _ = orc.init_source(sc, bk, src)
        etot = orc.exchange(sc, bk, e0dir, d0, solver.c, solver.dt, solver.nt, solver.K)
        return _np_loss(orc.collect(sc, bk, etot, rcv, solver.c, solver.dt), target_np)
    return loss


def _central(loss, alpha, scat, picks, h):
    out = []
    for which, idx in picks:
        vals = []
        for sign in (1, -1):
            a, s_ = alpha.copy(), scat.copy()
            (a if which == 0 else s_)[idx] += sign * h
            vals.append(loss(a, s_))
        out.append((vals[0] - vals[1]) / (2 * h))
    return np.array(out)


def _picks(shape, n, seed):
    rng = np.random.default_rng(seed)
    flat = rng.choice(2 * shape[0] * shape[1], size=n, replace=False)
    return [(int(q >= shape[0] * shape[1]), np.unravel_index(int(q % (shape[0] * shape[1])), shape)) for q in flat]


def _gradients(precision, alpha, scat, target):
    from sparrowpy_gb300.adjoint import DifferentiableExchange, as_source, energy_decay_loss, per_patch_room
    from sparrowpy_gb300.brdf import hemisphere_directions
    dirs = hemisphere_directions(8)
    r = per_patch_room((2.0, 1.5, 1.0), 0.5, dirs, 2, precision=precision)
    src = np.array([0.6, 0.5, 0.7])
    rcv = np.array([[1.4, 1.0, 0.5], [0.5, 1.1, 0.9]])
    solver = DifferentiableExchange(r, dirs, as_source(src), rcv, 343.0, 1e-3, 0.06, 6)
    a_t, s_t = _t(alpha, True), _t(scat, True)
    energy_decay_loss(solver(a_t, s_t), target).backward()
    return solver, r, src, rcv, a_t.grad.cpu().numpy(), s_t.grad.cpu().numpy()


def test_adjoint_gradients_against_fp64_references():
    from sparrowpy_gb300.adjoint import energy_decay_loss
    solver, r, src, rcv, alpha, scat, rng = _setup()
    target = solver.forward_only(_t(np.clip(alpha * 0.8 + 0.05, 0, 0.9)), _t(np.clip(scat * 0.7 + 0.1, 0, 1)))
    _, _, _, _, ga32, gs32 = _gradients("fp32", alpha, scat, target)
    solver64, r64, _, _, ga64, gs64 = _gradients("fp64", alpha, scat, target)
    g32 = np.concatenate([ga32.ravel(), gs32.ravel()])
    g64 = np.concatenate([ga64.ravel(), gs64.ravel()])
    scale = np.abs(g64).max()
    assert scale > 0
    # FP32 adjoint against the FP64 adjoint, every parameter
    assert np.abs(g32 - g64).max() <= 2e-3 * scale
    # 64 seeded random parameters: central differences (h = 1e-4) of the oracle and of the FP64 GPU forward
    picks = _picks(alpha.shape, 64, seed=17)
    h = 1e-4
    fd_orc = _central(_oracle_loss_fn(solver64, r64, src, rcv, target.cpu().numpy()), alpha, scat, picks, h)
    fd_gpu = _central(lambda a, s_: float(energy_decay_loss(solver64.forward_only(_t(a), _t(s_)), target)), alpha,
                      scat, picks, h)
    sel = lambda g_a, g_s: np.array([(g_a if w == 0 else g_s)[i] for w, i in picks])
    fd_scale = np.abs(fd_orc).max()
    bound = 1e-5 * np.abs(fd_orc) + 1e-7 * fd_scale
    assert np.all(np.abs(fd_gpu - fd_orc) <= bound)
    assert np.all(np.abs(sel(ga64, gs64) - fd_orc) <= bound)
    assert np.abs(sel(ga32, gs32) - fd_orc).max() <= 2e-3 * fd_scale


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
