"""CPU checks of the FP64 substep model used to judge the GPU adjoint: its forward map
agrees with the oracle's reference-exact stages, and its transpose agrees with central
differences of itself."""
import numpy as np
import pytest

import oracle_api as O
from adjoint_model import RolloutModel, SubstepModel, loss_grad_vy2, loss_vy2
from ffengine_gb300 import scenes

DT = 1 / 240


@pytest.fixture(scope="module")
def case():
    n = 16
    pos, vel = scenes.dam_break_particles(n, 0.4, 0.6, seed=0, velocity_sigma=0.5)
    solid = O.solid_phi(n, 1.0 / n)
    return n, pos, vel, solid, SubstepModel(n, pos, vel, solid, dt=DT)


def oracle_v1(n, pos, vel, solid):
    dx = 1.0 / n
    w = O.face_weights(n, solid)
    phi = O.postprocess_sdf(n, dx, solid, O.liquid_sdf(n, dx, pos))
    L = O.layers(5)
    adv = [O.extrapolate(f, v, L) for f, v in O.p2g(n, dx, pos, vel)]
    body = O.body_force(n, DT, (0, -9.81, 0), *adv)
    pr, it, ok, err, nf = O.pressure_solve(n, dx, DT, phi, w, body, tol=1e-12, float_scalars=False)
    proj, valid = O.apply_pressure(n, dx, DT, phi, w, pr, body)
    projx = [O.extrapolate(a, v, L) for a, v in zip(proj, valid)]
    cons = O.constrain(n, w, projx)
    saved = O.constrain(n, w, adv)
    return O.g2p(n, dx, 0.05, pos, vel, cons, saved)


def test_model_forward_matches_oracle(case):
    n, pos, vel, solid, m = case
    v1 = m.forward(vel)
    ref = oracle_v1(n, pos, vel, solid)
    assert np.abs(v1 - ref).max() <= 2e-5 * np.abs(ref).max()


def test_model_transpose_matches_its_differences(case):
    n, pos, vel, solid, m = case
    v0 = vel.astype(np.float64)
    v1 = m.forward(v0)
    mask = pos[:, 1] > 0.45
    g = m.vjp(loss_grad_vy2(v1, mask))
    rng = np.random.default_rng(5)
    for _ in range(8):
        d = rng.standard_normal(v0.shape)
        fd = (loss_vy2(m.forward(v0 + 1e-4 * d), mask) - loss_vy2(m.forward(v0 - 1e-4 * d), mask)) / 2e-4
        assert abs(fd - (g * d).sum()) <= 1e-7 * max(1.0, abs(fd))


@pytest.fixture(scope="module")
def floating():
    n = 16
    pos, vel = scenes.floating_block_particles(n, seed=3, velocity_sigma=0.5)
    return n, pos, vel, O.solid_phi(n, 1.0 / n)


def test_state_model_positions_match_oracle_advection(floating):
    n, pos, vel, solid = floating
    m = SubstepModel(n, pos, vel, solid, dt=DT)
    x1, v1 = m.forward_xv(pos, vel)
    # FP32 kernel weights cancel near the kernel radius; at the few faces whose total weight is
    # barely above the validity threshold the FP32 transfer and the FP64 model differ by ~1e-3
    assert np.abs(v1 - oracle_v1(n, pos, vel, solid)).max() <= 1e-4 * np.abs(v1).max()
    # the oracle's RK3 + collision handling on the same field: no particle of this scene collides
    us, scale, parts, uc, sc = m._fields(pos.astype(np.float64), vel.astype(np.float64))
    shapes = [(n, n, n + 1), (n, n + 1, n), (n + 1, n, n)]
    uvw = [uc[c].reshape(shapes[c]).astype(np.float32) for c in range(3)]
    ref = O.advect(n, 1.0 / n, DT, 5, pos, uvw, solid)
    assert np.abs(x1 - ref).max() <= 1e-6


def test_rollout_model_transpose_matches_its_differences(floating):
    n, pos, vel, solid = floating
    R = RolloutModel(n, pos, vel, solid, 2, dt=DT)
    rng = np.random.default_rng(7)
    cx, cv = rng.standard_normal(pos.shape), rng.standard_normal(pos.shape)
    gx, gv = R.vjp(cx, cv)
    x0, v0 = pos.astype(np.float64), vel.astype(np.float64)
    eps = 1e-6
    for _ in range(4):
        dxp, dvp = rng.standard_normal(pos.shape) / n, rng.standard_normal(pos.shape)
        xp, vp = R.forward(x0 + eps * dxp, v0 + eps * dvp)
        xm, vm = R.forward(x0 - eps * dxp, v0 - eps * dvp)
        fd = ((cx * (xp - xm)).sum() + (cv * (vp - vm)).sum()) / (2 * eps)
        assert abs(fd - ((gx * dxp).sum() + (gv * dvp).sum())) <= 1e-6 * abs(fd)
