"""CPU checks of the FP64 substep model used to judge the GPU adjoint: its forward map
agrees with the oracle's reference-exact stages, and its transpose agrees with central
differences of itself."""
import numpy as np
import pytest

import oracle_api as O
from adjoint_model import SubstepModel, loss_grad_vy2, loss_vy2
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
