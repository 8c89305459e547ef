"""Checkpointed rollout adjoint on the GPU (positions and velocities), checked against the
FP64 rollout model (tests/adjoint_model.py) anchored to the oracle's trajectory: its
transpose, and FP64 central differences (eps = 1e-6) along random directions.  The forward
is checked against the oracle (reference arithmetic).  Anchoring matters because FP32 kernel
weights near the kernel radius make the reference-arithmetic trajectory drift from an FP64
one at a few free-surface faces; the GPU linearises along the former.  The scene is a
floating fluid block whose particles stay clear of every wall, so that no particle is moved
by collision handling."""
import numpy as np
import pytest

import ffengine_gb300 as ffe
import oracle_api as O
from adjoint_model import RolloutModel, loss_grad_vy2
from ffengine_gb300 import scenes

pytestmark = pytest.mark.gpu
DT = 1 / 240


def make_sim(n, pos, vel, mode=0, tol=1e-12):
    sim = ffe.FluidSimulation(n, n, n, 1.0 / n)
    sim.PICFLIP_ratio = 0.05
    sim.CFL_condition_number = 5
    sim.enable_extreme_velocity_removal = False
    sim.add_body_force(0.0, -9.81, 0.0)
    sim.set_pressure_solver_mode(mode)
    sim.set_pressure_solver_tolerance(tol)
    sim.set_adjoint_tolerance(tol)
    sim.load_marker_particle_data(pos.shape[0], pos.tobytes(), vel.tobytes())
    sim.initialize()
    return sim


def state(sim):
    x = np.frombuffer(sim.get_marker_particle_position_data(), np.float32).reshape(-1, 3).copy()
    v = np.frombuffer(sim.get_marker_particle_velocity_data(), np.float32).reshape(-1, 3).copy()
    return x, v


def rel(a, b):
    return np.linalg.norm(np.asarray(a, np.float64) - b) / np.linalg.norm(b)


def oracle_trajectory(n, pos, vel, k):
    """k substeps of the oracle (reference arithmetic); no particle of the test scenes is removed,
    so this is the differentiable substep's map."""
    solid = O.solid_phi(n, 1.0 / n)
    states = [(pos, vel)]
    x, v = pos, vel
    for _ in range(k):
        x, v, _ = O.substep(n, 1.0 / n, DT, 0.05, 5, (0.0, -9.81, 0.0), solid, x, v, tol=1e-12)
        assert x.shape == pos.shape
        states.append((x, v))
    return states


def anchored_model(n, pos, vel, k):
    states = oracle_trajectory(n, pos, vel, k)
    return RolloutModel(n, pos, vel, O.solid_phi(n, 1.0 / n), k, anchors=states, dt=DT), states


@pytest.fixture(scope="module", params=[(16, 1), (16, 3), (32, 2)], ids=["16x1", "16x3", "32x2"])
def rollout(request):
    n, k = request.param
    pos, vel = scenes.floating_block_particles(n, seed=3, velocity_sigma=0.5)
    sim = make_sim(n, pos, vel)
    sim.rollout_forward(k, DT)
    xk, vk = state(sim)
    rng = np.random.default_rng(11)
    cx = rng.standard_normal(pos.shape).astype(np.float32)
    cv = rng.standard_normal(pos.shape).astype(np.float32)
    gx0, gv0, cnt = sim.rollout_adjoint(cx, cv)
    model, states = anchored_model(n, pos, vel, k)
    return dict(n=n, k=k, pos=pos, vel=vel, sim=sim, xk=xk, vk=vk, cx=cx, cv=cv, gx0=gx0, gv0=gv0, cnt=cnt,
                model=model, oracle=states[-1], after=state(sim))


def test_rollout_forward_matches_oracle(rollout):
    x, v = rollout["oracle"]
    assert np.abs(rollout["xk"] - x).max() <= 1e-5
    assert np.abs(rollout["vk"] - v).max() <= 1e-4 * np.abs(v).max()


def test_rollout_adjoint_leaves_final_state(rollout):
    x, v = rollout["after"]
    assert np.array_equal(x, rollout["xk"]) and np.array_equal(v, rollout["vk"])
    assert rollout["cnt"] == -1


def test_rollout_adjoint_matches_fp64_transpose(rollout):
    gxm, gvm = rollout["model"].vjp(rollout["cx"], rollout["cv"])
    assert rel(rollout["gv0"], gvm) <= 2e-3
    assert rel(rollout["gx0"], gxm) <= 2e-3


def test_rollout_adjoint_vs_central_differences(rollout):
    m, n = rollout["model"], rollout["n"]
    x0, v0 = rollout["pos"].astype(np.float64), rollout["vel"].astype(np.float64)
    cx, cv = rollout["cx"].astype(np.float64), rollout["cv"].astype(np.float64)
    gx, gv = rollout["gx0"].astype(np.float64), rollout["gv0"].astype(np.float64)
    rng = np.random.default_rng(1234)
    eps = 1e-6
    errs = []
    for _ in range(12):
        dxp, dvp = rng.standard_normal(x0.shape) / n, rng.standard_normal(v0.shape)
        xp, vp = m.forward(x0 + eps * dxp, v0 + eps * dvp)
        xm, vm = m.forward(x0 - eps * dxp, v0 - eps * dvp)
        fd = ((cx * (xp - xm)).sum() + (cv * (vp - vm)).sum()) / (2 * eps)
        errs.append(abs(fd - (gx * dxp).sum() - (gv * dvp).sum()) / abs(fd))
    assert np.median(errs) < 1e-3 and max(errs) < 1e-2


def test_rollout_builtin_loss(rollout):
    sim, m = rollout["sim"], rollout["model"]
    gx0, gv0, cnt = sim.rollout_adjoint(None, None, 0.5)
    mask = rollout["xk"][:, 1].astype(np.float64) > 0.5
    assert cnt == int(mask.sum()) > 0
    gxm, gvm = m.vjp(np.zeros_like(m.xk), loss_grad_vy2(m.vk, mask))
    assert rel(gv0, gvm) <= 2e-3 and rel(gx0, gxm) <= 2e-3


def test_single_substep_adjoint_agrees_with_rollout():
    n = 16
    pos, vel = scenes.floating_block_particles(n, seed=4, velocity_sigma=0.5)
    sim = make_sim(n, pos, vel)
    sim.rollout_forward(1, DT)
    g = np.random.default_rng(3).standard_normal(pos.shape).astype(np.float32)
    _, gv_roll, _ = sim.rollout_adjoint(None, g)
    sim2 = make_sim(n, pos, vel)
    sim2.substep_differentiable(DT)
    gv_one, _ = sim2.adjoint(g)
    assert np.array_equal(gv_roll, gv_one)


def test_torch_autograd_function_matches_model():
    torch = pytest.importorskip("torch")
    from torch_rollout import FlipRollout
    n, k = 16, 2
    pos, vel = scenes.floating_block_particles(n, seed=5, velocity_sigma=0.5)
    sim = make_sim(n, pos, vel)
    x0 = torch.tensor(pos, requires_grad=True)
    v0 = torch.tensor(vel, requires_grad=True)
    xk, vk = FlipRollout.apply(x0, v0, sim, k, DT)
    rng = np.random.default_rng(9)
    cx = torch.tensor(rng.standard_normal(pos.shape), dtype=torch.float32)
    cv = torch.tensor(rng.standard_normal(pos.shape), dtype=torch.float32)
    ((cx * xk).sum() + (cv * vk).sum()).backward()
    gxm, gvm = anchored_model(n, pos, vel, k)[0].vjp(cx.numpy(), cv.numpy())
    assert rel(x0.grad.numpy(), gxm) <= 2e-3 and rel(v0.grad.numpy(), gvm) <= 2e-3
