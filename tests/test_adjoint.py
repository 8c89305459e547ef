"""Adjoint of one substep on the GPU, checked against an FP64 model of the same affine
velocity map (tests/adjoint_model.py): its transpose (sparse LU, or a dense solve on a
small grid) and FP64 central finite differences (eps = 1e-4) along 64 random directions.
Loss: mean of vy^2 over particles with y > 0.5 after the substep (membership frozen)."""
import numpy as np
import pytest

import ffengine_gb300 as ffe
import oracle_api as O
from adjoint_model import SubstepModel, loss_grad_vy2, loss_vy2
from ffengine_gb300 import scenes

pytestmark = pytest.mark.gpu
DT = 1 / 240


def gpu_run(n, pos, vel, mode=0, tol=1e-12):
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
    sim.substep_differentiable(DT)
    p1 = np.frombuffer(sim.get_marker_particle_position_data(), np.float32).reshape(-1, 3)
    v1 = np.frombuffer(sim.get_marker_particle_velocity_data(), np.float32).reshape(-1, 3)
    g0, cnt = sim.adjoint(None, 0.5)
    return p1, v1, g0, cnt


@pytest.fixture(scope="module", params=[(16, True), (48, False)], ids=["16_dense", "48_sparse"])
def setup(request):
    n, dense = request.param
    pos, vel = scenes.dam_break_particles(n, 0.4, 0.6, seed=0, velocity_sigma=0.5)
    solid = O.solid_phi(n, 1.0 / n)
    p1, v1, g0, cnt = gpu_run(n, pos, vel)
    # the engine holds the batch in the reference's load-queue order (212,336 particles at 48^3
    # exceed one fragment of that queue), so the model starts from the same state
    pos, vel = O.as_loaded(pos), O.as_loaded(vel)
    model = SubstepModel(n, pos, vel, solid, dt=DT, dense=dense)
    v1m = model.forward(vel)
    mask = p1[:, 1].astype(np.float64) > 0.5
    return dict(n=n, pos=pos, vel=vel, p1=p1, v1=v1, g0=g0, cnt=cnt, model=model, v1m=v1m, mask=mask)


def test_forward_matches_fp64_model(setup):
    v1, v1m = setup["v1"], setup["v1m"]
    assert setup["cnt"] == int(setup["mask"].sum()) > 0
    assert np.abs(v1 - v1m).max() <= 1e-4 * np.abs(v1m).max()


def test_adjoint_matches_fp64_transpose(setup):
    m = setup["model"]
    gref = m.vjp(loss_grad_vy2(setup["v1m"], setup["mask"]))
    g = setup["g0"].astype(np.float64)
    assert np.linalg.norm(g - gref) <= 1e-3 * np.linalg.norm(gref)


def test_adjoint_vs_central_differences(setup):
    m, vel, mask = setup["model"], setup["vel"].astype(np.float64), setup["mask"]
    rng = np.random.default_rng(1234)
    eps = 1e-4
    g = setup["g0"].astype(np.float64)
    errs = []
    for _ in range(64):
        d = rng.standard_normal(vel.shape)
        lp = loss_vy2(m.forward(vel + eps * d), mask)
        lm = loss_vy2(m.forward(vel - eps * d), mask)
        fd = (lp - lm) / (2 * eps)
        errs.append(abs(fd - (g * d).sum()) / max(abs(fd), 1e-12))
    assert np.median(errs) < 1e-3 and max(errs) < 1e-2


def test_adjoint_mixed_precision_close():
    n = 24
    pos, vel = scenes.dam_break_particles(n, 0.4, 0.6, seed=2, velocity_sigma=0.5)
    _, _, g64, _ = gpu_run(n, pos, vel, mode=0, tol=1e-10)
    _, _, g32, _ = gpu_run(n, pos, vel, mode=1, tol=1e-6)
    assert np.linalg.norm(g32 - g64) <= 1e-3 * np.linalg.norm(g64)


def test_adjoint_warm_start_close():
    """Mixed solver: the adjoint's solve starts from the last adjoint solution (with the forward's
    warm start on), and the forward's pressure chain is not disturbed by the adjoint solves: three
    rounds of substep + adjoint agree with the same rounds from zero starts to the solve's accuracy."""
    n = 24
    pos, vel = scenes.dam_break_particles(n, 0.4, 0.6, seed=2, velocity_sigma=0.5)
    out = {}
    for warm in (0, 2):
        sim = ffe.FluidSimulation(n, n, n, 1.0 / n)
        sim.PICFLIP_ratio = 0.05
        sim.CFL_condition_number = 5
        sim.enable_extreme_velocity_removal = False
        sim.add_body_force(0.0, -9.81, 0.0)
        sim.set_pressure_solver_mode(1)
        sim.set_pressure_solver_tolerance(1e-6)
        sim.set_adjoint_tolerance(1e-6)
        sim.set_pressure_warm_start(warm)
        sim.load_marker_particle_data(pos.shape[0], pos.tobytes(), vel.tobytes())
        sim.initialize()
        gs = []
        for _ in range(3):
            sim.substep_differentiable(DT)
            assert sim.get_pressure_solver_stats()["success"]
            g, cnt = sim.adjoint(None, 0.5)
            assert cnt > 0 and np.isfinite(g).all()
            gs.append(g)
        out[warm] = gs
    for a, b in zip(out[0], out[2]):
        assert np.linalg.norm(a - b) <= 1e-3 * np.linalg.norm(a)
