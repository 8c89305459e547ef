"""GPU parity of the surface tension path: the curvature grid (ParticleLevelSet::calculateCurvatureGrid,
particlelevelset.cpp:196-291), the cluster status (pressuresolver.cpp:314-605) and the tension term in
the pressure system and the pressure application (pressuresolver.cpp:659-749, 1047-1205), against the
reference engine's golden vectors and the CPU oracle.

Bars:
  curvature grid (surface level set and curvature)  -- bit-exact;
  cluster status on surface cells                   -- equal to the oracle's sequential search;
  FP64 pressure solve with the tension term         -- the reference's iteration count, within
                                                        1e-6 of max|p| (order of the FP64 sums);
  projection with the tension term                  -- bit-exact;
  substep through FluidSimulation::update           -- counts equal, positions within 5e-6,
                                                        velocities within 2e-4 of max|v|;
  trajectory (20 substeps)                          -- counts, pressure iterations (+-1), moments
                                                        within the bounds the oracle itself meets.
"""
import numpy as np
import pytest

import gpu_api as G
import oracle_api as O
from conftest import golden_path

pytestmark = pytest.mark.gpu


def bits_equal(a, b):
    a = np.ascontiguousarray(a); b = np.ascontiguousarray(b)
    return a.shape == b.shape and np.array_equal(a.view(np.uint32), b.view(np.uint32))


@pytest.mark.parametrize("name", ["curv20", "curvsphere24", "tension20", "tensionsphere24"])
def test_curvature_grid_bitexact(name):
    d = dict(np.load(golden_path(name)))
    n, dx = int(d["n"]), float(d["dx"])
    surf, k = G.curvature_grid(n, dx, d["liquid_phi"])
    assert bits_equal(surf, d["surface_phi"])
    assert bits_equal(k, d["curvature"])


def test_curvature_grid_random_vs_oracle():
    """Level sets with many small droplets (large curvature, bands of several blocks) and one
    that never comes near the surface (empty band: node (0, 0, 0) is then not updated)."""
    nd = pytest.importorskip("scipy.ndimage")
    rng = np.random.default_rng(7)
    for n, sigma, q in ((24, 1.2, 0.4), (30, 2.0, 0.6), (17, 1.5, 0.5)):
        dx = 1.0 / n
        phi = nd.gaussian_filter(rng.standard_normal((n, n, n)), sigma).astype(np.float32)
        phi = ((phi - np.float32(np.quantile(phi, q))) * np.float32(8 * dx)).astype(np.float32)
        gs, gk = G.curvature_grid(n, dx, phi)
        os_, ok = O.curvature_grid(n, dx, phi)
        assert bits_equal(gs, os_) and bits_equal(gk, ok), n
    far = np.full((12, 12, 12), 0.9, np.float32)
    gs, gk = G.curvature_grid(12, 1 / 12, far)
    os_, ok = O.curvature_grid(12, 1 / 12, far)
    assert bits_equal(gs, os_) and bits_equal(gk, ok)


def _surface_cells(phi):
    sign = phi < 0
    diff = np.zeros(phi.shape, bool)
    for ax in range(3):
        for sh in (1, -1):
            diff |= sign != np.roll(sign, sh, axis=ax)
    inner = np.zeros(phi.shape, bool)
    inner[1:-1, 1:-1, 1:-1] = True
    return diff & inner


@pytest.mark.parametrize("trial", range(5))
def test_cluster_status_vs_oracle(trial):
    import ctypes
    nd = pytest.importorskip("scipy.ndimage")
    rng = np.random.default_rng(100 + trial)
    n = 20 + 2 * trial + (trial % 2)   # odd sizes leave partial 4^3 blocks
    phi = nd.gaussian_filter(rng.standard_normal((n, n, n)), 0.8 + 0.3 * trial).astype(np.float32)
    phi -= np.float32(np.quantile(phi, 0.3 + 0.1 * trial))
    phi = np.ascontiguousarray(phi)
    seq = np.zeros(phi.shape, np.int8)
    O.lib().oracle_cluster_status(n, n, n, O._p(phi), seq.ctypes.data_as(ctypes.c_void_p))
    seq = seq.view(np.uint8)
    gpu = G.cluster_status(phi)
    # classified before the search (border, pure blocks): identical everywhere
    pre = (seq == 16) | (gpu == 16)
    assert np.array_equal(seq[pre], gpu[pre])
    # the statuses the tension term reads: every surface cell
    surf = _surface_cells(phi)
    assert np.array_equal(seq[surf], gpu[surf])
    if trial < 2:
        assert ((gpu[surf] == 4) | (gpu[surf] == 8)).any()


@pytest.mark.parametrize("name", ["tension20", "tensionsphere24"])
def test_pressure_with_tension_fp64(name):
    d = dict(np.load(golden_path(name)))
    n, dx, dt = int(d["n"]), float(d["dx"]), float(d["dt"])
    w = O.face_weights(n, d["solid_phi"])
    body = [d["body_" + c] for c in "uvw"]
    pr, p64, st = G.pressure_solve_tension(n, dx, dt, d["liquid_phi"], w, body, d["curvature"],
                                           float(d["surface_tension"]), tol=1e-9, mode=0)
    assert st["success"]
    assert st["iters"] == int(d["pressure_iters"][0])
    ref = d["pressure"]
    assert np.abs(pr - ref).max() <= 1e-6 * np.abs(ref).max()
    # mixed precision reaches the same tolerance on the tensioned system
    pm, pm64, sm = G.pressure_solve_tension(n, dx, dt, d["liquid_phi"], w, body, d["curvature"],
                                            float(d["surface_tension"]), tol=1e-9, mode=1)
    assert sm["success"]
    assert np.abs(pm - ref).max() <= 1e-5 * np.abs(ref).max()


@pytest.mark.parametrize("name", ["tension20", "tensionsphere24"])
def test_projection_with_tension_bitexact(name):
    d = dict(np.load(golden_path(name)))
    n, dx, dt = int(d["n"]), float(d["dx"]), float(d["dt"])
    w = O.face_weights(n, d["solid_phi"])
    (u, v, ww), valid = G.apply_pressure_tension(n, dx, dt, d["liquid_phi"], w, d["pressure"],
                                                 [d["body_" + c] for c in "uvw"], d["curvature"],
                                                 float(d["surface_tension"]))
    for c, a, vv in zip("uvw", (u, v, ww), valid):
        assert bits_equal(a, d["proj_" + c]), c
        assert np.array_equal(vv, d["proj_valid" + c]), c


def _sim(d, tension):
    import ffengine_gb300 as ffe
    n = int(d["n"])
    sim = ffe.FluidSimulation(n, n, n, 1.0 / n)
    sim.enable_extreme_velocity_removal = False
    sim.add_body_force(0.0, -9.81, 0.0)
    sim.surface_tension = tension
    pos, vel = d["in_pos"], d["in_vel"]
    sim.load_marker_particle_data(pos.shape[0], pos.tobytes(), vel.tobytes())
    sim.initialize()
    sim.set_solid_level_set(np.ascontiguousarray(d["solid_phi"], np.float32).tobytes())
    return sim


def _state(sim):
    x = np.frombuffer(sim.get_marker_particle_position_data(), np.float32).reshape(-1, 3)
    v = np.frombuffer(sim.get_marker_particle_velocity_data(), np.float32).reshape(-1, 3)
    return x, v


@pytest.mark.parametrize("name", ["tension20", "tensionsphere24"])
def test_tension_substep_vs_reference(name):
    d = dict(np.load(golden_path(name)))
    sim = _sim(d, float(d["surface_tension"]))
    sim.update(float(d["dt"]))
    st = sim.get_frame_stats_data()
    assert st.substeps == 1
    assert abs(st.pressureSolverIterations - int(d["pressure_iters"][0])) <= 1
    x, v = _state(sim)
    assert x.shape == d["p1_pos"].shape
    assert np.abs(x - d["p1_pos"]).max() <= 5e-6
    assert np.abs(v - d["p1_vel"]).max() <= 2e-4 * max(np.abs(d["p1_vel"]).max(), 1.0)
    # the term is active: without it the velocities differ
    plain = _sim(d, 0.0)
    plain.update(float(d["dt"]))
    assert np.abs(_state(plain)[1] - d["p1_vel"]).max() > 2e-4 * max(np.abs(d["p1_vel"]).max(), 1.0)


def test_tension_trajectory_vs_reference():
    """20 substeps of FluidSimulation::update with surface tension; the reference trajectory's own
    curvature carries worker-thread noise (the oracle test of the same fixture says how), so the
    bounds are those the oracle meets."""
    d = dict(np.load(golden_path("tensiontraj16")))
    sim = _sim(d, float(d["surface_tension"]))
    for s in range(d["traj_stats"].shape[0]):
        sim.update(float(d["dt"]))
        m = d["traj_moments"][s]
        x, v = _state(sim)
        assert x.shape[0] == int(d["traj_stats"][s, 0]), s
        assert abs(sim.get_frame_stats_data().pressureSolverIterations - int(d["traj_stats"][s, 1])) <= 1, s
        assert np.abs(x.astype(np.float64).mean(0) - m[1:4]).max() < 1e-3
        assert np.abs(v.astype(np.float64).mean(0) - m[4:7]).max() < 2e-2


def test_tension_timestep_restriction():
    """FluidSimulation::_calculateNextTimeStep (fluidsimulation.cpp:10236-10256): with surface tension
    the substep is at most condition_number * sqrt(dx^3) * sqrt(1 / (k + 1e-6)), until the frame's
    last allowed substep takes the time left (raised to 40 here so that it does not)."""
    d = dict(np.load(golden_path("tensiontraj16")))
    k, cond = 200.0, 5.0
    sim = _sim(d, k)
    sim.surface_tension_condition_number = cond
    sim.max_time_steps_per_frame = 40
    frame = 1.0 / 30
    sim.update(frame)
    dx = 1.0 / int(d["n"])
    limit = cond * np.sqrt(dx ** 3) * np.sqrt(1.0 / (k + 1e-6))
    dts = sim.get_frame_substep_times()
    assert len(dts) >= int(np.floor(frame / limit))
    assert max(dts) <= limit * (1 + 1e-12)
    assert abs(sum(dts) - frame) < 1e-9


def test_tension_setters():
    import ffengine_gb300 as ffe
    sim = ffe.FluidSimulation(8, 8, 8, 1 / 8)
    assert sim.surface_tension == 0.0 and sim.surface_tension_condition_number == 10.0
    sim.surface_tension = 0.25
    sim.surface_tension_condition_number = 4.0
    assert sim.surface_tension == 0.25 and sim.surface_tension_condition_number == 4.0
    with pytest.raises(RuntimeError, match="surface tension must be greater"):
        sim.surface_tension = -1.0
    with pytest.raises(RuntimeError, match="condition number must be greater"):
        sim.surface_tension_condition_number = 0.0


def test_differentiable_substep_rejects_tension():
    import ffengine_gb300 as ffe
    sim = ffe.FluidSimulation(8, 8, 8, 1 / 8)
    sim.surface_tension = 0.5
    p = np.full((4, 3), 0.5, np.float32)
    sim.load_marker_particle_data(4, p.tobytes(), p.tobytes())
    sim.initialize()
    with pytest.raises(RuntimeError, match="surface tension"):
        sim.substep_differentiable(1 / 240)
