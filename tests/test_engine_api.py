"""The reference-facing API (ffengine_gb300.FluidSimulation over the C ABI) on the GPU:
lifecycle, error convention, particle I/O and a multi-frame trajectory against the
reference engine's golden trajectory."""
import numpy as np
import pytest

import ffengine_gb300 as ffe
from conftest import golden_path

pytestmark = pytest.mark.gpu


def make(n, pos, vel):
    sim = ffe.FluidSimulation(n, n, n, 1.0 / n)
    sim.enable_console_output = False
    sim.enable_surface_reconstruction = False
    sim.set_velocity_transfer_method_FLIP()
    sim.PICFLIP_ratio = 0.05
    sim.CFL_condition_number = 5
    sim.min_time_steps_per_frame = 1
    sim.max_time_steps_per_frame = 1
    sim.enable_extreme_velocity_removal = False
    sim.add_body_force(0.0, -9.81, 0.0)
    sim.load_marker_particle_data(pos.shape[0], pos.tobytes(), vel.tobytes())
    sim.initialize()
    return sim


def test_update_before_initialize_raises():
    sim = ffe.FluidSimulation(8, 8, 8, 0.125)
    with pytest.raises(RuntimeError, match="must be initialized"):
        sim.update(1 / 240)


def test_negative_dt_raises():
    sim = ffe.FluidSimulation(8, 8, 8, 0.125)
    sim.initialize()
    with pytest.raises(RuntimeError, match="delta time"):
        sim.update(-1.0)


def test_bad_dimensions_raise():
    with pytest.raises(RuntimeError):
        ffe.FluidSimulation(0, 8, 8, 0.125)


def test_empty_simulation_updates():
    sim = ffe.FluidSimulation(8, 8, 8, 0.125)
    sim.initialize()
    sim.update(1 / 240)
    assert sim.get_num_marker_particles() == 0
    assert sim.get_current_frame() == 1


def test_particles_outside_domain_dropped_on_load():
    pos = np.array([[0.5, 0.5, 0.5], [1.5, 0.5, 0.5], [-0.1, 0.2, 0.2]], np.float32)
    sim = make(8, pos, np.zeros_like(pos))
    assert sim.get_num_marker_particles() == 1


def test_trajectory_through_api_matches_reference():
    d = np.load(golden_path("traj16"))
    n = int(d["n"])
    sim = make(n, d["in_pos"], d["in_vel"])
    for s in range(d["traj_stats"].shape[0]):
        sim.update(float(d["dt"]))
        st = sim.get_frame_stats_data()
        assert st.substeps == 1 and st.pressureSolverSuccess == 1
        assert abs(st.pressureSolverIterations - int(d["traj_stats"][s, 1])) <= 1
        assert sim.get_num_marker_particles() == int(d["traj_moments"][s, 0])
    pos = np.frombuffer(sim.get_marker_particle_position_data(), np.float32).reshape(-1, 3)
    vel = np.frombuffer(sim.get_marker_particle_velocity_data(), np.float32).reshape(-1, 3)
    assert np.abs(pos - d["final_pos"]).max() < 1e-4
    assert np.abs(vel - d["final_vel"]).max() < 1e-2
    r = np.frombuffer(sim.get_marker_particle_position_data_range(10, 20), np.float32).reshape(-1, 3)
    assert np.array_equal(r, pos[10:20])


def test_cfl_substepping_and_stats():
    d = np.load(golden_path("rand20"))
    n = int(d["n"])
    sim = make(n, d["in_pos"], d["in_vel"] * 20)
    sim.max_time_steps_per_frame = 6
    sim.update(1 / 24)
    st = sim.get_frame_stats_data()
    assert 1 <= st.substeps <= 6
    assert st.fluidParticles == sim.get_num_marker_particles()
    assert sim.get_kernel_launch_count() > 0


def test_mixed_solver_mode_runs():
    d = np.load(golden_path("dam20"))
    n = int(d["n"])
    sim = make(n, d["in_pos"], d["in_vel"])
    sim.set_pressure_solver_mode(1)
    sim.set_pressure_solver_tolerance(1e-6)
    sim.update(float(d["dt"]))
    s = sim.get_pressure_solver_stats()
    assert s["success"] == 1 and s["rel_residual"] <= 1e-6
