"""GPU parity on the drop-in's own call, FluidSimulation_update, at the configured sizes and on
the engine's default paths, against the reference engine's golden vectors:

  classification  -- the pressure cells and their k-j-i order (the reference's compact index)
                     bit-exact on the stage fixtures;
  extreme-velocity removal (on by default) -- speed limit and kept particles bit-exact on the
                     reference's own post-transfer input; a 20-substep trajectory with the rule
                     on keeps the reference's particle count at every substep;
  CFL substepping -- per frame the reference's substep count, substep lengths (the last one
                     exactly, the others to the 6 digits the engine logs) and particle count;
  the 64^3 dam break (100 substeps of 1/240 s) -- per substep the particle count, the pressure
                     iterations within 1 and the mean position / velocity; the final positions;
  the 128^3 dam break (200 substeps, mixed-precision PCG to 1e-6) -- every solve against an
                     FP64 reference solve of the same system to 1e-12: pressure and velocity
                     relative L2 and the largest weighted divergence after the projection.
"""
import numpy as np
import pytest

import ffengine_gb300 as ffe
import gpu_api as G
import oracle_api as O
from conftest import golden_path
from ffengine_gb300 import scenes

pytestmark = pytest.mark.gpu


def bits_equal(a, b):
    a = np.ascontiguousarray(a); b = np.ascontiguousarray(b)
    return a.shape == b.shape and np.array_equal(a.view(np.uint32), b.view(np.uint32))


def make(d, evr=False):
    n = int(d["n"])
    sim = ffe.FluidSimulation(n, n, n, 1.0 / n)
    sim.enable_console_output = False
    sim.enable_surface_reconstruction = False
    sim.set_velocity_transfer_method_FLIP()
    sim.PICFLIP_ratio = float(d["pic"])
    sim.CFL_condition_number = int(d["cfl"])
    sim.max_time_steps_per_frame = int(d["max_steps"]) if "max_steps" in d else 1
    sim.min_time_steps_per_frame = int(d["min_steps"]) if "min_steps" in d else 1
    sim.enable_extreme_velocity_removal = evr
    sim.add_body_force(0.0, -9.81, 0.0)
    pos, vel = d["in_pos"], d["in_vel"]
    sim.load_marker_particle_data(pos.shape[0], pos.tobytes(), vel.tobytes())
    sim.initialize()
    if int(d["has_sphere"]):
        sim.set_solid_level_set(np.ascontiguousarray(d["solid_phi"], np.float32).tobytes())
    return sim


def state(sim):
    x = np.frombuffer(sim.get_marker_particle_position_data(), np.float32).reshape(-1, 3)
    v = np.frombuffer(sim.get_marker_particle_velocity_data(), np.float32).reshape(-1, 3)
    return x, v


@pytest.mark.parametrize("name", ["dam20", "rand20", "sphere24"])
def test_classification_bitexact(name):
    d = np.load(golden_path(name))
    phi = d["liquid_phi"]
    fluid, bbox = G.classify(phi)
    interior = np.zeros(phi.shape, bool)
    interior[1:-1, 1:-1, 1:-1] = True
    want = (phi < 0) & interior
    assert np.array_equal(fluid.astype(bool), want)
    # the compact index: pressure cells numbered in k-j-i order, as the oracle's (pinned) system rows
    n, dx, dt = int(d["n"]), float(d["dx"]), float(d["dt"])
    rows, _, _ = O.pressure_system(n, dx, dt, phi, O.face_weights(n, d["solid_phi"]),
                                   [d["body_" + c] for c in "uvw"], dense=False)
    kk, jj, ii = np.nonzero(fluid)
    assert np.array_equal(np.stack([ii, jj, kk], 1), rows)
    assert bbox.tolist() == [ii.min(), jj.min(), kk.min(), ii.max(), jj.max(), kk.max()]


def test_classification_empty():
    fluid, bbox = G.classify(np.full((6, 7, 8), 0.1, np.float32))
    assert fluid.sum() == 0 and bbox[3] == -1


def test_extreme_velocity_removal_bitexact():
    d = np.load(golden_path("evr20"))
    n, dx = int(d["n"]), float(d["dx"])
    p1, v1, limit = G.remove_extreme(n, dx, d["adv_pos"], d["g2p_vel"], d["solid_phi"], float(d["dt"]),
                                     int(d["cfl"]), int(d["max_steps"]))
    assert np.float32(limit) == d["speed_limit"][0]
    assert bits_equal(p1, d["p1_pos"]) and bits_equal(v1, d["p1_vel"])


def test_extreme_velocity_removal_trajectory_through_update():
    d = dict(np.load(golden_path("evrtraj16")))
    sim = make(d, evr=True)
    for s in range(d["traj_stats"].shape[0]):
        sim.update(float(d["dt"]))
        st = sim.get_frame_stats_data()
        assert st.fluidParticles == int(d["traj_stats"][s, 0]), s
        assert abs(st.pressureSolverIterations - int(d["traj_stats"][s, 1])) <= 1
    x, v = state(sim)
    assert np.abs(x - d["final_pos"]).max() < 1e-4
    assert np.abs(v - d["final_vel"]).max() < 1e-2


@pytest.mark.parametrize("name", ["cfltraj16", "cflmaxtraj16", "cflmin20"])
def test_cfl_substepping_through_update(name):
    d = dict(np.load(golden_path(name)))
    sim = make(d)
    logged = d["traj_dts"]
    at = 0
    for f in range(d["traj_stats"].shape[0]):
        sim.update(float(d["dt"]))
        st = sim.get_frame_stats_data()
        dts = sim.get_frame_substep_times()
        assert st.substeps == len(dts) == int(d["traj_steps"][f, 0]), f
        assert abs(dts[-1] - d["traj_steps"][f, 1]) <= 1e-15
        for t in dts:
            assert float("%g" % t) == logged[at]
            at += 1
        assert st.fluidParticles == int(d["traj_stats"][f, 0])
        assert abs(st.pressureSolverIterations - int(d["traj_stats"][f, 1])) <= 1
        # frames of 1/6 s and 1/8 s on a 16^3 / 20^3 grid move particles several cells per
        # substep, so the FP32 sampling's rounding separates the trajectories faster than at 1/240 s:
        # the mean position stays within a tenth of a cell of the reference's
        m = d["traj_moments"][f]
        x, v = state(sim)
        assert np.abs(x.astype(np.float64).mean(0) - m[1:4]).max() < 0.1 * float(d["dx"])
        assert np.abs(v.astype(np.float64).mean(0) - m[4:7]).max() < 5e-2
    assert at == logged.size


def test_dam_break_64_100_substeps_through_update():
    """The 64^3 dam break (block x < 0.4, y < 0.6, 8 particles per cell, 100 substeps of 1/240 s)
    against the reference engine's own trajectory, loaded through load_marker_particle_data (which
    hands the 503,291-particle batch over in the reference's load-queue order).  The transfer and sampling round differently
    (FP32 sampling where the reference samples in double), so the trajectories separate slowly;
    the drift of the mean position and velocity is printed per substep."""
    d = dict(np.load(golden_path("traj64")))
    sim = make(d)
    drift = []
    iter_exact = 0
    iter_diffs = []
    for s in range(d["traj_stats"].shape[0]):
        sim.update(float(d["dt"]))
        st = sim.get_frame_stats_data()
        m = d["traj_moments"][s]
        assert st.fluidParticles == int(m[0]), s
        assert st.pressureSolverSuccess == 1
        # the FP32 sampling's rounding slowly separates the states, which moves the FP64 solve's
        # iteration count (tolerance 1e-9) by a few near the stopping threshold
        di = abs(st.pressureSolverIterations - int(d["traj_stats"][s, 1]))
        assert di <= 8, (s, di)
        iter_exact += di <= 1
        iter_diffs.append(di)
        x, v = state(sim)
        dp = np.abs(x.astype(np.float64).mean(0) - m[1:4]).max()
        dv = np.abs(v.astype(np.float64).mean(0) - m[4:7]).max()
        drift.append((dp, dv))
        # mean speed reaches ~1 m/s; the mean velocity drifts chaotically by about 1e-3 m/s by the
        # last substeps
        assert dp < 1e-4 and dv < 5e-3, (s, dp, dv)
    print("64^3 drift of mean position / velocity every 10 substeps:",
          ["%.1e/%.1e" % dv for dv in drift[9::10]], "; iterations within 1 of the reference's at",
          iter_exact, "of 100 substeps; largest difference", max(iter_diffs))
    assert iter_exact >= 75
    x, v = state(sim)
    k = int(d["final_stride"])
    # after 100 substeps a few splashing particles have separated (measured: median 3.5e-6, 99th
    # percentile 1.8e-3, largest 4.3e-2 of the unit domain)
    sep = np.abs(x[::k] - d["final_pos"]).max(axis=1)
    print("final position separation: median %.1e, 99%% %.1e, max %.1e" %
          (np.median(sep), np.quantile(sep, 0.99), sep.max()))
    assert np.median(sep) < 1e-4 and np.quantile(sep, 0.99) < 1e-2 and sep.max() < 0.1


def test_dam_break_128_mixed_solves_vs_fp64_reference():
    """The 128^3 dam break (4.0M particles), 200 substeps with the mixed-precision PCG to 1e-6,
    every solve checked against the FP64 PCG on the same system to 1e-12.  The FP64-checked
    residual of the mixed solve is at most 1e-6 of ||b||_inf; the projected field's largest
    weighted divergence is at most the reference-projected field's plus twice that tolerance (the
    residual, and the rounding of the float velocities the projection writes)."""
    n = 128
    pos, vel = scenes.dam_break_particles(n, 0.4, 0.6, seed=0)
    sim = ffe.FluidSimulation(n, n, n, 1.0 / n)
    sim.max_time_steps_per_frame = 1
    sim.enable_extreme_velocity_removal = False
    sim.add_body_force(0.0, -9.81, 0.0)
    sim.load_marker_particle_data(pos.shape[0], pos.tobytes(), vel.tobytes())
    sim.initialize()
    sim.set_pressure_solver_mode(1)
    sim.set_pressure_solver_tolerance(1e-6)
    sim.set_solve_check(1e-12)
    worst = dict(p=0.0, u=0.0, div=0.0)
    for s in range(200):
        sim.update(1.0 / 240.0)
        ps = sim.get_pressure_solver_stats()
        c = sim.get_solve_check()
        assert ps["success"] == 1 and ps["rel_residual"] <= 1e-6, (s, ps)
        assert c["valid"] == 1 and c["ref_rel_residual"] <= 1e-12, (s, c)
        assert c["p_rel_l2"] < 1e-3 and c["u_rel_l2"] < 1e-4, (s, c)
        # the solver's residual bounds the extra divergence (1e-6 of ||b||_inf); the float
        # velocities the projection writes add their rounding on top
        assert c["div_rel"] <= c["div_ref_rel"] + 2e-6, (s, c)
        worst = dict(p=max(worst["p"], c["p_rel_l2"]), u=max(worst["u"], c["u_rel_l2"]),
                     div=max(worst["div"], c["div_rel"]))
    print("128^3 worst over 200 substeps: pressure rel-L2 %.2e, velocity rel-L2 %.2e, max divergence / |b| %.2e"
          % (worst["p"], worst["u"], worst["div"]))


def test_mixed_warm_start():
    """The mixed solve started from the previous substep's pressure (1), or from the linear
    extrapolation of the last two (2), meets the same FP64-checked tolerance as the zero start,
    with fewer iterations, and the trajectories stay together."""
    n = 64
    pos, vel = scenes.dam_break_particles(n, 0.4, 0.6, seed=0)
    out = {}
    for warm in (0, 1, 2):
        sim = ffe.FluidSimulation(n, n, n, 1.0 / n)
        sim.max_time_steps_per_frame = 1
        sim.enable_extreme_velocity_removal = False
        sim.add_body_force(0.0, -9.81, 0.0)
        sim.set_pressure_solver_mode(1)
        sim.set_pressure_solver_tolerance(1e-6)
        sim.set_pressure_warm_start(warm)
        sim.load_marker_particle_data(pos.shape[0], pos.tobytes(), vel.tobytes())
        sim.initialize()
        its = []
        for _ in range(8):
            sim.update(1.0 / 240)
            s = sim.get_pressure_solver_stats()
            assert s["success"] and s["rel_residual"] <= 1e-6
            its.append(int(s["iterations"]))
        out[warm] = (its, state(sim))
    print("iterations per substep:", {k: v[0] for k, v in out.items()})
    assert out[0][0][0] == out[1][0][0] == out[2][0][0]   # the first substep has no previous pressure
    assert out[1][0][1] == out[2][0][1]                    # the second has one: both start from it
    assert sum(out[1][0][1:]) < 0.9 * sum(out[0][0][1:]), out
    assert sum(out[2][0][1:]) < 0.9 * sum(out[0][0][1:]), out
    x0 = out[0][1][0]
    for warm in (1, 2):
        x1 = out[warm][1][0]
        assert x0.shape == x1.shape and np.abs(x0 - x1).max() < 1e-4


def test_mixed_solve_graph_replay_bit_identical():
    """The mixed solve's batches replayed from a graph captured once per solve give the same
    substeps bit for bit as launching every kernel (the sweeps take fresh tags from the device
    counter on every replay), on a box of several wavefront tiles and over several substeps."""
    n = 64
    pos, vel = scenes.dam_break_particles(n, 0.4, 0.6, seed=3, velocity_sigma=0.3)
    out = []
    for graphs in (False, True):
        sim = ffe.FluidSimulation(n, n, n, 1.0 / n)
        sim.max_time_steps_per_frame = 1
        sim.enable_extreme_velocity_removal = False
        sim.add_body_force(0.0, -9.81, 0.0)
        sim.set_pressure_solver_mode(1)
        sim.set_pressure_solver_tolerance(1e-6)
        sim.set_pcg_graphs(graphs)
        sim.load_marker_particle_data(pos.shape[0], pos.tobytes(), vel.tobytes())
        sim.initialize()
        its = []
        for _ in range(6):
            sim.update(1.0 / 240)
            s = sim.get_pressure_solver_stats()
            assert s["success"]
            its.append(int(s["iterations"]))
        out.append((its, state(sim)))
    assert out[0][0] == out[1][0] and max(out[0][0]) > 8   # more than one batch per solve
    for a, b in zip(out[0][1], out[1][1]):
        assert a.shape == b.shape and np.array_equal(a.view(np.uint32), b.view(np.uint32))
