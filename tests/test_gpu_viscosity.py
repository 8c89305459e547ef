"""GPU parity of the viscosity solve (ViscositySolver, viscositysolver.cpp) against the
reference engine's golden vectors (viscosity mode) and the CPU oracle.

Bars:
  volumes, face -> row table, system (columns and values), rhs  -- bit-exact;
  MIC(0) factor (pivots and lower values)                          -- bit-exact;
  solve     -- the reference stops on |r|inf <= 1e-4 |b|inf with float dot products summed in
               order; the GPU sums them in FP64, so the iteration count may differ by a few.  The
               GPU solution meets the same stopping rule on the reference's own system (residual
               recomputed in FP64), and two solutions that both stop there lie within 1e-3 of
               max|v| of each other on these cases;
  substep   -- counts equal; positions within 5e-6, velocities within 2e-4 of max|v|;
  trajectory -- 20 substeps: counts, pressure iterations (+-1), moments.
"""
import numpy as np
import pytest

import gpu_api as G
import oracle_api as O
from conftest import golden_path

pytestmark = pytest.mark.gpu

CASES = ["visc20", "viscsphere24"]


def bits_equal(a, b):
    a = np.ascontiguousarray(a); b = np.ascontiguousarray(b)
    return a.shape == b.shape and np.array_equal(a.view(np.uint32), b.view(np.uint32))


@pytest.fixture(scope="module", params=CASES)
def case(request):
    d = dict(np.load(golden_path(request.param)))
    n, dx = int(d["n"]), float(d["dx"])
    d["gpu"] = G.viscosity(n, dx, float(d["dt"]), d["liquid_phi"], d["solid_phi"], float(d["viscosity"]),
                           [d["visc_in_" + c] for c in "uvw"], debug=True)
    return d


def test_viscosity_volumes_bitexact(case):
    _, st, dbg = case["gpu"]
    for g in ("center", "u", "v", "w", "eu", "ev", "ew"):
        assert bits_equal(dbg["vol"][g], case["visc_vol_" + g]), g
    assert np.array_equal(dbg["index"], case["visc_index"])
    assert st["n"] == int(case["visc_stats"][0])


def test_viscosity_system_bitexact(case):
    _, st, dbg = case["gpu"]
    assert np.array_equal(dbg["rowstart"], case["visc_rowstart"])
    assert np.array_equal(dbg["col"], case["visc_col"])
    assert bits_equal(dbg["val"], case["visc_val"]) and bits_equal(dbg["rhs"], case["visc_rhs"])


def test_viscosity_mic0_factor_bitexact(case):
    _, st, dbg = case["gpu"]
    assert np.array_equal(dbg["ic_colstart"], case["visc_ic_colstart"])
    assert np.array_equal(dbg["ic_rowindex"], case["visc_ic_rowindex"])
    assert bits_equal(dbg["ic_invdiag"], case["visc_ic_invdiag"])
    assert bits_equal(dbg["ic_value"], case["visc_ic_value"])


def test_viscosity_solve_vs_reference(case):
    (u, v, w), st, dbg = case["gpu"]
    assert st["success"]
    assert abs(st["iters"] - int(case["visc_stats"][1])) <= 3
    # the stopping rule, on the reference's system
    rs, col, val, rhs = case["visc_rowstart"], case["visc_col"], case["visc_val"], case["visc_rhs"]
    x = dbg["soln"].astype(np.float64)
    rows = np.repeat(np.arange(rs.size - 1), np.diff(rs.astype(np.int64)))
    ax = np.bincount(rows, weights=val.astype(np.float64) * x[col], minlength=rs.size - 1)
    res = np.abs(rhs.astype(np.float64) - ax).max()
    assert res <= 1e-4 * np.abs(rhs).max() * (1 + 1e-3) + 1e-7 * np.abs(rhs).max()
    ref = [case["visc_" + c] for c in "uvw"]
    scale = max(max(np.abs(a).max() for a in ref), 1e-30)
    for a, b in zip((u, v, w), ref):
        assert np.abs(a - b).max() <= 1e-3 * scale
        assert np.array_equal(a == 0, b == 0)   # faces outside the system are cleared


def test_viscosity_deterministic(case):
    n, dx = int(case["n"]), float(case["dx"])
    (u, v, w), st, _ = G.viscosity(n, dx, float(case["dt"]), case["liquid_phi"], case["solid_phi"],
                                   float(case["viscosity"]), [case["visc_in_" + c] for c in "uvw"])
    (u0, v0, w0), st0, _ = case["gpu"]
    assert st == st0 and bits_equal(u, u0) and bits_equal(v, v0) and bits_equal(w, w0)


def test_viscosity_no_liquid_leaves_field():
    """Without liquid the system is empty: only the velocity constraint that precedes the solve
    (fluidsimulation.cpp:6023) touches the field."""
    n, dx = 12, 1.0 / 12
    solid = O.solid_phi(n, dx)
    phi = np.full((n, n, n), 0.5 * dx, np.float32)
    uvw = [np.full(s, 0.25, np.float32) for s in ((n, n, n + 1), (n, n + 1, n), (n + 1, n, n))]
    (u, v, w), st, _ = G.viscosity(n, dx, 1 / 240, phi, solid, 1.0, uvw)
    assert st["n"] == 0 and st["success"]
    want = O.constrain(n, O.face_weights(n, solid), uvw)
    assert all(np.array_equal(a, b) for a, b in zip((u, v, w), want))


def test_viscosity_substep_vs_reference(case):
    import ffengine_gb300 as ffe
    n = int(case["n"])
    sim = ffe.FluidSimulation(n, n, n, 1.0 / n)
    sim.set_viscosity_warm_start(False)   # the reference solver's zero start (iteration counts)
    sim.enable_extreme_velocity_removal = False
    sim.add_body_force(0.0, -9.81, 0.0)
    sim.viscosity = float(case["viscosity"])
    pos, vel = case["in_pos"], case["in_vel"]
    sim.load_marker_particle_data(pos.shape[0], pos.tobytes(), vel.tobytes())
    sim.initialize()
    sim.set_solid_level_set(np.ascontiguousarray(case["solid_phi"], np.float32).tobytes())
    sim.update(float(case["dt"]))
    st = sim.get_frame_stats_data()
    assert st.viscositySolverEnabled == 1 and st.viscositySolverSuccess == 1
    assert abs(st.viscositySolverIterations - int(case["visc_stats"][1])) <= 3
    x = np.frombuffer(sim.get_marker_particle_position_data(), np.float32).reshape(-1, 3)
    v = np.frombuffer(sim.get_marker_particle_velocity_data(), np.float32).reshape(-1, 3)
    assert x.shape == case["p1_pos"].shape
    assert np.abs(x - case["p1_pos"]).max() <= 5e-6
    assert np.abs(v - case["p1_vel"]).max() <= 2e-4 * max(np.abs(case["p1_vel"]).max(), 1.0)


def test_viscosity_trajectory_20_substeps_vs_reference():
    import ffengine_gb300 as ffe
    d = dict(np.load(golden_path("visctraj16")))
    n = int(d["n"])
    sim = ffe.FluidSimulation(n, n, n, 1.0 / n)
    sim.set_viscosity_warm_start(False)   # the reference solver's zero start (iteration counts)
    sim.enable_extreme_velocity_removal = False
    sim.add_body_force(0.0, -9.81, 0.0)
    sim.viscosity = float(d["viscosity"])
    pos, vel = d["in_pos"], d["in_vel"]
    sim.load_marker_particle_data(pos.shape[0], pos.tobytes(), vel.tobytes())
    sim.initialize()
    sim.set_solid_level_set(np.ascontiguousarray(d["solid_phi"], np.float32).tobytes())
    for s in range(d["traj_stats"].shape[0]):
        sim.update(float(d["dt"]))
        m = d["traj_moments"][s]
        x = np.frombuffer(sim.get_marker_particle_position_data(), np.float32).reshape(-1, 3).astype(np.float64)
        v = np.frombuffer(sim.get_marker_particle_velocity_data(), np.float32).reshape(-1, 3).astype(np.float64)
        assert x.shape[0] == int(m[0])
        assert abs(sim.get_frame_stats_data().pressureSolverIterations - int(d["traj_stats"][s, 1])) <= 1
        assert np.abs(x.mean(0) - m[1:4]).max() < 1e-5
        assert np.abs(v.mean(0) - m[4:7]).max() < 2e-4


def test_viscosity_setters():
    import ffengine_gb300 as ffe
    sim = ffe.FluidSimulation(8, 8, 8, 1 / 8)
    assert sim.viscosity == 0.0
    assert sim.viscosity_solver_error_tolerance == 1e-4 and sim.viscosity_solver_max_iterations == 900
    sim.viscosity = 2.5
    sim.viscosity_solver_error_tolerance = 1e-5
    sim.viscosity_solver_max_iterations = 50
    assert sim.viscosity == 2.5 and sim.viscosity_solver_error_tolerance == 1e-5
    assert sim.viscosity_solver_max_iterations == 50
    with pytest.raises(RuntimeError, match="viscosity must be greater"):
        sim.viscosity = -1.0


def test_differentiable_substep_rejects_viscosity():
    import ffengine_gb300 as ffe
    sim = ffe.FluidSimulation(8, 8, 8, 1 / 8)
    sim.viscosity = 1.0
    p = np.full((4, 3), 0.5, np.float32)
    sim.load_marker_particle_data(4, p.tobytes(), p.tobytes())
    sim.initialize()
    with pytest.raises(RuntimeError, match="viscosity solve"):
        sim.substep_differentiable(1 / 240)


def synthetic_system(shape, seed=0):
    """A dam-break-like liquid block and a sphere of liquid in a closed box of the given cells
    (non-cubic), random face velocities: a system whose component boxes span several 16 x 16 tiles."""
    ni, nj, nk = shape
    dx = 1.0 / max(shape)
    rng = np.random.default_rng(seed)
    zc, yc, xc = np.meshgrid((np.arange(nk) + 0.5) * dx, (np.arange(nj) + 0.5) * dx, (np.arange(ni) + 0.5) * dx,
                             indexing="ij")
    block = np.maximum(np.maximum(xc - 0.45 * ni * dx, yc - 0.55 * nj * dx), zc - 0.8 * nk * dx)
    sphere = np.sqrt((xc - 0.7 * ni * dx) ** 2 + (yc - 0.7 * nj * dx) ** 2 + (zc - 0.4 * nk * dx) ** 2) - 0.15
    liquid = np.minimum(block, sphere).astype(np.float32)
    zn, yn, xn = np.meshgrid(np.arange(nk + 1) * dx, np.arange(nj + 1) * dx, np.arange(ni + 1) * dx, indexing="ij")
    walls = np.minimum.reduce([xn, ni * dx - xn, yn, nj * dx - yn, zn, nk * dx - zn]) - 1.5 * dx
    obstacle = np.sqrt((xn - 0.25 * ni * dx) ** 2 + (yn - 0.2 * nj * dx) ** 2 + (zn - 0.5 * nk * dx) ** 2) - 0.1
    solid = np.minimum(walls, obstacle).astype(np.float32)
    uvw = [rng.normal(0, 1, s).astype(np.float32)
           for s in ((nk, nj, ni + 1), (nk, nj + 1, ni), (nk + 1, nj, ni))]
    return dx, liquid, solid, uvw


PRECOND_CASES = ["visc20", "viscsphere24", (45, 38, 52), (64, 40, 36)]


@pytest.mark.parametrize("which", PRECOND_CASES, ids=str)
def test_viscosity_preconditioner_forms(which):
    """The tiled wavefront forms against the reference-order level form.  Swept along the grid's z
    axis (form 3) the forward sweep (L z = b) is bit-identical; with both sweeps it is within float
    rounding of the level form (its backward sweep subtracts the couplings to the later components
    before a row's own neighbours).  Along each box's shortest axis (form 0, the default) a row's
    own neighbours are also subtracted in the box's axis order: within float rounding in both
    sweeps.  The cooperative form is bit-identical to the level form."""
    if isinstance(which, str):
        d = dict(np.load(golden_path(which)))
        n = int(d["n"])
        shape, dx, dt, visc = (n, n, n), float(d["dx"]), float(d["dt"]), float(d["viscosity"])
        liquid, solid, uvw = d["liquid_phi"], d["solid_phi"], [d["visc_in_" + c] for c in "uvw"]
    else:
        shape, dt, visc = which, 1.0 / 240, 1.0
        dx, liquid, solid, uvw = synthetic_system(which)
    args = (shape, dx, dt, liquid, solid, visc, uvw)
    lv1 = G.viscosity_precondition(*args, form=1, sweeps=1)
    assert lv1.size > 1000
    assert bits_equal(G.viscosity_precondition(*args, form=3, sweeps=1), lv1)
    lv2 = G.viscosity_precondition(*args, form=1, sweeps=2)
    assert bits_equal(G.viscosity_precondition(*args, form=2, sweeps=2), lv2)

    def close(a, b):
        return (np.abs(a - b).max() <= 2e-5 * np.abs(b).max() and
                np.linalg.norm(a - b) <= 2e-6 * np.linalg.norm(b))

    assert close(G.viscosity_precondition(*args, form=0, sweeps=1), lv1)
    for form in (0, 3):
        z = G.viscosity_precondition(*args, form=form, sweeps=2)
        assert close(z, lv2), form
        assert bits_equal(G.viscosity_precondition(*args, form=form, sweeps=2), z)   # deterministic


def test_viscosity_solve_forms_agree(case):
    """The substep's viscosity solve with the level-form preconditioner meets the same stopping
    rule, and the two solutions agree within the solve's tolerance."""
    import ffengine_gb300 as ffe
    n = int(case["n"])
    out = []
    for form in (0, 1, 3):
        sim = ffe.FluidSimulation(n, n, n, 1.0 / n)
        sim.set_viscosity_warm_start(False)   # the reference solver's zero start (iteration counts)
        sim.enable_extreme_velocity_removal = False
        sim.add_body_force(0.0, -9.81, 0.0)
        sim.viscosity = float(case["viscosity"])
        sim.set_viscosity_preconditioner(form)
        pos, vel = case["in_pos"], case["in_vel"]
        sim.load_marker_particle_data(pos.shape[0], pos.tobytes(), vel.tobytes())
        sim.initialize()
        sim.set_solid_level_set(np.ascontiguousarray(case["solid_phi"], np.float32).tobytes())
        sim.update(float(case["dt"]))
        st = sim.get_frame_stats_data()
        assert st.viscositySolverSuccess == 1
        assert abs(st.viscositySolverIterations - int(case["visc_stats"][1])) <= 3
        out.append(np.frombuffer(sim.get_marker_particle_velocity_data(), np.float32).reshape(-1, 3).copy())
    for o in (out[0], out[2]):
        assert o.shape == out[1].shape
        assert np.abs(o - out[1]).max() <= 2e-4 * max(np.abs(out[1]).max(), 1.0)
    with pytest.raises(RuntimeError, match="preconditioner form"):
        sim.set_viscosity_preconditioner(4)


def test_viscosity_warm_start():
    """The viscosity PCG started from the field before the solve stops on the zero start's rule
    (|r|inf <= tol |b|inf), so every substep's solve succeeds; over a trajectory it needs fewer
    iterations and the particles stay with the zero-start run's to the solve's accuracy."""
    import ffengine_gb300 as ffe
    d = dict(np.load(golden_path("visctraj16")))
    n = int(d["n"])
    out = {}
    for warm in (False, True):
        sim = ffe.FluidSimulation(n, n, n, 1.0 / n)
        sim.set_viscosity_warm_start(warm)
        sim.enable_extreme_velocity_removal = False
        sim.add_body_force(0.0, -9.81, 0.0)
        sim.viscosity = float(d["viscosity"])
        pos, vel = d["in_pos"], d["in_vel"]
        sim.load_marker_particle_data(pos.shape[0], pos.tobytes(), vel.tobytes())
        sim.initialize()
        sim.set_solid_level_set(np.ascontiguousarray(d["solid_phi"], np.float32).tobytes())
        its = []
        for _ in range(10):
            sim.update(float(d["dt"]))
            st = sim.get_frame_stats_data()
            assert st.viscositySolverEnabled == 1 and st.viscositySolverSuccess == 1
            its.append(int(st.viscositySolverIterations))
        x = np.frombuffer(sim.get_marker_particle_position_data(), np.float32).reshape(-1, 3)
        v = np.frombuffer(sim.get_marker_particle_velocity_data(), np.float32).reshape(-1, 3)
        out[warm] = (its, x.copy(), v.copy())
    print("viscosity iterations, zero / warm start:", out[False][0], out[True][0])
    assert sum(out[True][0][1:]) < sum(out[False][0][1:])
    assert out[True][1].shape == out[False][1].shape
    assert np.abs(out[True][1] - out[False][1]).max() <= 1e-4
    assert np.abs(out[True][2] - out[False][2]).max() <= 2e-3 * max(np.abs(out[False][2]).max(), 1.0)
