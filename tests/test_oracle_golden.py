"""Pins the CPU oracle against golden vectors produced by the reference engine.

The fixtures in tests/golden/ come from the unmodified reference engine
(tests/golden/make_golden.py + oracle/ref_harness.cpp).  Every stage of the substep must
match bit for bit: the oracle restates the reference's float/double semantics exactly.
"""
import numpy as np
import pytest

import oracle_api as O
from conftest import golden_path

STAGE_CASES = ["dam20", "rand20", "sphere24"]


def bits_equal(a, b):
    a = np.ascontiguousarray(a); b = np.ascontiguousarray(b)
    return a.shape == b.shape and np.array_equal(a.view(np.uint32), b.view(np.uint32))


@pytest.fixture(scope="module", params=STAGE_CASES)
def case(request):
    d = dict(np.load(golden_path(request.param)))
    d["name"] = request.param
    return d


def test_face_weights(case):
    n = int(case["n"])
    for c, w in zip("uvw", O.face_weights(n, case["solid_phi"])):
        assert bits_equal(w, case["weight_" + c])


def test_liquid_sdf_bitexact(case):
    n, dx = int(case["n"]), float(case["dx"])
    raw = O.liquid_sdf(n, dx, case["in_pos"])
    assert bits_equal(raw, case["liquid_phi_raw"])
    phi = O.postprocess_sdf(n, dx, case["solid_phi"], raw)
    assert bits_equal(phi, case["liquid_phi"])


def test_classification_bitexact(case):
    phi = case["liquid_phi"]
    interior = np.zeros(phi.shape, bool)
    interior[1:-1, 1:-1, 1:-1] = True
    cells = (phi < 0) & interior
    n, dx, dt = int(case["n"]), float(case["dx"]), float(case["dt"])
    w = O.face_weights(n, case["solid_phi"])
    got, _, _ = O.pressure_system(n, dx, dt, phi, w, [case["body_" + c] for c in "uvw"], dense=False)
    kk, jj, ii = np.nonzero(cells)          # k-j-i order, i fastest
    assert np.array_equal(got, np.stack([ii, jj, kk], 1))


def test_p2g_and_extrapolation_bitexact(case):
    n, dx = int(case["n"]), float(case["dx"])
    g = O.p2g(n, dx, case["in_pos"], case["in_vel"])
    L = O.layers(int(case["cfl"]))
    for c, (f, v) in zip("uvw", g):
        assert bits_equal(f, case["p2g_" + c])
        assert np.array_equal(v, case["p2g_valid" + c])
        assert bits_equal(O.extrapolate(f, v, L), case["adv_" + c])


def test_body_force_bitexact(case):
    n, dt = int(case["n"]), float(case["dt"])
    out = O.body_force(n, dt, (0.0, -9.81, 0.0), *[case["adv_" + c] for c in "uvw"])
    for c, a in zip("uvw", out):
        assert bits_equal(a, case["body_" + c])


def test_pressure_solve_bitexact(case):
    n, dx, dt = int(case["n"]), float(case["dx"]), float(case["dt"])
    w = O.face_weights(n, case["solid_phi"])
    body = [case["body_" + c] for c in "uvw"]
    pr, iters, ok, err, nf = O.pressure_solve(n, dx, dt, case["liquid_phi"], w, body)
    assert ok and iters == int(case["pressure_iters"][0])
    assert np.float32(err) == case["pressure_error"][0]
    assert bits_equal(pr, case["pressure"])
    (u, v, ww), valid = O.apply_pressure(n, dx, dt, case["liquid_phi"], w, pr, body)
    L = O.layers(int(case["cfl"]))
    for c, a, vv in zip("uvw", (u, v, ww), valid):
        assert bits_equal(a, case["proj_" + c])
        assert np.array_equal(vv, case["proj_valid" + c])
        assert bits_equal(O.extrapolate(a, vv, L), case["projx_" + c])


def test_constrain_g2p_advect_remove_bitexact(case):
    n, dx, dt = int(case["n"]), float(case["dx"]), float(case["dt"])
    w = O.face_weights(n, case["solid_phi"])
    cons = O.constrain(n, w, [case["projx_" + c] for c in "uvw"])
    saved = O.constrain(n, w, [case["adv_" + c] for c in "uvw"])
    for c, a, s in zip("uvw", cons, saved):
        assert bits_equal(a, case["cons_" + c])
        assert bits_equal(s, case["saved_" + c])
    vel = O.g2p(n, dx, float(case["pic"]), case["p0_pos"], case["in_vel"], cons, saved)
    assert bits_equal(vel, case["g2p_vel"])
    pos = O.advect(n, dx, dt, int(case["cfl"]), case["p0_pos"], cons, case["solid_phi"])
    assert bits_equal(pos, case["adv_pos"])
    p1, v1 = O.remove(n, dx, pos, vel, case["solid_phi"])
    assert bits_equal(p1, case["p1_pos"]) and bits_equal(v1, case["p1_vel"])


def test_trajectory_bitexact_30_substeps():
    d = np.load(golden_path("traj16"))
    n, dx, dt = int(d["n"]), float(d["dx"]), float(d["dt"])
    pos, vel = d["in_pos"], d["in_vel"]
    for s in range(d["traj_stats"].shape[0]):
        pos, vel, st = O.substep(n, dx, dt, float(d["pic"]), int(d["cfl"]), (0, -9.81, 0), d["solid_phi"], pos, vel)
        assert pos.shape[0] == int(d["traj_moments"][s, 0])
        assert st["iters"] == int(d["traj_stats"][s, 1])
    assert bits_equal(pos, d["final_pos"]) and bits_equal(vel, d["final_vel"])


def test_analytic_box_matches_reference_band():
    """The product computes the closed-domain solid level set analytically; inside the
    reference's exact band (3 cells) it agrees with the reference's box-mesh SDF."""
    d = np.load(golden_path("dam20"))
    n, dx = int(d["n"]), float(d["dx"])
    ref = d["solid_phi"]
    ana = O.solid_phi(n, dx)
    band = np.abs(ref) < 3 * dx
    assert np.abs(ana[band] - ref[band]).max() < 1e-6
    assert np.array_equal(np.sign(ana), np.sign(ref))


# ---- APIC transfer (velocityadvector.cpp:543-623, fluidsimulation.cpp:6791-6843) ----
@pytest.fixture(scope="module", params=["apic20", "apicsphere24"])
def apic(request):
    return dict(np.load(golden_path(request.param)))


def test_apic_p2g_bitexact(apic):
    n, dx = int(apic["n"]), float(apic["dx"])
    for c, (f, v) in zip("uvw", O.p2g_apic(n, dx, apic["in_pos"], apic["in_vel"], apic["in_aff"])):
        assert bits_equal(f, apic["p2g_" + c])
        assert np.array_equal(v, apic["p2g_valid" + c])


def test_apic_g2p_bitexact(apic):
    n, dx = int(apic["n"]), float(apic["dx"])
    vel, aff = O.g2p_apic(n, dx, apic["p0_pos"], [apic["cons_" + c] for c in "uvw"])
    assert bits_equal(vel, apic["g2p_vel"])
    assert bits_equal(aff, apic["g2p_aff"])


def test_apic_substep_bitexact(apic):
    n, dx = int(apic["n"]), float(apic["dx"])
    solid = apic["solid_phi"]
    pos, vel, aff, st = O.substep_apic(n, dx, float(apic["dt"]), int(apic["cfl"]), (0.0, -9.81, 0.0), solid,
                                       apic["in_pos"], apic["in_vel"], apic["in_aff"])
    assert bits_equal(pos, apic["p1_pos"]) and bits_equal(vel, apic["p1_vel"]) and bits_equal(aff, apic["p1_aff"])


def test_apic_trajectory_bitexact():
    d = dict(np.load(golden_path("apictraj16")))
    n, dx = int(d["n"]), float(d["dx"])
    solid = d["solid_phi"]
    pos, vel, aff = d["in_pos"], d["in_vel"], d["in_aff"]
    for s in range(d["traj_stats"].shape[0]):
        pos, vel, aff, st = O.substep_apic(n, dx, float(d["dt"]), int(d["cfl"]), (0.0, -9.81, 0.0), solid, pos, vel, aff)
        assert pos.shape[0] == int(d["traj_stats"][s, 0])
    assert bits_equal(pos, d["final_pos"]) and bits_equal(vel, d["final_vel"]) and bits_equal(aff, d["final_aff"])


# ---- viscosity solve (ViscositySolver) against the reference's own system, factor and solution ----

@pytest.fixture(scope="module", params=["visc20", "viscsphere24"])
def visc(request):
    return dict(np.load(golden_path(request.param)))


def _visc_run(d):
    n, dx = int(d["n"]), float(d["dx"])
    return O.viscosity(n, dx, float(d["dt"]), d["liquid_phi"], d["solid_phi"], float(d["viscosity"]),
                       [d["visc_in_" + c] for c in "uvw"], debug=True)


def test_viscosity_volumes_and_system_bitexact(visc):
    (_, _, _), st, dbg = _visc_run(visc)
    for g in ("center", "u", "v", "w", "eu", "ev", "ew"):
        assert bits_equal(dbg["vol"][g], visc["visc_vol_" + g]), g
    assert np.array_equal(dbg["index"], visc["visc_index"])
    assert st["n"] == int(visc["visc_stats"][0])
    assert np.array_equal(dbg["rowstart"], visc["visc_rowstart"])
    assert np.array_equal(dbg["col"], visc["visc_col"])
    assert bits_equal(dbg["val"], visc["visc_val"]) and bits_equal(dbg["rhs"], visc["visc_rhs"])


def test_viscosity_mic0_factor_bitexact(visc):
    _, _, dbg = _visc_run(visc)
    assert np.array_equal(dbg["ic_colstart"], visc["visc_ic_colstart"])
    assert np.array_equal(dbg["ic_rowindex"], visc["visc_ic_rowindex"])
    assert bits_equal(dbg["ic_invdiag"], visc["visc_ic_invdiag"]) and bits_equal(dbg["ic_value"], visc["visc_ic_value"])


def test_viscosity_solve_bitexact(visc):
    (u, v, w), st, dbg = _visc_run(visc)
    assert st["iters"] == int(visc["visc_stats"][1]) and st["success"] == bool(visc["visc_stats"][2])
    assert bits_equal(np.float32(st["error"]), visc["visc_error"][0])
    assert bits_equal(dbg["soln"], visc["visc_soln"])
    for c, a in zip("uvw", (u, v, w)):
        assert bits_equal(a, visc["visc_" + c]), c


def test_viscosity_substep_bitexact(visc):
    n, dx = int(visc["n"]), float(visc["dx"])
    pos, vel, st = O.substep_visc(n, dx, float(visc["dt"]), float(visc["pic"]), int(visc["cfl"]), (0.0, -9.81, 0.0),
                                  visc["solid_phi"], visc["in_pos"], visc["in_vel"], float(visc["viscosity"]))
    assert bits_equal(pos, visc["p1_pos"]) and bits_equal(vel, visc["p1_vel"])


def test_viscosity_trajectory_bitexact():
    d = dict(np.load(golden_path("visctraj16")))
    n, dx = int(d["n"]), float(d["dx"])
    pos, vel = d["in_pos"], d["in_vel"]
    for s in range(d["traj_stats"].shape[0]):
        pos, vel, st = O.substep_visc(n, dx, float(d["dt"]), float(d["pic"]), int(d["cfl"]), (0.0, -9.81, 0.0),
                                      d["solid_phi"], pos, vel, float(d["viscosity"]))
        assert pos.shape[0] == int(d["traj_stats"][s, 0]) and st["iters"] == int(d["traj_stats"][s, 1])
    assert bits_equal(pos, d["final_pos"]) and bits_equal(vel, d["final_vel"])


# ---- surface curvature grid (the surface-tension input) against the reference ----

@pytest.mark.parametrize("name", ["curv20", "curvsphere24"])
def test_curvature_grid_bitexact(name):
    d = dict(np.load(golden_path(name)))
    n, dx = int(d["n"]), float(d["dx"])
    surf, k = O.curvature_grid(n, dx, d["liquid_phi"])
    assert bits_equal(surf, d["surface_phi"])
    assert bits_equal(k, d["curvature"])


# ---- pressure solve with surface tension (cluster status + ghost-fluid tension term) ----

@pytest.mark.parametrize("name", ["tension20", "tensionsphere24"])
def test_pressure_with_surface_tension_bitexact(name):
    d = dict(np.load(golden_path(name)))
    n, dx, dt = int(d["n"]), float(d["dx"]), float(d["dt"])
    surf, k = O.curvature_grid(n, dx, d["liquid_phi"])
    assert bits_equal(surf, d["surface_phi"]) and bits_equal(k, d["curvature"])
    w = [d["weight_" + c] for c in "uvw"]
    body = [d["body_" + c] for c in "uvw"]
    pr, iters, ok, err, nf = O.pressure_solve_tension(n, dx, dt, d["liquid_phi"], w, body, k,
                                                      float(d["surface_tension"]))
    assert ok and iters == int(d["pressure_iters"][0])
    assert bits_equal(pr, d["pressure"])
    # the term is active: without it the pressure differs
    p0 = O.pressure_solve(n, dx, dt, d["liquid_phi"], w, body)[0]
    assert not np.array_equal(p0, pr)
    # the velocity update with the tension term in the ghost pressure (pressuresolver.cpp:1047-1205)
    (u, v, ww), valid = O.apply_pressure_tension(n, dx, dt, d["liquid_phi"], w, d["pressure"], body, k,
                                                 float(d["surface_tension"]))
    for c, a, vv in zip("uvw", (u, v, ww), valid):
        assert bits_equal(a, d["proj_" + c]), c
        assert np.array_equal(vv, d["proj_valid" + c])


def test_surface_tension_trajectory():
    """20 substeps through the reference's own FluidSimulation::update with surface tension against
    the oracle substep.  Inside update() the curvature grid is computed on a worker thread, whose
    uninitialised re-initialisation temporary (levelsetsolver.cpp:95) holds stale data of that
    thread's allocator arena rather than the copy of the input the main-thread stage harness sees;
    the surface tension term therefore differs slightly from the first substep on (mean velocity
    ~7e-5) and the trajectories drift apart chaotically.  Particle counts and pressure iteration
    counts stay equal at every substep, and the moments stay within these bounds; the bit-exact
    substep check is test_pressure_with_surface_tension_bitexact."""
    d = dict(np.load(golden_path("tensiontraj16")))
    n, dx = int(d["n"]), float(d["dx"])
    pos, vel = d["in_pos"], d["in_vel"]
    for s in range(d["traj_stats"].shape[0]):
        pos, vel, st = O.substep_tension(n, dx, float(d["dt"]), float(d["pic"]), int(d["cfl"]), (0.0, -9.81, 0.0),
                                         d["solid_phi"], pos, vel, float(d["surface_tension"]))
        m = d["traj_moments"][s]
        assert pos.shape[0] == int(d["traj_stats"][s, 0]) and st["iters"] == int(d["traj_stats"][s, 1]), s
        assert np.abs(pos.astype(np.float64).mean(0) - m[1:4]).max() < 1e-3
        assert np.abs(vel.astype(np.float64).mean(0) - m[4:7]).max() < 2e-2


def test_speed_limit_and_extreme_removal_bitexact():
    """Extreme-velocity removal on (the engine's default): the speed limit of the post-transfer
    velocities and the removal it drives, against the reference's own dump."""
    d = dict(np.load(golden_path("evr20")))
    n, dx = int(d["n"]), float(d["dx"])
    limit = O.speed_limit(d["g2p_vel"], int(d["cfl"]), dx, float(d["dt"]), int(d["max_steps"]))
    assert np.float32(limit) == d["speed_limit"][0]
    p1, v1 = O.remove_extreme(n, dx, d["adv_pos"], d["g2p_vel"], d["solid_phi"], limit)
    assert bits_equal(p1, d["p1_pos"]) and bits_equal(v1, d["p1_vel"])
    # the rule removed particles that the solid and per-cell rules keep
    p0, _ = O.remove(n, dx, d["adv_pos"], d["g2p_vel"], d["solid_phi"])
    assert p0.shape[0] > p1.shape[0]


def test_extreme_removal_trajectory_bitexact():
    """20 substeps with the rule on: the fastest particle is dropped whenever few particles are
    near its speed, so the particle count falls by about one per substep."""
    d = dict(np.load(golden_path("evrtraj16")))
    n, dx, dt = int(d["n"]), float(d["dx"]), float(d["dt"])
    pos, vel = d["in_pos"], d["in_vel"]
    for s in range(d["traj_stats"].shape[0]):
        pos, vel, st = O.substep(n, dx, dt, float(d["pic"]), int(d["cfl"]), (0, -9.81, 0), d["solid_phi"], pos, vel,
                                 evr=(dt, int(d["max_steps"])))
        assert pos.shape[0] == int(d["traj_stats"][s, 0]) and st["iters"] == int(d["traj_stats"][s, 1]), s
    assert d["traj_stats"][-1, 0] < d["in_pos"].shape[0] - 10
    assert bits_equal(pos, d["final_pos"]) and bits_equal(vel, d["final_vel"])


def _logged(t):
    """A substep length as the engine logs it (an ostream at its default 6 significant digits)."""
    return float("%g" % t)


@pytest.mark.parametrize("name", ["cfltraj16", "cflmaxtraj16", "cflmin20"])
def test_frame_loop_substeps_bitexact(name):
    """FluidSimulation::update's CFL substepping: per frame the substep count, every substep's
    length (the last one exactly, the others as logged) and the state after the frame."""
    d = dict(np.load(golden_path(name)))
    n, dx, fdt = int(d["n"]), float(d["dx"]), float(d["dt"])
    pos, vel = d["in_pos"], d["in_vel"]
    logged = d["traj_dts"]
    at = 0
    counts = set()
    for f in range(d["traj_stats"].shape[0]):
        pos, vel, dts, sts = O.update(n, dx, fdt, f, int(d["min_steps"]), int(d["max_steps"]), float(d["pic"]),
                                      int(d["cfl"]), (0, -9.81, 0), d["solid_phi"], pos, vel)
        assert len(dts) == int(d["traj_steps"][f, 0]), f
        assert dts[-1] == d["traj_steps"][f, 1]
        for t in dts:
            assert _logged(t) == logged[at]
            at += 1
        counts.add(len(dts))
        assert pos.shape[0] == int(d["traj_stats"][f, 0])
        # the frame reports its last substep's solve (the reference resets the status per solve)
        assert sts[-1]["iters"] == int(d["traj_stats"][f, 1])
    assert at == logged.size and len(counts) > 1
    k = int(d["final_stride"])
    assert bits_equal(pos[::k], d["final_pos"]) and bits_equal(vel[::k], d["final_vel"])


def test_load_queue_order():
    """The reference's load queue (FragmentedVector, 5e6-byte fragments) hands a batch of more than
    208,333 particle records back with record k E replaced by record (k - 1) E wherever k E (1 / E)
    rounds below k: at 208,333 and 416,666 for the 64^3 dam break's 503,291 particles."""
    a = np.arange(503291 * 3, dtype=np.float32).reshape(-1, 3)
    b = O.as_loaded(a)
    moved = np.nonzero(np.any(a != b, axis=1))[0]
    assert moved.tolist() == [208333, 416666]
    assert np.array_equal(b[208333], a[0]) and np.array_equal(b[416666], a[208333])
    assert np.array_equal(O.as_loaded(a[:208333]), a[:208333])


def test_dam_break_64_100_substeps_bitexact():
    """The 64^3 dam break (block x < 0.4, y < 0.6, 8 particles per cell) through 100 substeps of
    1/240 s, from the batch as the reference's load queue hands it over: particle counts and
    pressure iterations at every substep, and the final state (every 64th particle), bit for bit."""
    d = dict(np.load(golden_path("traj64")))
    n, dx, dt = int(d["n"]), float(d["dx"]), float(d["dt"])
    pos, vel = O.as_loaded(d["in_pos"]), O.as_loaded(d["in_vel"])
    for s in range(d["traj_stats"].shape[0]):
        pos, vel, st = O.substep(n, dx, dt, float(d["pic"]), int(d["cfl"]), (0, -9.81, 0), d["solid_phi"], pos, vel)
        assert pos.shape[0] == int(d["traj_moments"][s, 0]) and st["iters"] == int(d["traj_stats"][s, 1]), s
    k = int(d["final_stride"])
    assert bits_equal(pos[::k], d["final_pos"]) and bits_equal(vel[::k], d["final_vel"])


# ---- solid level set of mesh obstacles (meshlevelset.cpp, meshobject.cpp, fluidsimulation.cpp:5277-5333) ----

@pytest.mark.parametrize("name", ["meshsphere24", "meshmix32", "meshislands20"])
def test_mesh_solid_level_set_bitexact(name):
    """The reference's solid level set after the first obstacle update: an icosphere; a torus, a
    box through the domain boundary, a box with its corners on grid nodes, a disabled box and an
    inverted sphere; 30 islands in one object (per-island level sets with the mesh expansion)
    and 10 in another.  The reference draws the inside test's line jitter from rand(); the
    harness fixes the draws to the values the oracle uses by default."""
    d = dict(np.load(golden_path(name)))
    n, dx = int(d["n"]), float(d["dx"])
    objs = O.mesh_objects(d)
    assert bits_equal(O.solid_level_set(n, dx, objs), d["solid_phi"])
    tests = int(d["rand_calls"][0]) // 3
    assert bits_equal(O.solid_level_set(n, dx, objs, np.tile(d["jitter"], (tests, 1))), d["solid_phi"])


def test_mesh_solid_level_set_reproduces_every_golden_solid():
    """Every golden's solid level set (the closed domain, with the icosphere obstacle where the
    scene has the sphere) is the mesh path's output bit for bit, although those runs drew their
    line jitter from the C library's rand()."""
    import glob
    from ffengine_gb300 import scenes
    count = 0
    for path in sorted(glob.glob(golden_path("*"))):
        d = np.load(path)
        if "solid_phi" not in d or "has_sphere" not in d:
            continue
        n, dx = int(d["n"]), float(d["dx"])
        objs = []
        if int(d["has_sphere"]):
            v, t = scenes.icosphere(*[float(x) for x in d["sphere"]], 4)
            objs = [(v, t, 0, 0.0)]
        assert bits_equal(O.solid_level_set(n, dx, objs), d["solid_phi"]), path
        count += 1
    assert count >= 20


def test_mesh_jitter_on_a_diagonal_flips_signs():
    """Why the line jitter has distinct components: with equal ones the lines through the
    diagonal of the domain box's floor and ceiling hit the shared edge of two triangles, and
    the nodes there get the wrong sign (the reference with rand() returning 0 does the same)."""
    n, dx = 16, 1.0 / 16
    good = O.solid_level_set(n, dx)
    jit = 0.001 * dx
    bad = O.solid_level_set(n, dx, jitter=np.full((4, 3), jit, np.float32))
    assert (good > 0).all() or (np.sign(good) != np.sign(bad)).any()
    assert (np.sign(good) != np.sign(bad)).sum() > 0


# ---- FFP3 fluid-particle output (classification, id bins, file data) ----

@pytest.mark.parametrize("name", ["ffp3traj20", "ffp3traj16"])
def test_ffp3_output_bytes_match_reference(name):
    """The reference's FFP3 bytes after every update, from the particles it held then: the liquid
    level set and its surface level set recomputed, the particles classified and grouped."""
    d = dict(np.load(golden_path(name)))
    n, dx = int(d["n"]), float(d["dx"])
    flags, amount = int(d["ffp3_flags"]), float(d["ffp3_amount"])
    steps = int(d["traj_stats"].shape[0])
    for s in range(steps):
        pos, vel, ids = d["ffp3_%d_pos" % s], d["ffp3_%d_vel" % s], d["ffp3_%d_ids" % s]
        surface = O.surface_level_set(n, dx, d["solid_phi"], pos)
        types, data = O.ffp3(n, dx, surface, pos, vel, ids, flags & 7, amount)
        for tag in ("pos", "id", "vel", "speed"):
            key = "ffp3_%d_data_%s" % (s, tag)
            if key in d:
                assert np.array_equal(data[tag], d[key]), (s, tag)
        head = d["ffp3_%d_data_pos" % s].view(np.uint32)
        assert head[3] == int(round(65536 * amount))
        assert np.count_nonzero(types == 3) == 0   # every particle classified


@pytest.mark.parametrize("name", ["sphere24", "dam20"])
def test_condition_solid_velocity_field_is_a_no_op(name):
    """PressureSolver::_conditionSolidVelocityField (pressuresolver.cpp:161-288) only writes zeros
    into the solid velocity field, at faces around fluid pockets enclosed by solids.  With static
    solids that field is zero before the reference's solve and still zero after it, so the step
    changes nothing; the oracle and the GPU leave it out, and the pressure they compute matches the
    reference's (test_pressure_solve_bitexact here, the GPU parity tests on the device)."""
    d = dict(np.load(golden_path(name)))
    absmax = d["solid_velocity_absmax"]
    assert absmax.shape == (6,)
    assert np.all(absmax == 0.0)
