"""GPU parity: every kernel group of libffengine_gb300.so against the reference engine's
golden vectors and the CPU oracle, on identical inputs.

Bars (per stage):
  bit-exact  -- solid level set, face weights, particle sort, liquid SDF (raw and
                post-processed), extrapolation, projection, removal;
  1e-6 rel.  -- P2G face values (summation order differs from the reference's particle
                order); valid flags equal;
  FP64 PCG   -- same iteration count as the reference, pressure within 1e-6 of max|p|;
  mixed PCG  -- FP64-checked ||b - A p||_inf <= 1e-6 ||b||_inf (the solve tolerance);
  G2P/RK3    -- FP32 MAC sampling where the reference samples in double: velocities
                within 2e-5 relative to max|v|, positions within 2e-6 (absolute, domain 1).
"""
import numpy as np
import pytest

import gpu_api as G
import oracle_api as O
from conftest import golden_path

pytestmark = pytest.mark.gpu

CASES = ["dam20", "rand20", "sphere24"]


def bits_equal(a, b):
    a = np.ascontiguousarray(a); b = np.ascontiguousarray(b)
    return a.shape == b.shape and np.array_equal(a.view(np.uint32), b.view(np.uint32))


@pytest.fixture(scope="module", params=CASES)
def case(request):
    d = dict(np.load(golden_path(request.param)))
    d["name"] = request.param
    return d


def test_solid_phi_matches_oracle():
    """The engine's default solid level set: the closed domain's box mesh (bit-exact with the
    oracle's mesh path), with analytic spheres united in double (the sphere extension)."""
    for n, sph in [(20, ()), (24, [(0.6, 0.3, 0.5, 0.15)]), (33, [(0.5, 0.5, 0.5, 0.2), (0.2, 0.7, 0.4, 0.1)])]:
        dx = 1.0 / n
        want = O.solid_level_set(n, dx).astype(np.float64)
        g = np.arange(n + 1) * dx
        z, y, x = np.meshgrid(g, g, g, indexing="ij")
        for cx, cy, cz, r in sph:
            want = np.minimum(want, np.sqrt((x - cx) * (x - cx) + (y - cy) * (y - cy) + (z - cz) * (z - cz)) - r)
        assert bits_equal(G.solid_phi(n, dx, sph), want.astype(np.float32))


def test_face_weights_bitexact(case):
    n = int(case["n"])
    for c, w in zip("uvw", G.face_weights(n, case["solid_phi"])):
        assert bits_equal(w, case["weight_" + c])


def test_sort_is_stable_counting_sort(case):
    n, dx = int(case["n"]), float(case["dx"])
    pos = case["in_pos"]
    cs, si = G.sort_particles(n, dx, pos)
    idx = np.floor(pos.astype(np.float64) * (1.0 / dx)).astype(np.int64)
    key = idx[:, 0] + n * (idx[:, 1] + n * idx[:, 2])
    assert np.array_equal(si, np.argsort(key, kind="stable"))
    assert np.array_equal(cs, np.concatenate([[0], np.cumsum(np.bincount(key, minlength=n ** 3))]))


def test_sort_empty_and_single():
    cs, si = G.sort_particles(8, 1 / 8, np.zeros((0, 3), np.float32))
    assert cs.sum() == 0 and si.size == 0
    cs, si = G.sort_particles(8, 1 / 8, np.array([[0.51, 0.26, 0.9]], np.float32))
    assert si.tolist() == [0] and cs[-1] == 1


def test_liquid_sdf_bitexact(case):
    n, dx = int(case["n"]), float(case["dx"])
    raw = G.liquid_sdf(n, dx, case["in_pos"])
    assert bits_equal(raw, case["liquid_phi_raw"])
    post = G.liquid_sdf(n, dx, case["in_pos"], case["solid_phi"], post=True)
    assert bits_equal(post, case["liquid_phi"])


def test_liquid_sdf_random_vs_oracle():
    rng = np.random.default_rng(7)
    for n in (12, 31):
        dx = 1.0 / n
        pos = rng.random((3000, 3)).astype(np.float32) * np.float32(0.999)
        assert bits_equal(G.liquid_sdf(n, dx, pos), O.liquid_sdf(n, dx, pos))


def test_p2g_within_1e6(case):
    n, dx = int(case["n"]), float(case["dx"])
    g = G.p2g(n, dx, case["in_pos"], case["in_vel"])
    for c, (f, v) in zip("uvw", g):
        ref = case["p2g_" + c]
        assert np.array_equal(v, case["p2g_valid" + c])
        scale = max(np.abs(ref).max(), 1e-30)
        assert np.abs(f - ref).max() <= 1e-6 * scale + 1e-12


def test_p2g_deterministic(case):
    n, dx = int(case["n"]), float(case["dx"])
    a = G.p2g(n, dx, case["in_pos"], case["in_vel"])
    b = G.p2g(n, dx, case["in_pos"], case["in_vel"])
    for (fa, va), (fb, vb) in zip(a, b):
        assert bits_equal(fa, fb) and np.array_equal(va, vb)


def test_p2g_three_components_in_one_pass_bitexact(case):
    """The substep's P2G transfers to the three components in one pass over the particles of each
    3 x 3 x 3 window; every face's sums are the one-component kernel's, in the same order."""
    n, dx = int(case["n"]), float(case["dx"])
    a = G.p2g(n, dx, case["in_pos"], case["in_vel"])
    b = G.p2g(n, dx, case["in_pos"], case["in_vel"], per_component=True)
    for (fa, va), (fb, vb) in zip(a, b):
        assert bits_equal(fa, fb) and np.array_equal(va, vb)


def test_extrapolation_bitexact(case):
    L = O.layers(int(case["cfl"]))
    for c in "uvw":
        got = G.extrapolate(case["p2g_" + c], case["p2g_valid" + c], L)
        assert bits_equal(got, case["adv_" + c])
        got = G.extrapolate(case["proj_" + c], case["proj_valid" + c], L)
        assert bits_equal(got, case["projx_" + c])


def test_pressure_fp64_matches_reference(case):
    n, dx, dt = int(case["n"]), float(case["dx"]), float(case["dt"])
    w = O.face_weights(n, case["solid_phi"])
    body = [case["body_" + c] for c in "uvw"]
    pr, p64, st = G.pressure_solve(n, dx, dt, case["liquid_phi"], w, body, tol=1e-9, mode=0)
    assert st["success"]
    assert st["iters"] == int(case["pressure_iters"][0])
    ref = case["pressure"]
    assert np.abs(pr - ref).max() <= 1e-6 * np.abs(ref).max()


@pytest.mark.parametrize("tol", [1e-6, 1e-9])
def test_pressure_mixed_fp64_checked(case, tol):
    n, dx, dt = int(case["n"]), float(case["dx"]), float(case["dt"])
    w = O.face_weights(n, case["solid_phi"])
    body = [case["body_" + c] for c in "uvw"]
    pr, p64, st = G.pressure_solve(n, dx, dt, case["liquid_phi"], w, body, tol=tol, mode=1)
    assert st["success"]
    inf, rel2 = O.pressure_residual(n, dx, dt, case["liquid_phi"], w, body, p64)
    assert inf <= tol * 1.0001
    # against the FP64 oracle solve to 1e-12
    p_ref, it, ok, err, nf = O.pressure_solve(n, dx, dt, case["liquid_phi"], w, body, tol=1e-12, float_scalars=False)
    rel = np.linalg.norm(p64 - p_ref) / np.linalg.norm(p_ref)
    assert rel < 1e4 * tol


def test_projection_bitexact(case):
    n, dx, dt = int(case["n"]), float(case["dx"]), float(case["dt"])
    w = O.face_weights(n, case["solid_phi"])
    (u, v, ww), valid = G.apply_pressure(n, dx, dt, case["liquid_phi"], w, case["pressure"],
                                         [case["body_" + c] for c in "uvw"])
    for c, a, vv in zip("uvw", (u, v, ww), valid):
        assert bits_equal(a, case["proj_" + c])
        assert np.array_equal(vv, case["proj_valid" + c])


def test_g2p_close(case):
    n, dx = int(case["n"]), float(case["dx"])
    cons = [case["cons_" + c] for c in "uvw"]
    saved = [case["saved_" + c] for c in "uvw"]
    vel = G.g2p(n, dx, float(case["pic"]), case["p0_pos"], case["in_vel"], cons, saved)
    ref = case["g2p_vel"]
    assert np.abs(vel - ref).max() <= 2e-5 * max(np.abs(ref).max(), 1.0)


def test_advect_close(case):
    n, dx, dt = int(case["n"]), float(case["dx"]), float(case["dt"])
    cons = [case["cons_" + c] for c in "uvw"]
    pos = G.advect(n, dx, dt, int(case["cfl"]), case["p0_pos"], cons, case["solid_phi"])
    assert np.abs(pos - case["adv_pos"]).max() <= 2e-6


def test_remove_bitexact(case):
    n, dx = int(case["n"]), float(case["dx"])
    p1, v1 = G.remove(n, dx, case["adv_pos"], case["g2p_vel"], case["solid_phi"])
    assert bits_equal(p1, case["p1_pos"]) and bits_equal(v1, case["p1_vel"])


def test_remove_cell_cap_in_particle_order():
    n, dx = 8, 1.0 / 8
    solid = O.solid_phi(n, dx)
    rng = np.random.default_rng(3)
    pos = (np.array([4.5, 4.5, 4.5]) * dx + (rng.random((40, 3)) - 0.5) * 0.9 * dx).astype(np.float32)
    vel = rng.standard_normal((40, 3)).astype(np.float32)
    gp, gv = G.remove(n, dx, pos, vel, solid, max_per_cell=7)
    op, ov = O.remove(n, dx, pos, vel, solid, max_per_cell=7)
    assert gp.shape[0] == 7 and bits_equal(gp, op) and bits_equal(gv, ov)


def test_full_substep_vs_oracle(case):
    n, dx, dt = int(case["n"]), float(case["dx"]), float(case["dt"])
    args = (n, dx, dt, float(case["pic"]), int(case["cfl"]), (0.0, -9.81, 0.0), case["solid_phi"])
    gp, gv, gs = G.substep(*args, case["in_pos"], case["in_vel"])
    op, ov, os_ = O.substep(*args, case["in_pos"], case["in_vel"])
    assert gp.shape == op.shape
    assert abs(gs["iters"] - os_["iters"]) <= 1
    assert np.abs(gp - op).max() <= 5e-6
    assert np.abs(gv - ov).max() <= 1e-4 * max(np.abs(ov).max(), 1.0)


def test_substep_deterministic(case):
    n, dx, dt = int(case["n"]), float(case["dx"]), float(case["dt"])
    args = (n, dx, dt, float(case["pic"]), int(case["cfl"]), (0.0, -9.81, 0.0), case["solid_phi"],
            case["in_pos"], case["in_vel"])
    a = G.substep(*args)
    b = G.substep(*args)
    assert bits_equal(a[0], b[0]) and bits_equal(a[1], b[1])


def test_trajectory_30_substeps_vs_reference():
    d = np.load(golden_path("traj16"))
    n, dx, dt = int(d["n"]), float(d["dx"]), float(d["dt"])
    pos, vel = d["in_pos"], d["in_vel"]
    for s in range(d["traj_stats"].shape[0]):
        pos, vel, st = G.substep(n, dx, dt, float(d["pic"]), int(d["cfl"]), (0, -9.81, 0), d["solid_phi"], pos, vel)
        m = d["traj_moments"][s]
        assert pos.shape[0] == int(m[0])
        assert abs(st["iters"] - int(d["traj_stats"][s, 1])) <= 1
        assert np.abs(pos.astype(np.float64).mean(0) - m[1:4]).max() < 1e-5
        assert np.abs(vel.astype(np.float64).mean(0) - m[4:7]).max() < 1e-4
    assert np.abs(pos - d["final_pos"]).max() < 1e-4


def _system(n, seed, xb=0.6, yb=0.7, sigma=1.0, sphere=()):
    from ffengine_gb300 import scenes
    pos, vel = scenes.dam_break_particles(n, xb, yb, seed=seed, velocity_sigma=sigma)
    dx = 1.0 / n
    solid = O.solid_phi(n, dx, sphere)
    phi = O.postprocess_sdf(n, dx, solid, O.liquid_sdf(n, dx, pos))
    uvw = [O.extrapolate(f, v, O.layers(5)) for f, v in O.p2g(n, dx, pos, vel)]
    return dx, phi, O.face_weights(n, solid), O.body_force(n, 1 / 240, (0, -9.81, 0), *uvw)


@pytest.mark.parametrize("n,xb,yb,sphere", [(19, 0.6, 0.7, ()), (37, 0.9, 0.3, ((0.5, 0.2, 0.5, 0.2),)),
                                           (40, 0.15, 0.95, ()), (23, 0.99, 0.99, ((0.5, 0.5, 0.5, 0.3),))])
@pytest.mark.parametrize("mode", [0, 1])
def test_wavefront_mic_bit_identical_to_hyperplane_levels(n, xb, yb, sphere, mode):
    """The wavefront kernels factor and apply exactly the hyperplane-ordered MIC(0): the
    whole solve (iterations and pressure bits) must not change, in FP64 and in FP32 (the mixed
    solve in the axis-ordered copy and in the grid's order alike)."""
    dx, phi, w, body = _system(n, 11, xb, yb, 1.0, sphere)
    for order in ((0, 4) if mode else (0,)):
        a = G.pressure_solve(n, dx, 1 / 240, phi, w, body, tol=1e-7, mode=mode | order)
        b = G.pressure_solve(n, dx, 1 / 240, phi, w, body, tol=1e-7, mode=mode | 2 | order)
        assert a[2]["iters"] == b[2]["iters"] and a[2]["success"] and b[2]["success"]
        assert bits_equal(a[0], b[0])
        assert np.array_equal(a[1], b[1])


def test_wavefront_single_cell_box():
    n = 8
    dx = 1.0 / n
    phi = np.full((n, n, n), 3 * dx, np.float32)
    phi[4, 3, 2] = -0.5 * dx
    solid = O.solid_phi(n, dx)
    w = O.face_weights(n, solid)
    u = np.zeros((n, n, n + 1), np.float32); v = np.zeros((n, n + 1, n), np.float32); ww = np.zeros((n + 1, n, n), np.float32)
    v[4, 3, 2] = 0.3
    pr, p64, st = G.pressure_solve(n, dx, 1 / 240, phi, w, (u, v, ww), tol=1e-9, mode=0)
    ref, it, ok, err, nf = O.pressure_solve(n, dx, 1 / 240, phi, w, (u, v, ww), tol=1e-9)
    assert st["success"] and st["iters"] == it and np.abs(pr - ref).max() <= 1e-6 * max(np.abs(ref).max(), 1e-30)


@pytest.mark.parametrize("n", [19, 38, 40])
def test_pressure_mixed_row_alignments(n):
    """FP32 vector kernels run on aligned four-cell groups when ni is a multiple of 4 and per
    cell otherwise; both reach the FP64-checked tolerance against the oracle's FP64 system."""
    dx, phi, w, body = _system(n, 5, 0.7, 0.6, 1.0, ((0.55, 0.35, 0.5, 0.15),))
    for tol in (1e-6, 1e-8):
        pr, p64, st = G.pressure_solve(n, dx, 1 / 240, phi, w, body, tol=tol, mode=1)
        assert st["success"]
        inf, rel2 = O.pressure_residual(n, dx, 1 / 240, phi, w, body, p64)
        assert inf <= tol * 1.0001


@pytest.mark.parametrize("n", [48, 64])
def test_mixed_solve_axis_order(n):
    """The mixed solve in the axis-ordered copy of the pressure box (its shortest axis swept by the
    MIC(0) wavefront) against the same solve in the grid's order: both meet the FP64-checked
    tolerance, their iteration counts differ by a few at most and the solutions agree to the
    solver's accuracy; the FP64 solver ignores the setting."""
    from ffengine_gb300 import scenes
    dx, dt = 1.0 / n, 1.0 / 240
    pos, _ = scenes.dam_break_particles(n, 0.4, 0.6, seed=0)
    solid = O.solid_level_set(n, dx)
    phi = G.liquid_sdf(n, dx, pos, solid, post=True)
    w = G.face_weights(n, solid)
    rng = np.random.default_rng(n)
    uvw = [rng.standard_normal(a.shape).astype(np.float32) for a in w]
    tol = 1e-9
    p_auto, x_auto, s_auto = G.pressure_solve(n, dx, dt, phi, w, uvw, tol=tol, mode=1)
    p_grid, x_grid, s_grid = G.pressure_solve(n, dx, dt, phi, w, uvw, tol=tol, mode=1 | 4)
    assert s_auto["success"] and s_grid["success"]
    for x in (x_auto, x_grid):
        inf, _ = O.pressure_residual(n, dx, dt, phi, w, uvw, x)
        assert inf <= tol * 1.0001
    assert abs(s_auto["iters"] - s_grid["iters"]) <= 3, (s_auto["iters"], s_grid["iters"])
    assert np.linalg.norm(x_auto - x_grid) <= 1e-6 * np.linalg.norm(x_grid)
    f_auto = G.pressure_solve(n, dx, dt, phi, w, uvw, tol=tol, mode=0)
    f_grid = G.pressure_solve(n, dx, dt, phi, w, uvw, tol=tol, mode=4)
    assert bits_equal(f_auto[1], f_grid[1]) and f_auto[2]["iters"] == f_grid[2]["iters"]
