"""GPU parity of the APIC velocity transfer (velocityadvector.cpp:543-623 and
fluidsimulation.cpp:6791-6843) against the reference engine's golden vectors in APIC mode and
the CPU oracle, on identical inputs.

Bars:
  P2G        -- face values within 1e-6 of max|ref| (the GPU sums each face in cell order, the
                reference in particle order); valid flags equal.
  G2P        -- affine vectors bit-exact (same float gradient weights, same node order);
                velocities within 2e-5 of max|v| (FP32 MAC sampling, double in the reference).
  substep    -- counts equal; positions within 5e-6, velocities within 1e-4 of max|v|, affine
                vectors within 1e-4 of max|affine| (the pressure solve and G2P sampling differ
                at rounding level, and the affine vector is a velocity difference over dx).
  trajectory -- 20 substeps: per-substep particle counts equal, moments as the FLIP trajectory.
"""
import numpy as np
import pytest

import gpu_api as G
import oracle_api as O
from conftest import golden_path

pytestmark = pytest.mark.gpu

CASES = ["apic20", "apicsphere24"]


def bits_equal(a, b):
    a = np.ascontiguousarray(a); b = np.ascontiguousarray(b)
    return a.shape == b.shape and np.array_equal(a.view(np.uint32), b.view(np.uint32))


@pytest.fixture(scope="module", params=CASES)
def case(request):
    d = dict(np.load(golden_path(request.param)))
    d["name"] = request.param
    return d


def test_apic_p2g_within_1e6(case):
    n, dx = int(case["n"]), float(case["dx"])
    g = G.p2g_apic(n, dx, case["in_pos"], case["in_vel"], case["in_aff"])
    for c, (f, v) in zip("uvw", g):
        ref = case["p2g_" + c]
        assert np.array_equal(v, case["p2g_valid" + c]), c
        scale = max(np.abs(ref).max(), 1e-30)
        assert np.abs(f - ref).max() <= 1e-6 * scale + 1e-12, c


def test_apic_p2g_block_border_drop(case):
    """The transfer drops the stencil nodes that lie outside the blocks a particle is assigned
    to; the GPU faces match the oracle (which restates that rule) and differ from a plain
    trilinear splat at the faces on 10-cell block borders."""
    n, dx = int(case["n"]), float(case["dx"])
    g = G.p2g_apic(n, dx, case["in_pos"], case["in_vel"], case["in_aff"])
    o = O.p2g_apic(n, dx, case["in_pos"], case["in_vel"], case["in_aff"])
    for (f, v), (of, ov) in zip(g, o):
        assert np.array_equal(v, ov)
        assert np.abs(f - of).max() <= 1e-6 * max(np.abs(of).max(), 1e-30) + 1e-12


def test_apic_p2g_deterministic(case):
    n, dx = int(case["n"]), float(case["dx"])
    a = G.p2g_apic(n, dx, case["in_pos"], case["in_vel"], case["in_aff"])
    b = G.p2g_apic(n, dx, case["in_pos"], case["in_vel"], case["in_aff"])
    for (fa, va), (fb, vb) in zip(a, b):
        assert bits_equal(fa, fb) and np.array_equal(va, vb)


def test_apic_p2g_zero_affine_is_trilinear_average():
    """With zero affine vectors, a single particle gives every face of its stencil its velocity."""
    n, dx = 12, 1.0 / 12
    pos = np.array([[0.43, 0.51, 0.47]], np.float32)
    vel = np.array([[1.5, -2.0, 0.25]], np.float32)
    g = G.p2g_apic(n, dx, pos, vel, np.zeros((1, 9), np.float32))
    o = O.p2g_apic(n, dx, pos, vel, np.zeros((1, 9), np.float32))
    for c, ((f, v), (of, ov)) in enumerate(zip(g, o)):
        assert np.array_equal(v, ov) and v.sum() == 8
        assert np.allclose(f[v == 1], vel[0, c], rtol=1e-6)


def test_apic_p2g_empty():
    n, dx = 8, 1.0 / 8
    e = np.zeros((0, 3), np.float32)
    for f, v in G.p2g_apic(n, dx, e, e, np.zeros((0, 9), np.float32)):
        assert not v.any() and not f.any()


def test_apic_g2p(case):
    n, dx = int(case["n"]), float(case["dx"])
    vel, aff = G.g2p_apic(n, dx, case["p0_pos"], [case["cons_" + c] for c in "uvw"])
    assert bits_equal(aff, case["g2p_aff"])
    ref = case["g2p_vel"]
    assert np.abs(vel - ref).max() <= 2e-5 * max(np.abs(ref).max(), 1.0)


def test_apic_substep_vs_reference(case):
    n, dx, dt = int(case["n"]), float(case["dx"]), float(case["dt"])
    gp, gv, ga, gs = G.substep_apic(n, dx, dt, int(case["cfl"]), (0.0, -9.81, 0.0), case["solid_phi"],
                                    case["in_pos"], case["in_vel"], case["in_aff"])
    assert gs["success"]
    assert gp.shape == case["p1_pos"].shape
    assert np.abs(gp - case["p1_pos"]).max() <= 5e-6
    assert np.abs(gv - case["p1_vel"]).max() <= 1e-4 * max(np.abs(case["p1_vel"]).max(), 1.0)
    ra = case["p1_aff"]
    assert np.abs(ga - ra).max() <= 1e-4 * max(np.abs(ra).max(), 1.0)


def test_apic_substep_deterministic(case):
    n, dx, dt = int(case["n"]), float(case["dx"]), float(case["dt"])
    args = (n, dx, dt, int(case["cfl"]), (0.0, -9.81, 0.0), case["solid_phi"], case["in_pos"], case["in_vel"],
            case["in_aff"])
    a = G.substep_apic(*args)
    b = G.substep_apic(*args)
    assert all(bits_equal(x, y) for x, y in zip(a[:3], b[:3]))


def test_apic_trajectory_20_substeps_vs_reference():
    d = np.load(golden_path("apictraj16"))
    n, dx, dt = int(d["n"]), float(d["dx"]), float(d["dt"])
    pos, vel, aff = d["in_pos"], d["in_vel"], d["in_aff"]
    for s in range(d["traj_stats"].shape[0]):
        pos, vel, aff, st = G.substep_apic(n, dx, dt, int(d["cfl"]), (0, -9.81, 0), d["solid_phi"], pos, vel, aff)
        m = d["traj_moments"][s]
        assert pos.shape[0] == int(m[0])
        assert abs(st["iters"] - int(d["traj_stats"][s, 1])) <= 1
        assert np.abs(pos.astype(np.float64).mean(0) - m[1:4]).max() < 1e-5
        assert np.abs(vel.astype(np.float64).mean(0) - m[4:7]).max() < 1e-4
    assert np.abs(pos - d["final_pos"]).max() < 1e-4
    fa = d["final_aff"]
    assert np.abs(aff - fa).max() <= 1e-3 * max(np.abs(fa).max(), 1.0)


# ---- the reference-facing API (FluidSimulation_* entry points) ----

def _sim(n, apic=True):
    import ffengine_gb300 as ffe
    sim = ffe.FluidSimulation(n, n, n, 1.0 / n)
    if apic:
        sim.set_velocity_transfer_method_APIC()
    return sim


def test_transfer_method_switches():
    sim = _sim(8, apic=False)
    assert sim.is_velocity_transfer_method_FLIP() and not sim.is_velocity_transfer_method_APIC()
    sim.set_velocity_transfer_method_APIC()
    assert sim.is_velocity_transfer_method_APIC() and not sim.is_velocity_transfer_method_FLIP()
    sim.set_velocity_transfer_method_FLIP()
    assert sim.is_velocity_transfer_method_FLIP()
    assert sim.PICAPIC_ratio == 0.0
    sim.PICAPIC_ratio = 0.25
    assert sim.PICAPIC_ratio == 0.25
    with pytest.raises(RuntimeError, match="PICAPIC ratio"):
        sim.PICAPIC_ratio = 1.5


def test_affine_data_round_trip_and_pairing():
    n = 10
    rng = np.random.default_rng(11)
    p1 = (0.1 + 0.8 * rng.random((50, 3))).astype(np.float32)
    p2 = (0.1 + 0.8 * rng.random((30, 3))).astype(np.float32)
    p2[3] = (1.5, 0.5, 0.5)   # outside the domain: dropped with its affine vectors
    a1 = [rng.standard_normal((50, 3)).astype(np.float32) for _ in range(3)]
    a2 = [rng.standard_normal((30, 3)).astype(np.float32) for _ in range(3)]
    sim = _sim(n)
    z1, z2 = np.zeros_like(p1), np.zeros_like(p2)
    sim.load_marker_particle_data(50, p1.tobytes(), z1.tobytes())
    sim.load_marker_particle_data(30, p2.tobytes(), z2.tobytes())
    sim.load_marker_particle_affine_data(50, *(a.tobytes() for a in a1))
    sim.load_marker_particle_affine_data(30, *(a.tobytes() for a in a2))
    sim.initialize()
    assert sim.get_num_marker_particles() == 79
    keep2 = np.ones(30, bool); keep2[3] = False
    for c, name in enumerate("xyz"):
        got = np.frombuffer(getattr(sim, "get_marker_particle_affine%s_data_range" % name)(0, 79), np.float32)
        want = np.concatenate([a1[c], a2[c][keep2]])
        assert np.array_equal(got.reshape(-1, 3), want)
    # after initialisation an affine batch pairs with the batch loaded just before it
    p3 = (0.2 + 0.6 * rng.random((5, 3))).astype(np.float32)
    a3 = [rng.standard_normal((5, 3)).astype(np.float32) for _ in range(3)]
    sim.load_marker_particle_data(5, p3.tobytes(), np.zeros_like(p3).tobytes())
    sim.load_marker_particle_affine_data(5, *(a.tobytes() for a in a3))
    got = np.frombuffer(sim.get_marker_particle_affinez_data_range(79, 84), np.float32).reshape(-1, 3)
    assert np.array_equal(got, a3[2])


def test_unpaired_affine_batches_start_at_zero():
    sim = _sim(8)
    p = np.full((4, 3), 0.5, np.float32)
    sim.load_marker_particle_data(4, p.tobytes(), p.tobytes())
    sim.load_marker_particle_data(4, p.tobytes(), p.tobytes())
    a = np.ones((4, 3), np.float32).tobytes()
    sim.load_marker_particle_affine_data(4, a, a, a)   # one affine batch for two particle batches
    sim.initialize()
    assert not np.frombuffer(sim.get_marker_particle_affinex_data_range(0, 8), np.float32).any()


def test_affine_getters_need_apic():
    sim = _sim(8, apic=False)
    p = np.full((4, 3), 0.5, np.float32)
    sim.load_marker_particle_data(4, p.tobytes(), p.tobytes())
    sim.initialize()
    with pytest.raises(RuntimeError, match="AFFINEX"):
        sim.get_marker_particle_affinex_data_range(0, 4)


def test_apic_frame_through_update_matches_substeps():
    """FluidSimulation_update with APIC runs the same substep as the stage-level entry point."""
    d = dict(np.load(golden_path("apic20")))
    n, dx = int(d["n"]), float(d["dx"])
    sim = _sim(n)
    sim.enable_extreme_velocity_removal = False
    sim.add_body_force(0.0, -9.81, 0.0)
    pos, vel, aff = d["in_pos"], d["in_vel"], d["in_aff"].reshape(-1, 3, 3)
    sim.load_marker_particle_data(pos.shape[0], pos.tobytes(), vel.tobytes())
    sim.load_marker_particle_affine_data(pos.shape[0], *(np.ascontiguousarray(aff[:, c]).tobytes() for c in range(3)))
    sim.initialize()
    sim.update(float(d["dt"]))
    st = sim.get_frame_stats_data()
    assert st.substeps == 1 and st.pressureSolverSuccess == 1
    gp, gv, ga, _ = G.substep_apic(n, dx, float(d["dt"]), 5, (0.0, -9.81, 0.0), O.solid_level_set(n, dx), pos, vel,
                                   d["in_aff"])
    m = sim.get_num_marker_particles()
    assert m == gp.shape[0]
    x = np.frombuffer(sim.get_marker_particle_position_data(), np.float32).reshape(-1, 3)
    ax = np.frombuffer(sim.get_marker_particle_affinex_data_range(0, m), np.float32).reshape(-1, 3)
    assert np.array_equal(x, gp) and np.array_equal(ax, ga[:, 0:3])


def test_differentiable_substep_rejects_apic():
    sim = _sim(8)
    p = np.full((4, 3), 0.5, np.float32)
    sim.load_marker_particle_data(4, p.tobytes(), p.tobytes())
    sim.initialize()
    with pytest.raises(RuntimeError, match="FLIP velocity transfer"):
        sim.substep_differentiable(1 / 240)
