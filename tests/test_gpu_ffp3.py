"""GPU parity of the FFP3 fluid-particle output (FluidSimulation::_classifyFluidParticleTypes,
_generateFluidParticleDataFFP3 and its file data, fluidsimulation.cpp:9477-9800) against the
reference engine's golden output and the CPU oracle.

Bars:
  the output of a given particle state (liquid level set, surface level set, classification,
    grouping, bytes)                                     -- bit-exact against the reference's bytes;
  through update() with ids loaded                       -- the bytes bit-exact against the oracle
    applied to the GPU's own particles after each update; the particle ids carried through the
    removal as the reference carries them; the type counts of the first output within a few
    particles of the reference's (the trajectories round differently);
  the API: settings, amount clamping, empty output before the first update, sizes.
"""
import numpy as np
import pytest

import gpu_api as G
import oracle_api as O
from conftest import golden_path

pytestmark = pytest.mark.gpu

CASES = ["ffp3traj20", "ffp3traj16"]


@pytest.mark.parametrize("name", CASES)
def test_ffp3_of_reference_state_bitexact(name):
    d = dict(np.load(golden_path(name)))
    n, dx = int(d["n"]), float(d["dx"])
    flags, amount = int(d["ffp3_flags"]), float(d["ffp3_amount"])
    for s in range(int(d["traj_stats"].shape[0])):
        pos, vel, ids = d["ffp3_%d_pos" % s], d["ffp3_%d_vel" % s], d["ffp3_%d_ids" % s]
        types, data = G.ffp3(n, dx, d["solid_phi"], pos, vel, ids, flags, amount)
        for tag in ("pos", "id", "vel", "speed"):
            key = "ffp3_%d_data_%s" % (s, tag)
            if key in d:
                assert np.array_equal(data[tag], d[key]), (s, tag)
            else:
                assert data[tag].size == 0
        # the same classification as the oracle's
        surface = O.surface_level_set(n, dx, d["solid_phi"], pos)
        otypes, _ = O.ffp3(n, dx, surface, pos, vel, ids, flags & 7, amount)
        assert np.array_equal(types, otypes)


def make(d):
    import ffengine_gb300 as ffe
    n = int(d["n"])
    sim = ffe.FluidSimulation(n, n, n, 1.0 / n)
    sim.enable_extreme_velocity_removal = False
    sim.add_body_force(0.0, -9.81, 0.0)
    flags = int(d["ffp3_flags"])
    sim.enable_fluid_particle_output = True
    sim.enable_fluid_particle_surface_output = bool(flags & 1)
    sim.enable_fluid_particle_boundary_output = bool(flags & 2)
    sim.enable_fluid_particle_interior_output = bool(flags & 4)
    sim.enable_fluid_particle_velocity_attribute = bool(flags & 8)
    sim.enable_fluid_particle_speed_attribute = bool(flags & 16)
    sim.fluid_particle_output_amount = float(d["ffp3_amount"])
    pos, vel, ids = d["in_pos"], d["in_vel"], d["in_ids"]
    sim.load_marker_particle_data(pos.shape[0], pos.tobytes(), vel.tobytes())
    sim.load_marker_particle_id_data(ids.shape[0], ids.tobytes())
    sim.initialize()
    if int(d["has_sphere"]):
        sim.set_solid_level_set(np.ascontiguousarray(d["solid_phi"], np.float32).tobytes())
    return sim


@pytest.mark.parametrize("name", CASES)
def test_ffp3_through_update(name):
    d = dict(np.load(golden_path(name)))
    n, dx = int(d["n"]), float(d["dx"])
    flags, amount = int(d["ffp3_flags"]), float(d["ffp3_amount"])
    sim = make(d)
    assert sim.get_fluid_particle_data() == b""   # no output before the first update
    for s in range(int(d["traj_stats"].shape[0])):
        sim.update(float(d["dt"]))
        m = sim.get_num_marker_particles()
        pos = np.frombuffer(sim.get_marker_particle_position_data(), np.float32).reshape(-1, 3)
        vel = np.frombuffer(sim.get_marker_particle_velocity_data(), np.float32).reshape(-1, 3)
        ids = np.frombuffer(sim.get_marker_particle_id_data_range(0, m), np.uint16)
        surface = O.surface_level_set(n, dx, d["solid_phi"], pos)
        _, want = O.ffp3(n, dx, surface, pos, vel, ids, flags & 7, amount)
        got = {"pos": sim.get_fluid_particle_data(), "id": sim.get_fluid_particle_id_attribute_data(),
               "vel": sim.get_fluid_particle_velocity_attribute_data(),
               "speed": sim.get_fluid_particle_speed_attribute_data()}
        for tag, bit in (("pos", 0), ("id", 0), ("vel", 8), ("speed", 16)):
            if bit and not flags & bit:
                assert got[tag] == b""
            else:
                assert got[tag] == want[tag].tobytes(), (s, tag)
        ref_ids = d["ffp3_%d_ids" % s]
        if ref_ids.size == m:   # the same particles removed: the ids follow them
            assert np.array_equal(ids, ref_ids), s
        if s == 0:
            head = np.frombuffer(got["pos"][:16], np.uint32)
            rhead = d["ffp3_0_data_pos"].view(np.uint32)[:4]
            assert head[3] == rhead[3]
            assert np.abs(head[:3].astype(np.int64) - rhead[:3].astype(np.int64)).max() <= 8


def test_ffp3_settings():
    import ffengine_gb300 as ffe
    sim = ffe.FluidSimulation(8, 8, 8, 1 / 8)
    assert not sim.enable_fluid_particle_output
    assert sim.enable_fluid_particle_surface_output and sim.enable_fluid_particle_boundary_output
    assert sim.enable_fluid_particle_interior_output
    assert not sim.enable_fluid_particle_velocity_attribute and not sim.enable_fluid_particle_speed_attribute
    assert sim.fluid_particle_output_amount == 1.0
    sim.fluid_particle_output_amount = 2.5
    assert sim.fluid_particle_output_amount == 1.0   # clamped as the reference clamps
    sim.fluid_particle_output_amount = 0.25
    assert sim.fluid_particle_output_amount == 0.25
    with pytest.raises(RuntimeError, match="amount must be greater"):
        sim.fluid_particle_output_amount = -0.1
    sim.enable_fluid_particle_boundary_output = False
    assert not sim.enable_fluid_particle_boundary_output


def test_ffp3_random_ids_and_amount_zero():
    """Without id data the particles get ids drawn uniformly from 0..65535; an output amount of 0
    writes the header alone."""
    import ffengine_gb300 as ffe
    from ffengine_gb300 import scenes
    n = 16
    pos, vel = scenes.dam_break_particles(n, 0.4, 0.6, seed=1)
    sim = ffe.FluidSimulation(n, n, n, 1.0 / n)
    sim.enable_fluid_particle_output = True
    sim.load_marker_particle_data(pos.shape[0], pos.tobytes(), vel.tobytes())
    sim.initialize()
    m = sim.get_num_marker_particles()
    ids = np.frombuffer(sim.get_marker_particle_id_data_range(0, m), np.uint16)
    assert ids.size == m and len(np.unique(ids)) > 0.9 * min(m, 65536) * (1 - m / 131072)
    sim.fluid_particle_output_amount = 0.0
    sim.update(1.0 / 240)
    data = sim.get_fluid_particle_data()
    assert len(data) == 16 and np.array_equal(np.frombuffer(data, np.uint32), [0, 0, 0, 0])


def test_ffp3_classification_dense_ball():
    """Classification of ~160k particles of a jittered ball against the oracle's (double trilinear
    sample of the surface level set): the GPU decides most particles on a float sample and falls back
    to the double one near the surface-width threshold; every type must agree."""
    n = 48
    dx = 1.0 / n
    rng = np.random.default_rng(7)
    g = (np.stack(np.meshgrid(*[np.arange(n)] * 3, indexing="ij"), -1).reshape(-1, 3) + 0.5) * dx
    inside = np.linalg.norm(g - 0.5, axis=1) < 0.35
    pos = (np.repeat(g[inside], 8, 0) + rng.uniform(-0.5, 0.5, (8 * int(inside.sum()), 3)) * dx).astype(np.float32)
    vel = rng.standard_normal(pos.shape).astype(np.float32)
    ids = rng.integers(0, 65536, pos.shape[0]).astype(np.uint16)
    solid = O.solid_phi(n, dx)
    types, _ = G.ffp3(n, dx, solid, pos, vel, ids, 7, 1.0)
    surface = O.surface_level_set(n, dx, solid, pos)
    otypes, _ = O.ffp3(n, dx, surface, pos, vel, ids, 7, 1.0)
    assert pos.shape[0] > 100000
    assert np.array_equal(types, otypes)
    assert (types == 0).sum() > 0 and (types == 2).sum() > 0
