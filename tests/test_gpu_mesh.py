"""GPU solid level set of static mesh obstacles against the reference's own solid level sets, and
the drop-in obstacle path (MeshObject_*, FluidSimulation_add_mesh_obstacle) through update().

Bars: the solid level set bit-exact (band distances, signs, islands, unions); a substep with the
icosphere added as a MeshObject within the substep bars of the other parity tests (positions
5e-6, velocities 2e-4 of max|v|) of the reference's substep with the same obstacle."""
import numpy as np
import pytest

import gpu_api as G
import oracle_api as O
from conftest import golden_path

pytestmark = pytest.mark.gpu


def bits_equal(a, b):
    a = np.ascontiguousarray(a); b = np.ascontiguousarray(b)
    return a.shape == b.shape and np.array_equal(a.view(np.uint32), b.view(np.uint32))


@pytest.mark.parametrize("name", ["meshsphere24", "meshmix32", "meshislands20"])
def test_solid_level_set_bitexact(name):
    d = dict(np.load(golden_path(name)))
    n, dx = int(d["n"]), float(d["dx"])
    assert bits_equal(G.solid_level_set(n, dx, O.mesh_objects(d)), d["solid_phi"])


@pytest.mark.parametrize("name", ["dam20", "traj64", "sphere24", "cflmin20"])
def test_domain_and_sphere_solids_bitexact(name):
    from ffengine_gb300 import scenes
    d = dict(np.load(golden_path(name)))
    n, dx = int(d["n"]), float(d["dx"])
    objs = []
    if int(d["has_sphere"]):
        v, t = scenes.icosphere(*[float(x) for x in d["sphere"]], 4)
        objs = [(v, t, 0, 0.0)]
    assert bits_equal(G.solid_level_set(n, dx, objs), d["solid_phi"])


def test_solid_level_set_random_meshes_vs_oracle():
    """Meshes the goldens do not hold, on a 40^3 grid: a torus through a wall, 40 islands with a
    negative expansion and an inverted box, with the fixed line jitter and with explicit ones."""
    from ffengine_gb300 import scenes
    n, dx = 40, 1.0 / 40
    objs = [(*scenes.torus(0.1, 0.5, 0.5, 0.35, 0.06, nu=48, nv=12), 0, 0.0),
            (*scenes.scattered_boxes(40, (0.2, 0.05, 0.2), (0.8, 0.4, 0.8), 0.05, seed=9), 0, -0.01),
            (*scenes.box_mesh((0.05, 0.05, 0.05), (0.95, 0.9, 0.95)), 1, 0.0)]
    jit = np.random.default_rng(5).uniform(-1e-3 * dx, 1e-3 * dx, (6, 3)).astype(np.float32)
    for j in (None, jit):
        assert bits_equal(G.solid_level_set(n, dx, objs, j), O.solid_level_set(n, dx, objs, j))


def _sim(d, mesh=True):
    import ffengine_gb300 as ffe
    from ffengine_gb300 import scenes
    n = int(d["n"])
    sim = ffe.FluidSimulation(n, n, n, 1.0 / n)
    sim.enable_extreme_velocity_removal = False
    sim.add_body_force(0.0, -9.81, 0.0)
    keep = []
    if mesh and int(d["has_sphere"]):
        v, t = scenes.icosphere(*[float(x) for x in d["sphere"]], 4)
        ob = ffe.MeshObject(n, n, n, 1.0 / n)
        ob.update_mesh_static(ffe.TriangleMesh(v, t))
        sim.add_mesh_obstacle(ob)
        keep.append(ob)
    pos, vel = d["in_pos"], d["in_vel"]
    sim.load_marker_particle_data(pos.shape[0], pos.tobytes(), vel.tobytes())
    sim.initialize()
    return sim, keep


def test_substep_with_mesh_obstacle_vs_reference():
    """sphere24 through the drop-in calls only: the icosphere as a MeshObject, no solid level set
    handed over."""
    d = dict(np.load(golden_path("sphere24")))
    sim, keep = _sim(d)
    sim.update(float(d["dt"]))
    x = np.frombuffer(sim.get_marker_particle_position_data(), np.float32).reshape(-1, 3)
    v = np.frombuffer(sim.get_marker_particle_velocity_data(), np.float32).reshape(-1, 3)
    assert x.shape == d["p1_pos"].shape
    assert np.abs(x - d["p1_pos"]).max() <= 5e-6
    assert np.abs(v - d["p1_vel"]).max() <= 2e-4 * max(np.abs(d["p1_vel"]).max(), 1.0)


def test_disabled_and_removed_obstacles():
    """A disabled obstacle and a removed one leave the substep bit-identical to no obstacle;
    enabling it again changes the result."""
    import ffengine_gb300 as ffe
    d = dict(np.load(golden_path("sphere24")))

    def run(setup):
        sim, keep = _sim(d)
        setup(sim, keep)
        sim.update(float(d["dt"]))
        return np.frombuffer(sim.get_marker_particle_position_data(), np.float32).reshape(-1, 3).copy()

    plain = _sim(d, mesh=False)[0]
    plain.update(float(d["dt"]))
    base = np.frombuffer(plain.get_marker_particle_position_data(), np.float32).reshape(-1, 3).copy()

    def disable(sim, keep):
        keep[0].enable = False

    def remove(sim, keep):
        sim.remove_mesh_obstacle(keep[0])

    def toggle(sim, keep):
        keep[0].enable = False
        keep[0].enable = True

    assert bits_equal(run(disable), base)
    assert bits_equal(run(remove), base)
    with_ob = run(toggle)
    assert with_ob.shape != base.shape or not bits_equal(with_ob, base)


def test_mesh_object_api():
    import ffengine_gb300 as ffe
    from ffengine_gb300 import scenes
    sim = ffe.FluidSimulation(8, 8, 8, 1 / 8)
    ob = ffe.MeshObject(8, 8, 8, 1 / 8)
    assert ob.enable and not ob.inverse and ob.friction == 0.0 and ob.mesh_expansion == 0.0
    ob.inverse = True
    assert ob.inverse
    ob.friction = 3.0
    assert ob.friction == 1.0
    ob.friction = -1.0
    assert ob.friction == 0.0
    ob.mesh_expansion = 0.25
    assert ob.mesh_expansion == 0.25
    v, t = scenes.box_mesh((0.2, 0.2, 0.2), (0.4, 0.4, 0.4))
    ob.update_mesh_static(ffe.TriangleMesh(v, t))
    sim.add_mesh_obstacle(ob)
    with pytest.raises(RuntimeError, match="already been added"):
        sim.add_mesh_obstacle(ob)
    sim.remove_mesh_obstacle(ob)
    with pytest.raises(RuntimeError, match="could not find mesh obstacle"):
        sim.remove_mesh_obstacle(ob)
    bad = t.copy()
    bad[0, 0] = 99
    with pytest.raises(RuntimeError, match="index out of range"):
        ob.update_mesh_static(ffe.TriangleMesh(v, bad))
    with pytest.raises(RuntimeError, match="animated"):
        ob.update_mesh_animated(ffe.TriangleMesh(v, t), ffe.TriangleMesh(v, t), ffe.TriangleMesh(v, t))
    sim.add_mesh_obstacle(ob)
    sim.remove_mesh_obstacles()
    sim.add_mesh_obstacle(ob)
