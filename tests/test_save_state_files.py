"""Save-state particle files: the GPU writer against the bake script's own writer loop, and the
GPU loader against its loader loop.

The reference writes each marker-particle attribute of a save state by reading particle ranges of
2^21 through the engine's range getters and appending the bytes to one file per attribute
(src/addon/bake.py:2864-2905), and reads them back in the same 2^21-particle batches through
load_marker_particle_data / load_marker_particle_affine_data (bake.py:554-721).  Those two loops
are restated here, over this library's own range getters and loaders, as the reference
behaviour; the GPU writer and loader must produce the same bytes and the same state.
"""
import os

import numpy as np
import pytest

import ffengine_gb300 as ffe
import oracle_api as O
from ffengine_gb300 import scenes

pytestmark = pytest.mark.gpu

CHUNK = 2 ** 21
ATTRS = ["position", "velocity", "affinex", "affiney", "affinez"]


def bake_write(sim, directory):
    """bake.py:2864-2905 for position, velocity and (APIC) the affine vectors."""
    n = sim.get_num_marker_particles()
    getters = {"position": sim.get_marker_particle_position_data_range,
               "velocity": sim.get_marker_particle_velocity_data_range}
    if sim.is_velocity_transfer_method_APIC():
        getters.update({"affinex": sim.get_marker_particle_affinex_data_range,
                        "affiney": sim.get_marker_particle_affiney_data_range,
                        "affinez": sim.get_marker_particle_affinez_data_range})
    for i in range(n // CHUNK + 1):
        s, e = i * CHUNK, min((i + 1) * CHUNK, n)
        for name, get in getters.items():
            with open(os.path.join(directory, name + ".data"), "ab" if i else "wb") as f:
                f.write(get(s, e))
    return list(getters)


def bake_load(sim, directory, apic):
    """bake.py:656-690 for position, velocity and (APIC) the affine vectors."""
    rd = lambda name, a, b: open(os.path.join(directory, name + ".data"), "rb").read()[a:b]
    n = os.path.getsize(os.path.join(directory, "position.data")) // 12
    for i in range(n // CHUNK + 1):
        a, b = i * 12 * CHUNK, min((i + 1) * 12 * CHUNK, 12 * n)
        count = (b - a) // 12
        sim.load_marker_particle_data(count, rd("position", a, b), rd("velocity", a, b))
        if apic:
            sim.load_marker_particle_affine_data(count, rd("affinex", a, b), rd("affiney", a, b), rd("affinez", a, b))


def make(n, apic, xb=0.4, yb=0.6, steps=1):
    pos, vel = scenes.dam_break_particles(n, xb, yb, seed=0, velocity_sigma=0.3)
    sim = ffe.FluidSimulation(n, n, n, 1.0 / n)
    if apic:
        sim.set_velocity_transfer_method_APIC()
    sim.enable_extreme_velocity_removal = False
    sim.add_body_force(0.0, -9.81, 0.0)
    sim.load_marker_particle_data(pos.shape[0], pos.tobytes(), vel.tobytes())
    sim.initialize()
    for _ in range(steps):
        sim.update(1.0 / 240.0)
    return sim


def state(sim):
    n = sim.get_num_marker_particles()
    out = [sim.get_marker_particle_position_data(), sim.get_marker_particle_velocity_data()]
    if sim.is_velocity_transfer_method_APIC():
        out += [sim.get_marker_particle_affinex_data_range(0, n), sim.get_marker_particle_affiney_data_range(0, n),
                sim.get_marker_particle_affinez_data_range(0, n)]
    return out


# 128^3: 4.03M particles, three chunks of 2^21 (the last one partial)
@pytest.fixture(scope="module", params=[(128, True), (24, False)])
def sim_case(request):
    n, apic = request.param
    return make(n, apic), apic, n


def test_writer_bytes_match_bake_writer(sim_case, tmp_path):
    sim, apic, _ = sim_case
    ref_dir, gpu_dir = tmp_path / "ref", tmp_path / "gpu"
    ref_dir.mkdir(); gpu_dir.mkdir()
    names = bake_write(sim, str(ref_dir))
    assert names == (ATTRS if apic else ATTRS[:2])
    for name in names:
        sim.write_marker_particle_file(name, str(gpu_dir / (name + ".data")))
        a = (ref_dir / (name + ".data")).read_bytes()
        b = (gpu_dir / (name + ".data")).read_bytes()
        assert len(a) == 12 * sim.get_num_marker_particles() and a == b, name


def test_writer_append(sim_case, tmp_path):
    sim = sim_case[0]
    p = str(tmp_path / "pos.data")
    sim.write_marker_particle_file("position", p)
    sim.write_marker_particle_file("position", p, append=True)
    one = sim.get_marker_particle_position_data()
    assert open(p, "rb").read() == one + one


def test_loader_matches_bake_loader(sim_case, tmp_path):
    sim, apic, grid = sim_case
    names = ATTRS if apic else ATTRS[:2]
    for name in names:
        sim.write_marker_particle_file(name, str(tmp_path / (name + ".data")))
    a = ffe.FluidSimulation(grid, grid, grid, 1.0 / grid)
    b = ffe.FluidSimulation(grid, grid, grid, 1.0 / grid)
    if apic:
        a.set_velocity_transfer_method_APIC(); b.set_velocity_transfer_method_APIC()
    bake_load(a, str(tmp_path), apic)
    paths = [str(tmp_path / (x + ".data")) for x in names]
    count = b.load_marker_particle_files(*paths) if apic else b.load_marker_particle_files(paths[0], paths[1])
    assert count == sim.get_num_marker_particles()
    a.initialize(); b.initialize()
    sa, sb = state(a), state(b)
    assert all(x == y for x, y in zip(sa, sb))
    # each 2^21-particle batch comes back in the reference's load-queue order (a batch larger than
    # one 5e6-byte fragment repeats the first record of a fragment at the next fragment's start)
    want = []
    for k, saved in enumerate(state(sim)):
        arr = np.frombuffer(saved, np.float32).reshape(-1, 3)
        rec = 24 if k < 2 else 36
        want.append(np.concatenate([O.as_loaded(arr[i:i + CHUNK], rec) for i in range(0, arr.shape[0], CHUNK)]
                                   or [arr]).tobytes())
    assert all(x == y for x, y in zip(sb, want))


def test_writer_errors(tmp_path):
    sim = make(12, False, steps=0)
    with pytest.raises(RuntimeError, match="AFFINEX"):
        sim.write_marker_particle_file("affinex", str(tmp_path / "a.data"))
    with pytest.raises(RuntimeError, match="cannot open"):
        sim.write_marker_particle_file("position", str(tmp_path / "missing" / "p.data"))
    with pytest.raises(RuntimeError, match="cannot open"):
        sim.load_marker_particle_files(str(tmp_path / "none.data"), str(tmp_path / "none2.data"))


def test_pinned_buffers_take_the_direct_path(tmp_path):
    """Page-locked host buffers are read by the upload kernels directly (no staging copy): the same
    particles as through pageable buffers; read back into a page-locked buffer."""
    import ctypes
    import numpy as np
    import torch
    from ffengine_gb300 import FluidSimulationMarkerParticleData_t, call
    sim = make(24, False, steps=1)
    n = sim.get_num_marker_particles()
    pos = np.frombuffer(sim.get_marker_particle_position_data(), np.float32).reshape(-1, 3).copy()
    vel = np.frombuffer(sim.get_marker_particle_velocity_data(), np.float32).reshape(-1, 3).copy()
    hp = torch.from_numpy(pos).pin_memory()
    hv = torch.from_numpy(vel[::-1].copy()).pin_memory()
    d = FluidSimulationMarkerParticleData_t()
    d.size = n
    d.positions = ctypes.cast(hp.data_ptr(), ctypes.c_char_p)
    d.velocities = ctypes.cast(hv.data_ptr(), ctypes.c_char_p)
    P = ctypes.c_void_p
    call("FluidSimulation_gb300_set_marker_particle_data", [P, FluidSimulationMarkerParticleData_t], None, sim(), d)
    out = torch.zeros((n, 3), dtype=torch.float32).pin_memory()
    call("FluidSimulation_get_marker_particle_velocity_data", [P, P], None, sim(), out.data_ptr())
    assert np.array_equal(out.numpy(), vel[::-1])
    assert np.array_equal(np.frombuffer(sim.get_marker_particle_position_data(), np.float32).reshape(-1, 3), pos)
