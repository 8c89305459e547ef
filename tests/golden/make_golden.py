"""Generates the golden vectors under tests/golden/ by running the reference engine.

The reference engine (rlguy/Blender-FLIP-Fluids src/engine, unmodified) is compiled by
oracle/build_ref.sh into oracle/_ref/, together with oracle/ref_harness.cpp, which drives
one FluidSimulation through the per-substep hot path and dumps every intermediate array.
This script writes the seeded scene inputs, runs the harness and packs its outputs into
compressed .npz fixtures with a SHA-256 manifest.  It needs the reference sources, so it
runs only where they are present; the fixtures it writes are committed and travel alone.

Usage: python tests/golden/make_golden.py [--ref REFERENCE_ROOT] [--skip-build]
(REFERENCE_ROOT defaults to FFGPU_REFERENCE_ROOT, else a checkout named "reference" beside the repo)
"""
import argparse
import hashlib
import json
import os
import struct
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "blender-flip-fluids_gb300"))
from ffengine_gb300 import scenes  # noqa: E402

HARNESS = os.path.join(ROOT, "oracle", "_ref", "ref_harness")

# name: (mode, n, xb, yb, velocity_sigma, sphere or None, substeps[, affine sigma for the APIC transfer
#        or None[, constant viscosity or None[, dump the surface curvature grid[, surface tension
#        or None[, options]]]]])
# options: "steps": (min, max) time steps per frame (default 1, 1); "frame_dt": the update's delta
# time (default DT); "evr": extreme-velocity removal on; "outliers": speeds given to evenly spaced
# particles (seeded random directions), so that the removal rule has fast particles to act on;
# "ffp3": (output flags, output amount): FFP3 fluid-particle output on, with seeded uint16 particle
# ids loaded beside the particles (flags bit0..2 surface, boundary, interior, bit3 velocity, bit4
# speed attribute); every update's FFP3 data and the particles after it are stored.
CASES = {
    "dam20": ("stages", 20, 0.4, 0.6, 0.0, None, 1),
    "rand20": ("stages", 20, 0.4, 0.6, 0.5, None, 1),
    "sphere24": ("stages", 24, 0.7, 0.45, 1.0, (0.6, 0.3, 0.5, 0.15), 1),
    "traj16": ("traj", 16, 0.4, 0.6, 0.0, None, 30),
    "traj64": ("traj", 64, 0.4, 0.6, 0.0, None, 100),
    "apic20": ("stages", 20, 0.4, 0.6, 0.5, None, 1, 10.0),
    "apicsphere24": ("stages", 24, 0.7, 0.45, 1.0, (0.6, 0.3, 0.5, 0.15), 1, 10.0),
    "apictraj16": ("traj", 16, 0.4, 0.6, 0.0, None, 20, 0.0),
    "visc20": ("stages", 20, 0.4, 0.6, 0.5, None, 1, None, 1.0),
    "viscsphere24": ("stages", 24, 0.7, 0.45, 1.0, (0.6, 0.3, 0.5, 0.15), 1, None, 4.0),
    "visctraj16": ("traj", 16, 0.4, 0.6, 0.0, None, 20, None, 1.0),
    "curv20": ("stages", 20, 0.4, 0.6, 0.5, None, 1, None, None, True),
    "curvsphere24": ("stages", 24, 0.7, 0.45, 1.0, (0.6, 0.3, 0.5, 0.15), 1, None, None, True),
    "tension20": ("stages", 20, 0.4, 0.6, 0.5, None, 1, None, None, True, 0.05),
    "tensionsphere24": ("stages", 24, 0.7, 0.45, 1.0, (0.6, 0.3, 0.5, 0.15), 1, None, None, True, 0.2),
    "tensiontraj16": ("traj", 16, 0.4, 0.6, 0.0, None, 20, None, None, False, 0.05),
    # CFL substepping through update(): per-frame substep counts and lengths.  1..6 substeps per
    # 1/6 s frame; 1..3 (the last substep takes the remainder when the limit is hit); 2..4 with
    # the sphere (the minimum caps each substep at half the frame)
    "cfltraj16": ("traj", 16, 0.4, 0.6, 0.0, None, 12, None, None, False, None,
                  {"steps": (1, 6), "frame_dt": 1.0 / 6.0}),
    "cflmaxtraj16": ("traj", 16, 0.4, 0.6, 1.0, None, 12, None, None, False, None,
                     {"steps": (1, 3), "frame_dt": 1.0 / 6.0}),
    "cflmin20": ("traj", 20, 0.5, 0.5, 1.0, (0.6, 0.3, 0.5, 0.15), 8, None, None, False, None,
                 {"steps": (2, 4), "frame_dt": 1.0 / 8.0}),
    # extreme-velocity removal on (the drop-in's default): one substep with the stages dumped,
    # and a trajectory through update()
    "evr20": ("stages", 20, 0.4, 0.6, 0.5, None, 1, None, None, False, None,
              {"steps": (1, 6), "evr": True, "outliers": (70, 130, 200, 260, 330, 380, 420, 450, 455, 460,
                                                           470, 480)}),
    "evrtraj16": ("traj", 16, 0.4, 0.6, 0.5, None, 20, None, None, False, None,
                  {"evr": True, "outliers": (40, 55, 80, 90, 95, 96, 97, 98)}),
    # FFP3 fluid-particle output: every type and attribute, ids above half the id range left out
    # (with the sphere); surface and interior particles only, the full id range
    "ffp3traj20": ("traj", 20, 0.45, 0.6, 0.5, (0.6, 0.3, 0.5, 0.15), 4, None, None, False, None,
                   {"ffp3": (31, 0.5)}),
    "ffp3traj16": ("traj", 16, 0.4, 0.6, 0.0, None, 3, None, None, False, None, {"ffp3": (21, 1.0)}),
}


# Solid level sets of static mesh obstacles ("mesh" harness mode): n, then (mesh, flags, mesh
# expansion) per obstacle; flags bit0 inversed, bit1 disabled.
def _mesh_cases():
    ico = scenes.icosphere(0.6, 0.3, 0.5, 0.15, 4)
    d32 = 1.0 / 32
    return {
        # the sphere of the *sphere24 scenes as a mesh obstacle
        "meshsphere24": (24, [(ico, 0, 0.0)]),
        # a torus, a box through the domain boundary, a box whose corners lie on grid nodes, a
        # disabled box and an inverted sphere (liquid only inside it)
        "meshmix32": (32, [(scenes.torus(0.45, 0.5, 0.55, 0.22, 0.07), 0, 0.0),
                           (scenes.box_mesh((-0.2, 0.1, 0.2), (0.3, 0.35, 0.6)), 0, 0.0),
                           (scenes.box_mesh((8 * d32, 4 * d32, 16 * d32), (16 * d32, 8 * d32, 24 * d32)), 0, 0.0),
                           (scenes.box_mesh((0.6, 0.6, 0.6), (0.8, 0.8, 0.8)), 2, 0.0),
                           (scenes.icosphere(0.5, 0.5, 0.5, 0.47, 3), 1, 0.0)]),
        # 30 islands in one object (the per-island path, with mesh expansion) and 10 in another
        # (one level set of the whole mesh; the expansion is not applied there)
        "meshislands20": (20, [(scenes.scattered_boxes(30, (0.05, 0.05, 0.05), (0.95, 0.95, 0.95), 0.07, seed=3),
                                0, 0.03),
                               (scenes.scattered_boxes(10, (0.1, 0.1, 0.1), (0.9, 0.5, 0.9), 0.09, seed=4),
                                0, 0.03)]),
    }


MESH_CASES = _mesh_cases()


def run_mesh_case(name, spec, tmp):
    n, objs = spec
    inp = os.path.join(tmp, name + ".in")
    out = os.path.join(tmp, name)
    os.makedirs(out, exist_ok=True)
    with open(inp, "wb") as f:
        f.write(struct.pack("<idi", n, 1.0 / n, len(objs)))
        for (v, t), flags, exp in objs:
            f.write(struct.pack("<ifii", flags, exp, len(v), len(t)))
            f.write(np.ascontiguousarray(v, dtype="<f4").tobytes())
            f.write(np.ascontiguousarray(t, dtype="<i4").tobytes())
    subprocess.run([HARNESS, "mesh", inp, out], check=True)
    n1 = n + 1
    arrays = {"n": np.int32(n), "dx": np.float64(1.0 / n),
              "nverts": np.array([len(v) for (v, t), _, _ in objs], np.int32),
              "ntris": np.array([len(t) for (v, t), _, _ in objs], np.int32),
              "verts": np.concatenate([np.asarray(v, np.float32) for (v, t), _, _ in objs]),
              "tris": np.concatenate([np.asarray(t, np.int32) for (v, t), _, _ in objs]),
              "flags": np.array([fl for _, fl, _ in objs], np.int32),
              "expansion": np.array([e for _, _, e in objs], np.float32),
              "solid_phi": load_bin(out, "solid_phi", "<f4", (n1, n1, n1)),
              "rand_calls": load_bin(out, "rand_calls", "<i8"),
              "jitter": load_bin(out, "jitter", "<f4"), "draw_order": load_bin(out, "draw_order", "<f4")}
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, **arrays)
    with open(path, "rb") as f:
        return hashlib.sha256(f.read()).hexdigest()


def affine_input(np_, sigma, seed=7):
    """Seeded affine vectors (9 floats per particle: x, y, z component vectors), N(0, sigma^2)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    return (rng.standard_normal((np_, 9)) * sigma).astype(np.float32)
DT = 1.0 / 240.0
PIC = 0.05
CFL = 5


def add_outliers(vel, speeds, seed=11):
    """Evenly spaced particles get the given speeds along seeded random directions."""
    vel = vel.copy()
    rng = np.random.Generator(np.random.PCG64(seed))
    stride = vel.shape[0] // (len(speeds) + 1)
    for q, sp in enumerate(speeds):
        d = rng.standard_normal(3)
        vel[(q + 1) * stride] = (sp * d / np.linalg.norm(d)).astype(np.float32)
    return vel


def particle_ids(np_, seed=5):
    """Seeded uint16 particle ids, uniform over the id range."""
    rng = np.random.Generator(np.random.PCG64(seed))
    return rng.integers(0, 65536, np_, dtype=np.uint16)


def write_input(path, n, pos, vel, sphere, substeps, aff=None, visc=None, curvature=False, tension=None,
                opts=None, ids=None):
    opts = opts or {}
    flags = ((1 if sphere else 0) | (2 if aff is not None else 0) | (4 if visc is not None else 0) |
             (8 if curvature else 0) | (16 if tension is not None else 0) | (32 if "steps" in opts else 0) |
             (64 if opts.get("evr") else 0) | (256 if "ffp3" in opts else 0))
    sc = sphere if sphere else (0.0, 0.0, 0.0, 0.0)
    with open(path, "wb") as f:
        f.write(struct.pack("<iiii", n, pos.shape[0], flags, substeps))
        f.write(struct.pack("<dddi", 1.0 / n, opts.get("frame_dt", DT), PIC, CFL))
        f.write(struct.pack("<dddd", *sc))
        f.write(np.ascontiguousarray(pos, dtype="<f4").tobytes())
        f.write(np.ascontiguousarray(vel, dtype="<f4").tobytes())
        if aff is not None:
            f.write(np.ascontiguousarray(aff, dtype="<f4").tobytes())
        if visc is not None:
            f.write(struct.pack("<d", visc))
        if tension is not None:
            f.write(struct.pack("<d", tension))
        if "steps" in opts:
            f.write(struct.pack("<ii", *opts["steps"]))
        if "ffp3" in opts:
            f.write(struct.pack("<id", *opts["ffp3"]))
            f.write(np.ascontiguousarray(ids, dtype="<u2").tobytes())


def load_bin(d, name, dtype, shape=None):
    a = np.fromfile(os.path.join(d, name + ".bin"), dtype=dtype)
    return a.reshape(shape) if shape is not None else a


def moments(pos, vel):
    v2 = (vel.astype(np.float64) ** 2).sum(axis=1)
    return np.concatenate([[pos.shape[0]], pos.astype(np.float64).mean(axis=0),
                           vel.astype(np.float64).mean(axis=0), [v2.mean(), np.sqrt(v2.max())]])


def run_case(name, spec, tmp):
    mode, n, xb, yb, sigma, sphere, substeps = spec[:7]
    apic = len(spec) > 7 and spec[7] is not None
    visc = spec[8] if len(spec) > 8 else None
    curvature = bool(spec[9]) if len(spec) > 9 else False
    tension = spec[10] if len(spec) > 10 else None
    opts = spec[11] if len(spec) > 11 else {}
    pos, vel = scenes.dam_break_particles(n, xb, yb, seed=0, velocity_sigma=sigma)
    if "outliers" in opts:
        vel = add_outliers(vel, opts["outliers"])
    aff = affine_input(pos.shape[0], spec[7]) if apic else None
    ids = particle_ids(pos.shape[0]) if "ffp3" in opts else None
    inp = os.path.join(tmp, name + ".in")
    out = os.path.join(tmp, name)
    os.makedirs(out, exist_ok=True)
    write_input(inp, n, pos, vel, sphere, substeps, aff, visc, curvature, tension, opts, ids)
    subprocess.run([HARNESS, mode, inp, out], check=True)
    arrays = {"n": np.int32(n), "dx": np.float64(1.0 / n), "dt": np.float64(opts.get("frame_dt", DT)),
              "pic": np.float64(PIC), "cfl": np.int32(CFL),
              "sphere": np.array(sphere if sphere else (0, 0, 0, 0), np.float64),
              "has_sphere": np.int32(1 if sphere else 0),
              "in_pos": pos, "in_vel": vel, "apic": np.int32(1 if apic else 0)}
    if apic:
        arrays["in_aff"] = aff
    if visc is not None:
        arrays["viscosity"] = np.float64(visc)
    if tension is not None:
        arrays["surface_tension"] = np.float64(tension)
    steps = opts.get("steps", (1, 1))
    arrays["min_steps"], arrays["max_steps"] = np.int32(steps[0]), np.int32(steps[1])
    arrays["evr"] = np.int32(1 if opts.get("evr") else 0)
    if "ffp3" in opts:
        arrays["in_ids"] = ids
        arrays["ffp3_flags"], arrays["ffp3_amount"] = np.int32(opts["ffp3"][0]), np.float64(opts["ffp3"][1])
    n1 = n + 1
    if mode == "stages":
        grids_c = ["liquid_phi_raw", "liquid_phi", "pressure"]
        for g in grids_c:
            arrays[g] = load_bin(out, g, "<f4", (n, n, n))
        arrays["solid_phi"] = load_bin(out, "solid_phi", "<f4", (n1, n1, n1))
        shapes = {"u": (n, n, n1), "v": (n, n1, n), "w": (n1, n, n)}  # [k][j][i]
        for pre in ["p2g", "adv", "body", "proj", "projx", "cons", "saved"]:
            for c in "uvw":
                arrays[f"{pre}_{c}"] = load_bin(out, f"{pre}_{c}", "<f4", shapes[c])
        for pre in ["p2g", "proj"]:
            for c in "uvw":
                arrays[f"{pre}_valid{c}"] = load_bin(out, f"{pre}_valid{c}", "u1", shapes[c])
        for c in "uvw":
            arrays[f"weight_{c}"] = load_bin(out, f"weight_{c}", "<f4", shapes[c])
        arrays["solid_velocity_absmax"] = load_bin(out, "solid_velocity_absmax", "<f4")
        arrays["pressure_iters"] = load_bin(out, "pressure_iters", "<i4")
        arrays["pressure_error"] = load_bin(out, "pressure_error", "<f4")
        arrays["p0_pos"] = load_bin(out, "p0_pos", "<f4", (-1, 3))
        arrays["g2p_vel"] = load_bin(out, "g2p_vel", "<f4", (-1, 3))
        arrays["adv_pos"] = load_bin(out, "adv_pos", "<f4", (-1, 3))
        arrays["p1_pos"] = load_bin(out, "p1_pos", "<f4", (-1, 3))
        arrays["p1_vel"] = load_bin(out, "p1_vel", "<f4", (-1, 3))
        if apic:
            arrays["g2p_aff"] = load_bin(out, "g2p_aff", "<f4", (-1, 9))
            arrays["p1_aff"] = load_bin(out, "p1_aff", "<f4", (-1, 9))
        if opts.get("evr"):
            arrays["speed_limit"] = load_bin(out, "speed_limit", "<f4")
        if curvature:
            arrays["surface_phi"] = load_bin(out, "surface_phi", "<f4", (n, n, n))
            arrays["curvature"] = load_bin(out, "curvature", "<f4", (n, n, n))
        if visc is not None:
            for pre in ["visc_in", "visc"]:
                for c in "uvw":
                    arrays[f"{pre}_{c}"] = load_bin(out, f"{pre}_{c}", "<f4", shapes[c])
            vshapes = {"center": (n, n, n), "u": shapes["u"], "v": shapes["v"], "w": shapes["w"],
                       "eu": (n1, n1, n), "ev": (n1, n, n1), "ew": (n, n1, n1)}
            for g, shp in vshapes.items():
                arrays["visc_vol_" + g] = load_bin(out, "visc_vol_" + g, "<f4", shp)
            arrays["visc_index"] = load_bin(out, "visc_index", "<i4")
            arrays["visc_stats"] = load_bin(out, "visc_stats", "<i4")
            arrays["visc_error"] = load_bin(out, "visc_error", "<f4")
            if int(arrays["visc_stats"][0]) > 0:
                for g, dt_ in [("rowstart", "<u4"), ("col", "<u4"), ("val", "<f4"), ("rhs", "<f4"),
                               ("ic_invdiag", "<f4"), ("ic_colstart", "<u4"), ("ic_rowindex", "<u4"),
                               ("ic_value", "<f4"), ("soln", "<f4")]:
                    arrays["visc_" + g] = load_bin(out, "visc_" + g, dt_)
    else:
        arrays["solid_phi"] = load_bin(out, "solid_phi", "<f4", (n1, n1, n1))
        stats = load_bin(out, "traj_stats", "<f8", (substeps, 4))
        arrays["traj_stats"] = stats
        arrays["traj_steps"] = load_bin(out, "traj_steps", "<f8", (substeps, 2))
        arrays["traj_dts"] = load_bin(out, "traj_dts", "<f8")
        mom = []
        for s in range(substeps):
            p = load_bin(out, "traj%03d_pos" % (s + 1), "<f4", (-1, 3))
            v = load_bin(out, "traj%03d_vel" % (s + 1), "<f4", (-1, 3))
            mom.append(moments(p, v))
        arrays["traj_moments"] = np.array(mom)
        if "ffp3" in opts:
            fl = opts["ffp3"][0]
            for s in range(substeps):
                t = "traj%03d" % (s + 1)
                arrays["ffp3_%d_pos" % s] = load_bin(out, t + "_pos", "<f4", (-1, 3))
                arrays["ffp3_%d_vel" % s] = load_bin(out, t + "_vel", "<f4", (-1, 3))
                arrays["ffp3_%d_ids" % s] = load_bin(out, t + "_ids", "<u2")
                for tag, bit in (("pos", 0), ("id", 0), ("vel", 8), ("speed", 16)):
                    if bit == 0 or fl & bit:
                        arrays["ffp3_%d_data_%s" % (s, tag)] = load_bin(out, t + "_ffp_" + tag, "u1")
        # final state: full for small grids, every 64th particle for large ones
        stride = 1 if n <= 16 else 64
        arrays["final_stride"] = np.int32(stride)
        arrays["final_pos"] = p[::stride].copy()
        arrays["final_vel"] = v[::stride].copy()
        if apic:
            a = load_bin(out, "traj%03d_aff" % substeps, "<f4", (-1, 9))
            arrays["final_aff"] = a[::stride].copy()
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, **arrays)
    with open(path, "rb") as f:
        return hashlib.sha256(f.read()).hexdigest()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("FFGPU_REFERENCE_ROOT") or
                    os.path.join(os.path.dirname(ROOT), "reference"))
    ap.add_argument("--skip-build", action="store_true")
    ap.add_argument("--cases", nargs="*", default=list(CASES) + list(MESH_CASES))
    args = ap.parse_args()
    if not args.skip_build:
        subprocess.run([os.path.join(ROOT, "oracle", "build_ref.sh"), args.ref], check=True)
    manifest_path = os.path.join(HERE, "MANIFEST.json")
    manifest = json.load(open(manifest_path)) if os.path.exists(manifest_path) else {}
    with tempfile.TemporaryDirectory() as tmp:
        for name in args.cases:
            if name in MESH_CASES:
                n_, objs = MESH_CASES[name]
                manifest[name + ".npz"] = {"sha256": run_mesh_case(name, MESH_CASES[name], tmp),
                                           "spec": [str(n_)] + ["%d triangles, flags %d, expansion %g" %
                                                                (len(m[1]), fl, e) for m, fl, e in objs],
                                           "generator": "tests/golden/make_golden.py",
                                           "engine": "rlguy/Blender-FLIP-Fluids 1.8.5 src/engine"}
                print("wrote", name)
                continue
            manifest[name + ".npz"] = {"sha256": run_case(name, CASES[name], tmp),
                                       "spec": list(map(str, CASES[name])),
                                       "generator": "tests/golden/make_golden.py",
                                       "engine": "rlguy/Blender-FLIP-Fluids 1.8.5 src/engine"}
            print("wrote", name)
    with open(manifest_path, "w") as f:
        json.dump(manifest, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
