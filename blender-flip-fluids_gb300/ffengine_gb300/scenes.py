"""Seeded synthetic dam-break scenes for the FLIP substep.

A scene is a cubic MAC grid of n^3 cells with cell width dx = 1/n, filled with marker
particles in an axis-aligned fluid block (x < xb, y < yb, all z).  Each fluid cell holds
8 particles, one per 2x2x2 sub-cell, jittered uniformly inside its sub-cell.  This is the
reference engine's own seeding scheme for new fluid cells (8 particles per cell,
fluidsimulation.cpp:_addMarkerParticlesToCell), written with a portable random stream so
that the same arrays come out on every host.

The random stream is numpy's PCG64 seeded with ``seed``.  Cells are visited in k-j-i
order (i fastest) over the block's cell range i < ceil(xb*n), j < ceil(yb*n); within a
cell the 8 sub-cells are visited with x fastest, then y, then z; each sub-cell draws three
uniforms in [0, 1).  A particle is kept when x < xb and y < yb.
"""
import math

import numpy as np


def dam_break_particles(n, xb, yb, seed=0, velocity_sigma=0.0, zb=1.0):
    """Returns (positions, velocities) as float32 arrays of shape (N, 3).

    velocity_sigma > 0 draws velocities from N(0, velocity_sigma^2) per component from a
    second PCG64 stream seeded with seed + 1 (one normal triple per kept particle, in
    particle order); otherwise velocities are zero.
    """
    dx = 1.0 / n
    ni = min(n, int(math.ceil(xb * n)))
    nj = min(n, int(math.ceil(yb * n)))
    nk = min(n, int(math.ceil(zb * n)))
    rng = np.random.Generator(np.random.PCG64(seed))
    # sub-cell offsets, x fastest then y then z
    sub = np.array([[sx, sy, sz] for sz in range(2) for sy in range(2) for sx in range(2)],
                   dtype=np.float64)
    pos_chunks = []
    # one k-slab at a time keeps peak host memory small at 512^3
    ii, jj = np.meshgrid(np.arange(ni, dtype=np.float64), np.arange(nj, dtype=np.float64),
                         indexing="xy")
    cell_ij = np.stack([ii.ravel(), jj.ravel()], axis=1)   # (nj*ni, 2), i fastest
    for k in range(nk):
        u = rng.random((cell_ij.shape[0], 8, 3))
        cells = np.empty((cell_ij.shape[0], 1, 3))
        cells[:, 0, 0] = cell_ij[:, 0]
        cells[:, 0, 1] = cell_ij[:, 1]
        cells[:, 0, 2] = k
        p = (cells + 0.5 * sub[None, :, :] + 0.5 * u) * dx
        p = p.reshape(-1, 3)
        keep = (p[:, 0] < xb) & (p[:, 1] < yb) & (p[:, 2] < zb)
        pos_chunks.append(p[keep].astype(np.float32))
    pos = np.concatenate(pos_chunks, axis=0) if pos_chunks else np.zeros((0, 3), np.float32)
    if velocity_sigma > 0.0:
        vrng = np.random.Generator(np.random.PCG64(seed + 1))
        vel = (vrng.standard_normal((pos.shape[0], 3)) * velocity_sigma).astype(np.float32)
    else:
        vel = np.zeros_like(pos)
    return np.ascontiguousarray(pos), np.ascontiguousarray(vel)


def floating_block_particles(n, lo=(0.3, 0.3, 0.3), hi=(0.7, 0.62, 0.7), seed=0, velocity_sigma=0.0):
    """A fluid block away from every wall: the particles of dam_break_particles(n, hi[0],
    hi[1], zb=hi[2]) with x > lo[0], y > lo[1] and z > lo[2] (same streams, then filtered).
    With the default box no particle comes near the domain boundary for the first few
    substeps, so none is moved by collision handling."""
    pos, vel = dam_break_particles(n, hi[0], hi[1], seed=seed, velocity_sigma=velocity_sigma, zb=hi[2])
    keep = (pos[:, 0] > lo[0]) & (pos[:, 1] > lo[1]) & (pos[:, 2] > lo[2])
    return np.ascontiguousarray(pos[keep]), np.ascontiguousarray(vel[keep])


# Workloads named by what they are (grid size, fluid block, obstacle, particles per cell).
WORKLOADS = {
    "dam_break_64": dict(n=64, xb=0.4, yb=0.6, sphere=None),
    "dam_break_128": dict(n=128, xb=0.4, yb=0.6, sphere=None),
    "dam_break_sphere_256": dict(n=256, xb=0.35, yb=0.5, sphere=(0.6, 0.3, 0.5, 0.15)),
    "dam_break_sphere_512": dict(n=512, xb=0.4, yb=0.5, sphere=(0.6, 0.3, 0.5, 0.15)),
}


# ---- obstacle meshes (float32 vertices (V, 3), int32 triangles (T, 3)) ----

def icosphere(cx, cy, cz, r, subdiv=4):
    """Subdivided icosahedron of radius r about (cx, cy, cz): the 12 vertices (-1, t, 0) ... with
    t the golden ratio, normalised, each triangle split into four at its normalised edge
    midpoints `subdiv` times (a midpoint is created the first time its edge is met, faces in
    order, edges (a, b), (b, c), (c, a)); vertices are c + r p rounded once to float32."""
    t = (1.0 + math.sqrt(5.0)) / 2.0
    v = [[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t],
         [0, -1, -t], [0, 1, -t], [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]]
    f = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4),
         (11, 10, 2), (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8),
         (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)]

    def unit(p):
        n = math.sqrt(p[0] * p[0] + p[1] * p[1] + p[2] * p[2])
        return [p[0] / n, p[1] / n, p[2] / n]

    v = [unit([float(c) for c in p]) for p in v]
    for _ in range(subdiv):
        mid = {}

        def midpoint(a, b):
            key = (min(a, b), max(a, b))
            if key not in mid:
                v.append(unit([(v[a][q] + v[b][q]) / 2 for q in range(3)]))
                mid[key] = len(v) - 1
            return mid[key]

        nf = []
        for (a0, b0, c0) in f:
            a, b, c = midpoint(a0, b0), midpoint(b0, c0), midpoint(c0, a0)
            nf += [(a0, a, c), (b0, b, a), (c0, c, b), (a, b, c)]
        f = nf
    verts = np.array([[cx + r * p[0], cy + r * p[1], cz + r * p[2]] for p in v], np.float32)
    return verts, np.array(f, np.int32)


def box_mesh(lo, hi):
    """Axis-aligned box (8 vertices, 12 triangles) from corner lo to corner hi."""
    x0, y0, z0 = lo
    x1, y1, z1 = hi
    verts = np.array([[x0, y0, z0], [x1, y0, z0], [x1, y0, z1], [x0, y0, z1],
                      [x0, y1, z0], [x1, y1, z0], [x1, y1, z1], [x0, y1, z1]], np.float32)
    tris = np.array([[0, 1, 2], [0, 2, 3], [4, 7, 6], [4, 6, 5], [0, 3, 7], [0, 7, 4],
                     [1, 5, 6], [1, 6, 2], [0, 4, 5], [0, 5, 1], [3, 2, 6], [3, 6, 7]], np.int32)
    return verts, tris


def torus(cx, cy, cz, major, minor, nu=32, nv=16):
    """Torus about the y axis through (cx, cy, cz): nu x nv quads split into triangles."""
    u = 2.0 * np.pi * np.arange(nu) / nu
    w = 2.0 * np.pi * np.arange(nv) / nv
    uu, ww = np.meshgrid(u, w, indexing="ij")
    rad = major + minor * np.cos(ww)
    verts = np.stack([cx + rad * np.cos(uu), cy + minor * np.sin(ww), cz + rad * np.sin(uu)], -1)
    verts = verts.reshape(-1, 3).astype(np.float32)
    tris = []
    for a in range(nu):
        for b in range(nv):
            p, q = a * nv + b, ((a + 1) % nu) * nv + b
            p1, q1 = a * nv + (b + 1) % nv, ((a + 1) % nu) * nv + (b + 1) % nv
            tris += [(p, q, q1), (p, q1, p1)]
    return verts, np.array(tris, np.int32)


def merge_meshes(*meshes):
    """One mesh holding the given (vertices, triangles) pairs, indices offset."""
    vs, ts, off = [], [], 0
    for v, t in meshes:
        vs.append(np.asarray(v, np.float32))
        ts.append(np.asarray(t, np.int32) + off)
        off += len(v)
    return np.concatenate(vs), np.concatenate(ts)


def scattered_boxes(count, lo, hi, size, seed=0):
    """`count` separate small boxes (islands) with seeded corners in [lo, hi - size]."""
    rng = np.random.Generator(np.random.PCG64(seed))
    lo = np.asarray(lo, np.float64)
    span = np.asarray(hi, np.float64) - lo - size
    boxes = []
    for _ in range(count):
        a = lo + rng.random(3) * span
        boxes.append(box_mesh(tuple(a), tuple(a + size * (0.5 + rng.random(3)))))
    return merge_meshes(*boxes)
