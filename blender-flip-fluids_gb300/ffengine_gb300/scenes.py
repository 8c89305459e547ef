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
