"""Parity on non-cubic grids: the FLIP and APIC transfers, the APIC particle update and the
viscosity solve on (ni, nj, nk) = (23, 17, 31) and (10, 29, 12), against the CPU oracle (which is
pinned bit-exact to the reference on the golden vectors).  Non-cubic sizes put the 10-cell
transfer blocks, the face-grid index decodes and the viscosity levels (i + j + k + 2 comp) on
uneven extents in every direction.

Bars as on the cubic cases: P2G within 1e-6 of max|ref| with equal valid flags; APIC affine
vectors bit-exact; viscosity volumes, system and MIC(0) factor bit-exact, the GPU solution meeting
the reference's stopping rule on the oracle's system.
"""
from ctypes import byref, c_double, c_float

import numpy as np
import pytest

import gpu_api as G
import oracle_api as O

pytestmark = pytest.mark.gpu

F32, U8 = np.float32, np.uint8
SIZES = [(23, 17, 31), (10, 29, 12)]


def bits_equal(a, b):
    a = np.ascontiguousarray(a); b = np.ascontiguousarray(b)
    return a.shape == b.shape and np.array_equal(a.view(np.uint32), b.view(np.uint32))


def fshape(ni, nj, nk, c):
    return [(nk, nj, ni + 1), (nk, nj + 1, ni), (nk + 1, nj, ni)][c]


def scene(ni, nj, nk, seed=5):
    dx = 1.0 / max(ni, nj, nk)
    rng = np.random.default_rng(seed)
    hi = np.array([0.6 * ni, 0.7 * nj, nk - 1.5]) * dx
    lo = np.full(3, 1.5 * dx)
    n = int(8 * np.prod((hi - lo) / dx))
    pos = (lo + rng.random((n, 3)) * (hi - lo)).astype(F32)
    vel = rng.standard_normal((n, 3)).astype(F32)
    aff = (2.0 * rng.standard_normal((n, 9))).astype(F32)
    return dx, pos, vel, aff


def oracle_p2g(ni, nj, nk, dx, pos, vel, aff=None):
    out = []
    for c in range(3):
        f = np.empty(fshape(ni, nj, nk, c), F32); v = np.empty(f.shape, U8)
        if aff is None:
            O.lib().oracle_p2g_component(ni, nj, nk, c_double(dx), c_double(O.radius(dx)), pos.shape[0], O._p(pos),
                                         O._p(vel), c, O._p(f), O._p(v))
        else:
            O.lib().oracle_p2g_apic_component(ni, nj, nk, c_double(dx), c_double(O.radius(dx)), pos.shape[0],
                                              O._p(pos), O._p(vel), O._p(aff), c, O._p(f), O._p(v))
        out.append((f, v))
    return out


def gpu_p2g(ni, nj, nk, dx, pos, vel, aff=None):
    fs = [np.empty(fshape(ni, nj, nk, c), F32) for c in range(3)]
    vs = [np.empty(f.shape, U8) for f in fs]
    if aff is None:
        G._call("ffgpu_p2g", ni, nj, nk, c_double(dx), pos.shape[0], G._p(pos), G._p(vel), *map(G._p, fs),
                *map(G._p, vs))
    else:
        G._call("ffgpu_p2g_apic", ni, nj, nk, c_double(dx), pos.shape[0], G._p(pos), G._p(vel), G._p(aff),
                *map(G._p, fs), *map(G._p, vs))
    return list(zip(fs, vs))


@pytest.mark.parametrize("dims", SIZES)
@pytest.mark.parametrize("apic", [False, True])
def test_p2g_ragged(dims, apic):
    ni, nj, nk = dims
    dx, pos, vel, aff = scene(*dims)
    g = gpu_p2g(ni, nj, nk, dx, pos, vel, aff if apic else None)
    o = oracle_p2g(ni, nj, nk, dx, pos, vel, aff if apic else None)
    for (f, v), (of, ov) in zip(g, o):
        assert np.array_equal(v, ov)
        assert np.abs(f - of).max() <= 1e-6 * max(np.abs(of).max(), 1e-30) + 1e-12


@pytest.mark.parametrize("dims", SIZES)
def test_g2p_apic_ragged(dims):
    ni, nj, nk = dims
    dx, pos, _, _ = scene(*dims)
    rng = np.random.default_rng(9)
    uvw = [rng.standard_normal(fshape(ni, nj, nk, c)).astype(F32) for c in range(3)]
    gv = np.zeros_like(pos); ga = np.zeros((pos.shape[0], 9), F32)
    G._call("ffgpu_g2p_apic", ni, nj, nk, c_double(dx), pos.shape[0], G._p(pos), G._p(gv), G._p(ga), *map(G._p, uvw))
    ov = np.empty_like(pos); oa = np.empty((pos.shape[0], 9), F32)
    O.lib().oracle_g2p_apic(ni, nj, nk, c_double(dx), pos.shape[0], O._p(pos), O._p(ov), O._p(oa), *map(O._p, uvw))
    assert bits_equal(ga, oa)
    assert np.abs(gv - ov).max() <= 2e-5 * max(np.abs(ov).max(), 1.0)


def _visc_inputs(ni, nj, nk):
    dx, pos, _, _ = scene(ni, nj, nk)
    solid = np.empty((nk + 1, nj + 1, ni + 1), F32)
    O.lib().oracle_solid_phi(ni, nj, nk, c_double(dx), 0, None, O._p(solid))
    phi = np.empty((nk, nj, ni), F32)
    O.lib().oracle_liquid_sdf(ni, nj, nk, c_double(dx), c_double(O.radius(dx)), pos.shape[0], O._p(pos), O._p(phi))
    O.lib().oracle_postprocess_sdf(ni, nj, nk, c_double(dx), O._p(solid), O._p(phi))
    rng = np.random.default_rng(3)
    uvw = [rng.standard_normal(fshape(ni, nj, nk, c)).astype(F32) for c in range(3)]
    w = [np.empty(fshape(ni, nj, nk, c), F32) for c in range(3)]
    O.lib().oracle_face_weights(ni, nj, nk, O._p(solid), *map(O._p, w))
    O.lib().oracle_constrain(ni, nj, nk, *map(O._p, w), *map(O._p, uvw))
    return dx, phi, solid, uvw


def _visc_run(ni, nj, nk, dx, phi, solid, uvw, visc, debug_sizes, is_gpu):
    u, v, w = [a.copy() for a in uvw]
    nf = u.size + v.size + w.size
    vol = np.zeros(debug_sizes, F32)
    index = np.zeros(nf, np.int32)
    rowstart = np.zeros(nf + 1, np.uint32); col = np.zeros(15 * nf, np.uint32); val = np.zeros(15 * nf, F32)
    rhs = np.zeros(nf, F32); inv = np.zeros(nf, F32); cs = np.zeros(nf + 1, np.uint32)
    ri = np.zeros(15 * nf, np.uint32); lv = np.zeros(15 * nf, F32); soln = np.zeros(nf, F32)
    stats = np.zeros(3, np.int32)
    p = G._p if is_gpu else O._p
    if is_gpu:
        res = c_float(0)
        G._call("ffgpu_viscosity", ni, nj, nk, c_double(dx), c_double(1 / 240), p(phi), p(solid), c_double(visc),
                c_double(1e-4), 900, p(u), p(v), p(w), p(stats), byref(res), p(vol), p(index), p(rowstart), p(col),
                p(val), p(rhs), p(inv), p(cs), p(ri), p(lv), p(soln))
    else:
        res = c_float(0)
        vg = np.full((nk + 1, nj + 1, ni + 1), visc, F32)
        O.lib().oracle_viscosity(ni, nj, nk, c_double(dx), c_double(1 / 240), p(phi), p(solid), p(vg), c_double(1e-4),
                                 900, p(u), p(v), p(w), p(stats), byref(res), p(vol), p(index), p(rowstart), p(col),
                                 p(val), p(rhs), p(inv), p(cs), p(ri), p(lv), p(soln))
    m = int(stats[0])
    nnz, lnz = int(rowstart[m]), int(cs[m])
    return dict(n=m, iters=int(stats[1]), vol=vol, index=index, rowstart=rowstart[:m + 1], col=col[:nnz],
                val=val[:nnz], rhs=rhs[:m], inv=inv[:m], cs=cs[:m + 1], ri=ri[:lnz], lv=lv[:lnz], soln=soln[:m],
                uvw=(u, v, w))


@pytest.mark.parametrize("dims", SIZES)
def test_viscosity_ragged(dims):
    ni, nj, nk = dims
    dx, phi, solid, uvw = _visc_inputs(ni, nj, nk)
    vsize = (ni * nj * nk + (ni + 1) * nj * nk + ni * (nj + 1) * nk + ni * nj * (nk + 1) + ni * (nj + 1) * (nk + 1) +
             (ni + 1) * nj * (nk + 1) + (ni + 1) * (nj + 1) * nk)
    g = _visc_run(ni, nj, nk, dx, phi, solid, uvw, 2.0, vsize, True)
    o = _visc_run(ni, nj, nk, dx, phi, solid, uvw, 2.0, vsize, False)
    assert g["n"] == o["n"] > 0
    assert bits_equal(g["vol"], o["vol"]) and np.array_equal(g["index"], o["index"])
    for k in ("rowstart", "col", "cs", "ri"):
        assert np.array_equal(g[k], o[k]), k
    for k in ("val", "rhs", "inv", "lv"):
        assert bits_equal(g[k], o[k]), k
    rs, col, val, rhs = o["rowstart"], o["col"], o["val"], o["rhs"]
    rows = np.repeat(np.arange(rs.size - 1), np.diff(rs.astype(np.int64)))
    ax = np.bincount(rows, weights=val.astype(np.float64) * g["soln"].astype(np.float64)[col], minlength=rs.size - 1)
    assert np.abs(rhs.astype(np.float64) - ax).max() <= 1.001e-4 * np.abs(rhs).max()
    assert abs(g["iters"] - o["iters"]) <= 3
