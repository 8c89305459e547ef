"""ctypes access to the stage-level C-ABI functions of libffengine_gb300.so (tests only).

Same array conventions as oracle_api: numpy shape (d, h, w), x fastest.
"""
import ctypes
from ctypes import byref, c_double, c_float, c_int, c_void_p

import numpy as np

from ffengine_gb300 import load_library

F32 = np.float32
U8 = np.uint8


def _p(a):
    return a.ctypes.data_as(c_void_p) if a is not None else None


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


def _call(name, *args, restype=None):
    f = getattr(load_library(), name)
    f.restype = restype
    err = c_int(1)
    r = f(*args, byref(err))
    if not err.value:
        m = load_library().CBindings_get_error_message
        m.restype = ctypes.c_char_p
        raise RuntimeError(name + ": " + m().decode())
    return r


def solid_phi(n, dx, spheres=()):
    sp = np.array(spheres, np.float64).reshape(-1, 4)
    out = np.empty((n + 1, n + 1, n + 1), F32)
    _call("ffgpu_solid_phi", n, n, n, c_double(dx), len(sp), _p(_c(sp, np.float64)), _p(out))
    return out


def face_weights(n, solid):
    wu = np.empty((n, n, n + 1), F32); wv = np.empty((n, n + 1, n), F32); ww = np.empty((n + 1, n, n), F32)
    _call("ffgpu_face_weights", n, n, n, _p(_c(solid, F32)), _p(wu), _p(wv), _p(ww))
    return wu, wv, ww


def sort_particles(n, dx, pos):
    pos = _c(pos, F32)
    cs = np.empty(n * n * n + 1, np.int32)
    si = np.empty(max(pos.shape[0], 1), np.int32)
    _call("ffgpu_sort_particles", n, n, n, c_double(dx), pos.shape[0], _p(pos), _p(cs), _p(si))
    return cs, si[:pos.shape[0]]


def liquid_sdf(n, dx, pos, solid=None, post=False):
    pos = _c(pos, F32)
    out = np.empty((n, n, n), F32)
    _call("ffgpu_liquid_sdf", n, n, n, c_double(dx), pos.shape[0], _p(pos),
          _p(_c(solid, F32)) if solid is not None else None, 1 if post else 0, _p(out))
    return out


def p2g(n, dx, pos, vel, per_component=False):
    pos = _c(pos, F32); vel = _c(vel, F32)
    u = np.empty((n, n, n + 1), F32); v = np.empty((n, n + 1, n), F32); w = np.empty((n + 1, n, n), F32)
    vu = np.empty(u.shape, U8); vv = np.empty(v.shape, U8); vw = np.empty(w.shape, U8)
    _call("ffgpu_p2g_components" if per_component else "ffgpu_p2g", n, n, n, c_double(dx), pos.shape[0], _p(pos),
          _p(vel), _p(u), _p(v), _p(w), _p(vu), _p(vv), _p(vw))
    return [(u, vu), (v, vv), (w, vw)]


def extrapolate(grid, valid, layers):
    g = _c(grid, F32).copy()
    d, h, w = g.shape
    _call("ffgpu_extrapolate", w, h, d, _p(g), _p(_c(valid, U8)), layers)
    return g


def pressure_solve(n, dx, dt, phi, weights, uvw, tol=1e-9, maxit=900, mode=0):
    pr = np.empty((n, n, n), F32)
    p64 = np.empty((n, n, n), np.float64)
    stats = np.zeros(4, np.int32)
    errs = np.zeros(3, np.float64)
    args = [_c(phi, F32)] + [_c(a, F32) for a in weights] + [_c(a, F32) for a in uvw]
    _call("ffgpu_pressure_solve", n, n, n, c_double(dx), c_double(dt), *[_p(a) for a in args], c_double(tol),
          maxit, mode, _p(pr), _p(p64), _p(stats), _p(errs))
    return pr, p64, dict(iters=int(stats[0]), success=bool(stats[1]), outer=int(stats[2]), box=int(stats[3]),
                         error=float(errs[0]), rel_residual=float(errs[1]), bnorm=float(errs[2]))


def apply_pressure(n, dx, dt, phi, weights, pressure, uvw):
    u, v, w = [_c(a, F32).copy() for a in uvw]
    vu = np.empty(u.shape, U8); vv = np.empty(v.shape, U8); vw = np.empty(w.shape, U8)
    args = [_c(phi, F32)] + [_c(a, F32) for a in weights] + [_c(pressure, F32)]
    _call("ffgpu_apply_pressure", n, n, n, c_double(dx), c_double(dt), *[_p(a) for a in args], _p(u), _p(v), _p(w),
          _p(vu), _p(vv), _p(vw))
    return (u, v, w), (vu, vv, vw)


def g2p(n, dx, pic, pos, vel, uvw, saved):
    pos = _c(pos, F32)
    vel = _c(vel, F32).copy()
    _call("ffgpu_g2p", n, n, n, c_double(dx), c_double(pic), pos.shape[0], _p(pos), _p(vel),
          *[_p(_c(a, F32)) for a in uvw], *[_p(_c(a, F32)) for a in saved])
    return vel


def advect(n, dx, dt, cfl, pos, uvw, solid):
    pos = _c(pos, F32)
    out = np.empty_like(pos)
    _call("ffgpu_advect", n, n, n, c_double(dx), c_double(dt), cfl, pos.shape[0], _p(pos),
          *[_p(_c(a, F32)) for a in uvw], _p(_c(solid, F32)) if solid is not None else None, _p(out))
    return out


def remove(n, dx, pos, vel, solid, max_per_cell=250):
    pos = _c(pos, F32).copy(); vel = _c(vel, F32).copy()
    cnt = _call("ffgpu_remove", n, n, n, c_double(dx), pos.shape[0], _p(pos), _p(vel),
                _p(_c(solid, F32)) if solid is not None else None, max_per_cell, restype=c_int)
    return pos[:cnt].copy(), vel[:cnt].copy()


def remove_extreme(n, dx, pos, vel, solid, frame_dt, cfl, max_substeps, max_per_cell=250):
    pos = _c(pos, F32).copy(); vel = _c(vel, F32).copy()
    lim = c_float(0)
    cnt = _call("ffgpu_remove_extreme", n, n, n, c_double(dx), pos.shape[0], _p(pos), _p(vel),
                _p(_c(solid, F32)) if solid is not None else None, max_per_cell, c_double(frame_dt), cfl,
                max_substeps, byref(lim), restype=c_int)
    return pos[:cnt].copy(), vel[:cnt].copy(), lim.value


def classify(phi):
    d, h, w = phi.shape
    fluid = np.empty(phi.shape, U8)
    bbox = np.zeros(6, np.int32)
    _call("ffgpu_classify", w, h, d, _p(_c(phi, F32)), _p(fluid), _p(bbox))
    return fluid, bbox


def substep(n, dx, dt, pic, cfl, g, solid, pos, vel, tol=1e-9, maxit=900, mode=0):
    pos = _c(pos, F32).copy(); vel = _c(vel, F32).copy()
    stats = np.zeros(4, np.int32)
    errs = np.zeros(3, np.float64)
    cnt = _call("ffgpu_substep", n, n, n, c_double(dx), c_double(dt), c_double(pic), cfl, c_float(g[0]),
                c_float(g[1]), c_float(g[2]), _p(_c(solid, F32)) if solid is not None else None, c_double(tol),
                maxit, mode, pos.shape[0], _p(pos), _p(vel), _p(stats), _p(errs), restype=c_int)
    return pos[:cnt].copy(), vel[:cnt].copy(), dict(iters=int(stats[0]), success=bool(stats[1]),
                                                     outer=int(stats[2]), error=float(errs[0]),
                                                     rel_residual=float(errs[1]))


def p2g_apic(n, dx, pos, vel, aff9):
    pos = _c(pos, F32); vel = _c(vel, F32); aff9 = _c(aff9, F32)
    u = np.empty((n, n, n + 1), F32); v = np.empty((n, n + 1, n), F32); w = np.empty((n + 1, n, n), F32)
    vu = np.empty(u.shape, U8); vv = np.empty(v.shape, U8); vw = np.empty(w.shape, U8)
    _call("ffgpu_p2g_apic", n, n, n, c_double(dx), pos.shape[0], _p(pos), _p(vel), _p(aff9), _p(u), _p(v), _p(w),
          _p(vu), _p(vv), _p(vw))
    return [(u, vu), (v, vv), (w, vw)]


def g2p_apic(n, dx, pos, uvw):
    pos = _c(pos, F32)
    vel = np.zeros_like(pos)
    aff9 = np.zeros((pos.shape[0], 9), F32)
    _call("ffgpu_g2p_apic", n, n, n, c_double(dx), pos.shape[0], _p(pos), _p(vel), _p(aff9),
          *[_p(_c(a, F32)) for a in uvw])
    return vel, aff9


def substep_apic(n, dx, dt, cfl, g, solid, pos, vel, aff9, tol=1e-9, maxit=900, mode=0):
    pos = _c(pos, F32).copy(); vel = _c(vel, F32).copy(); aff9 = _c(aff9, F32).reshape(-1, 9).copy()
    stats = np.zeros(4, np.int32)
    errs = np.zeros(3, np.float64)
    cnt = _call("ffgpu_substep_apic", n, n, n, c_double(dx), c_double(dt), cfl, c_float(g[0]), c_float(g[1]),
                c_float(g[2]), _p(_c(solid, F32)) if solid is not None else None, c_double(tol), maxit, mode,
                pos.shape[0], _p(pos), _p(vel), _p(aff9), _p(stats), _p(errs), restype=c_int)
    return (pos[:cnt].copy(), vel[:cnt].copy(), aff9[:cnt].copy(),
            dict(iters=int(stats[0]), success=bool(stats[1]), error=float(errs[0])))


def viscosity_precondition(shape, dx, dt, liquid_phi, solid, visc, uvw, form, sweeps):
    """One viscosity preconditioner application to the system's rhs (form 0 wavefront, 1 levels,
    2 cooperative; sweeps 1 forward, 2 both).  Returns the rows' values."""
    ni, nj, nk = shape
    u, v, w = [_c(a, F32) for a in uvw]
    z = np.zeros(u.size + v.size + w.size, F32)
    n = _call("ffgpu_viscosity_precondition", ni, nj, nk, c_double(dx), c_double(dt), _p(_c(liquid_phi, F32)),
              _p(_c(solid, F32)), c_double(visc), _p(u), _p(v), _p(w), int(form), int(sweeps), _p(z),
              restype=ctypes.c_int)
    return z[:n].copy()


def viscosity(n, dx, dt, liquid_phi, solid, visc, uvw, tol=1e-4, maxit=900, debug=False):
    """GPU viscosity solve; same outputs as oracle_api.viscosity (constant viscosity)."""
    u, v, w = [_c(a, F32).copy() for a in uvw]
    nf = u.size + v.size + w.size
    stats = np.zeros(3, np.int32)
    res = ctypes.c_float(0)
    dbg = {}
    if debug:
        n1 = n + 1
        dbg = {"vol": np.zeros(n ** 3 + 3 * n * n * n1 + 3 * n * n1 * n1, F32), "index": np.zeros(nf, np.int32),
               "rowstart": np.zeros(nf + 1, np.uint32), "col": np.zeros(15 * nf, np.uint32),
               "val": np.zeros(15 * nf, F32), "rhs": np.zeros(nf, F32), "ic_invdiag": np.zeros(nf, F32),
               "ic_colstart": np.zeros(nf + 1, np.uint32), "ic_rowindex": np.zeros(15 * nf, np.uint32),
               "ic_value": np.zeros(15 * nf, F32), "soln": np.zeros(nf, F32)}
    g = lambda k: _p(dbg[k]) if debug else None
    _call("ffgpu_viscosity", n, n, n, c_double(dx), c_double(dt), _p(_c(liquid_phi, F32)), _p(_c(solid, F32)),
          c_double(visc), c_double(tol), maxit, _p(u), _p(v), _p(w), _p(stats), byref(res), g("vol"), g("index"),
          g("rowstart"), g("col"), g("val"), g("rhs"), g("ic_invdiag"), g("ic_colstart"), g("ic_rowindex"),
          g("ic_value"), g("soln"))
    st = dict(n=int(stats[0]), iters=int(stats[1]), success=bool(stats[2]), error=res.value)
    if debug:
        m = st["n"]
        nnz = int(dbg["rowstart"][m]) if m else 0
        dbg["rowstart"] = dbg["rowstart"][:m + 1]
        dbg["col"], dbg["val"] = dbg["col"][:nnz], dbg["val"][:nnz]
        for k in ("rhs", "ic_invdiag", "soln"):
            dbg[k] = dbg[k][:m]
        dbg["ic_colstart"] = dbg["ic_colstart"][:m + 1]
        lnz = int(dbg["ic_colstart"][m]) if m else 0
        dbg["ic_rowindex"], dbg["ic_value"] = dbg["ic_rowindex"][:lnz], dbg["ic_value"][:lnz]
        n1 = n + 1
        sizes = [n ** 3, n * n * n1, n * n * n1, n * n * n1, n * n1 * n1, n * n1 * n1, n * n1 * n1]
        parts = np.split(dbg["vol"], np.cumsum(sizes)[:-1])
        shapes = [(n, n, n), (n, n, n1), (n, n1, n), (n1, n, n), (n1, n1, n), (n1, n, n1), (n, n1, n1)]
        dbg["vol"] = dict(zip(["center", "u", "v", "w", "eu", "ev", "ew"], [p.reshape(s) for p, s in zip(parts, shapes)]))
    return (u, v, w), st, dbg


def curvature_grid(n, dx, phi):
    """GPU surface curvature grid: (surface_phi, curvature), as oracle_api.curvature_grid."""
    surf = np.empty((n, n, n), F32)
    k = np.empty((n, n, n), F32)
    _call("ffgpu_curvature_grid", n, n, n, c_double(dx), _p(_c(phi, F32)), _p(surf), _p(k))
    return surf, k


def cluster_status(phi):
    d, h, w = phi.shape
    st = np.empty(phi.shape, U8)
    _call("ffgpu_cluster_status", w, h, d, _p(_c(phi, F32)), _p(st))
    return st


def pressure_solve_tension(n, dx, dt, phi, weights, uvw, curvature, k_st, tol=1e-9, maxit=900, mode=0):
    pr = np.empty((n, n, n), F32)
    p64 = np.empty((n, n, n), np.float64)
    stats = np.zeros(4, np.int32)
    errs = np.zeros(3, np.float64)
    args = [_c(phi, F32)] + [_c(a, F32) for a in weights] + [_c(a, F32) for a in uvw]
    _call("ffgpu_pressure_solve_tension", n, n, n, c_double(dx), c_double(dt), *[_p(a) for a in args],
          _p(_c(curvature, F32)), c_double(k_st), c_double(tol), maxit, mode, _p(pr), _p(p64), _p(stats), _p(errs))
    return pr, p64, dict(iters=int(stats[0]), success=bool(stats[1]), outer=int(stats[2]), box=int(stats[3]),
                         error=float(errs[0]), rel_residual=float(errs[1]), bnorm=float(errs[2]))


def apply_pressure_tension(n, dx, dt, phi, weights, pressure, uvw, curvature, k_st):
    u, v, w = [_c(a, F32).copy() for a in uvw]
    vu = np.empty(u.shape, U8); vv = np.empty(v.shape, U8); vw = np.empty(w.shape, U8)
    args = [_c(phi, F32)] + [_c(a, F32) for a in weights] + [_c(pressure, F32), _c(curvature, F32)]
    _call("ffgpu_apply_pressure_tension", n, n, n, c_double(dx), c_double(dt), *[_p(a) for a in args],
          c_double(k_st), _p(u), _p(v), _p(w), _p(vu), _p(vv), _p(vw))
    return (u, v, w), (vu, vv, vw)


def solid_level_set(n, dx, objects=(), jitter=None):
    """GPU solid level set of the closed domain and static meshes; arguments as
    oracle_api.solid_level_set."""
    nv = np.array([len(o[0]) for o in objects] or [0], np.int32)
    nt = np.array([len(o[1]) for o in objects] or [0], np.int32)
    verts = _c(np.concatenate([np.asarray(o[0], F32).reshape(-1, 3) for o in objects])
               if objects else np.zeros((1, 3)), F32)
    tris = _c(np.concatenate([np.asarray(o[1], np.int32).reshape(-1, 3) for o in objects])
              if objects else np.zeros((1, 3)), np.int32)
    flags = np.array([o[2] for o in objects] or [0], np.int32)
    exp = np.array([o[3] for o in objects] or [0.0], F32)
    jit = None if jitter is None else _c(np.asarray(jitter, F32).reshape(-1, 3), F32)
    phi = np.empty((n + 1, n + 1, n + 1), F32)
    _call("ffgpu_solid_level_set", n, n, n, c_double(dx), len(objects), _p(nv), _p(nt), _p(verts), _p(tris),
          _p(flags), _p(exp), 0 if jit is None else jit.shape[0], _p(jit), _p(phi))
    return phi


def ffp3(n, dx, solid, pos, vel, ids, flags, amount):
    """GPU FFP3 output of the given particles: (types, {"pos", "id", "vel", "speed"} -> bytes), as
    oracle_api.ffp3 with the surface level set computed on the GPU."""
    pos, vel = _c(pos, F32), _c(vel, F32)
    ids = _c(ids, np.uint16)
    np_ = pos.shape[0]
    cap = 16 + 12 * 65536 + 12 * np_
    outs = [np.zeros(cap, np.uint8) for _ in range(4)]
    sizes = np.zeros(4, np.int64)
    types = np.zeros(max(np_, 1), np.uint8)
    _call("ffgpu_ffp3", n, n, n, c_double(dx), _p(_c(solid, F32)) if solid is not None else None, np_, _p(pos),
          _p(vel), _p(ids), int(flags), c_double(amount), *[_p(o) for o in outs], _p(sizes), _p(types))
    return types[:np_], {k: o[:int(s)].copy() for k, o, s in zip(("pos", "id", "vel", "speed"), outs, sizes)}
