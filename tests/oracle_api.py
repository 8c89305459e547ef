"""ctypes access to the CPU oracle (oracle/liboracle.so) -- test infrastructure only.

Arrays use the reference engine's grid layout: x fastest, numpy shape (d, h, w).
"""
import ctypes
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(ROOT, "oracle")
_lib = None

F32 = np.float32
U8 = np.uint8


def build():
    subprocess.run(["make", "-s", "-C", ORACLE_DIR], check=True)


def lib():
    global _lib
    if _lib is None:
        path = os.path.join(ORACLE_DIR, "liboracle.so")
        srcs = [os.path.join(ORACLE_DIR, f) for f in os.listdir(ORACLE_DIR) if f.endswith((".cpp", ".h"))]
        if not os.path.exists(path) or any(os.path.getmtime(s) > os.path.getmtime(path) for s in srcs):
            build()
        _lib = ctypes.CDLL(path)
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


def solid_phi(n, dx, spheres=()):
    sp = np.array(spheres, np.float64).reshape(-1, 4) if spheres else np.zeros((0, 4))
    out = np.empty((n + 1, n + 1, n + 1), F32)
    lib().oracle_solid_phi(n, n, n, ctypes.c_double(dx), len(sp), _p(_c(sp, np.float64)), _p(out))
    return out


def face_weights(n, solid):
    wu = np.empty((n, n, n + 1), F32); wv = np.empty((n, n + 1, n), F32); ww = np.empty((n + 1, n, n), F32)
    lib().oracle_face_weights(n, n, n, _p(_c(solid, F32)), _p(wu), _p(wv), _p(ww))
    return wu, wv, ww


def radius(dx):
    return 0.5 * dx * np.sqrt(3.0)


def liquid_sdf(n, dx, pos):
    pos = _c(pos, F32)
    out = np.empty((n, n, n), F32)
    lib().oracle_liquid_sdf(n, n, n, ctypes.c_double(dx), ctypes.c_double(radius(dx)), pos.shape[0], _p(pos), _p(out))
    return out


def postprocess_sdf(n, dx, solid, phi):
    phi = _c(phi, F32).copy()
    lib().oracle_postprocess_sdf(n, n, n, ctypes.c_double(dx), _p(_c(solid, F32)), _p(phi))
    return phi


_FSHAPE = {0: lambda n: (n, n, n + 1), 1: lambda n: (n, n + 1, n), 2: lambda n: (n + 1, n, n)}


def p2g(n, dx, pos, vel):
    pos = _c(pos, F32); vel = _c(vel, F32)
    out = []
    for d in range(3):
        f = np.empty(_FSHAPE[d](n), F32); v = np.empty(_FSHAPE[d](n), U8)
        lib().oracle_p2g_component(n, n, n, ctypes.c_double(dx), ctypes.c_double(radius(dx)), pos.shape[0],
                                   _p(pos), _p(vel), d, _p(f), _p(v))
        out.append((f, v))
    return out


def extrapolate(grid, valid, layers):
    g = _c(grid, F32).copy()
    d, h, w = g.shape
    lib().oracle_extrapolate(w, h, d, _p(g), _p(_c(valid, U8)), layers)
    return g


def layers(cfl):
    return int(np.ceil(np.sqrt(3) * cfl)) + 3


def body_force(n, dt, g, u, v, w):
    u = _c(u, F32).copy(); v = _c(v, F32).copy(); w = _c(w, F32).copy()
    lib().oracle_body_force(n, n, n, ctypes.c_double(dt), ctypes.c_float(g[0]), ctypes.c_float(g[1]),
                            ctypes.c_float(g[2]), _p(u), _p(v), _p(w))
    return u, v, w


def pressure_solve(n, dx, dt, phi, weights, uvw, tol=1e-9, maxit=900, float_scalars=True):
    pr = np.empty((n, n, n), F32)
    stats = np.zeros(2, np.int32)
    err = ctypes.c_double(0)
    args = [_c(phi, F32)] + [_c(a, F32) for a in weights] + [_c(a, F32) for a in uvw]
    nf = lib().oracle_pressure_solve(n, n, n, ctypes.c_double(dx), ctypes.c_double(dt), *[_p(a) for a in args],
                                     ctypes.c_double(tol), maxit, 1 if float_scalars else 0, _p(pr), _p(stats),
                                     ctypes.byref(err))
    return pr, int(stats[0]), bool(stats[1]), err.value, nf


def pressure_residual(n, dx, dt, phi, weights, uvw, p64):
    args = [_c(phi, F32)] + [_c(a, F32) for a in weights] + [_c(a, F32) for a in uvw]
    rel = ctypes.c_double(0)
    f = lib().oracle_pressure_residual
    f.restype = ctypes.c_double
    inf = f(n, n, n, ctypes.c_double(dx), ctypes.c_double(dt), *[_p(a) for a in args],
            _p(_c(p64, np.float64)), ctypes.byref(rel))
    return inf, rel.value


def pressure_system(n, dx, dt, phi, weights, uvw, maxn=20000, dense=True):
    args = [_c(phi, F32)] + [_c(a, F32) for a in weights] + [_c(a, F32) for a in uvw]
    cells = np.zeros((maxn, 3), np.int32)
    rhs = np.zeros(maxn, np.float64)
    cnt = lib().oracle_pressure_system(n, n, n, ctypes.c_double(dx), ctypes.c_double(dt), *[_p(a) for a in args],
                                       0, None, None, None)
    A = np.zeros((cnt, cnt), np.float64) if dense else None
    cells = np.zeros((cnt, 3), np.int32); rhs = np.zeros(cnt, np.float64)
    lib().oracle_pressure_system(n, n, n, ctypes.c_double(dx), ctypes.c_double(dt), *[_p(a) for a in args],
                                 cnt, _p(cells), _p(rhs), _p(A))
    return cells, rhs, A


def apply_pressure(n, dx, dt, phi, weights, pressure, uvw):
    u, v, w = [_c(a, F32).copy() for a in uvw]
    vu = np.empty(u.shape, U8); vv = np.empty(v.shape, U8); vw = np.empty(w.shape, U8)
    args = [_c(phi, F32)] + [_c(a, F32) for a in weights] + [_c(pressure, F32)]
    lib().oracle_apply_pressure(n, n, n, ctypes.c_double(dx), ctypes.c_double(dt), *[_p(a) for a in args],
                                _p(u), _p(v), _p(w), _p(vu), _p(vv), _p(vw))
    return (u, v, w), (vu, vv, vw)


def constrain(n, weights, uvw):
    u, v, w = [_c(a, F32).copy() for a in uvw]
    lib().oracle_constrain(n, n, n, *[_p(_c(a, F32)) for a in weights], _p(u), _p(v), _p(w))
    return u, v, w


def g2p(n, dx, pic, pos, vel, uvw, saved):
    vel = _c(vel, F32).copy()
    pos = _c(pos, F32)
    lib().oracle_g2p(n, n, n, ctypes.c_double(dx), ctypes.c_double(pic), pos.shape[0], _p(pos), _p(vel),
                     *[_p(_c(a, F32)) for a in uvw], *[_p(_c(a, F32)) for a in saved])
    return vel


def sample_mac(n, dx, pos, uvw):
    pos = _c(pos, F32)
    out = np.empty_like(pos)
    lib().oracle_sample_mac(n, n, n, ctypes.c_double(dx), pos.shape[0], _p(pos), *[_p(_c(a, F32)) for a in uvw], _p(out))
    return out


def advect(n, dx, dt, cfl, pos, uvw, solid):
    pos = _c(pos, F32)
    out = np.empty_like(pos)
    lib().oracle_advect(n, n, n, ctypes.c_double(dx), ctypes.c_double(dt), cfl, pos.shape[0], _p(pos),
                        *[_p(_c(a, F32)) for a in uvw], _p(_c(solid, F32)), _p(out))
    return out


def remove(n, dx, pos, vel, solid, max_per_cell=250):
    pos = _c(pos, F32).copy(); vel = _c(vel, F32).copy()
    cnt = lib().oracle_remove(n, n, n, ctypes.c_double(dx), pos.shape[0], _p(pos), _p(vel), _p(_c(solid, F32)),
                              max_per_cell)
    return pos[:cnt].copy(), vel[:cnt].copy()


def speed_limit(vel, cfl, dx, frame_dt, max_steps):
    """The extreme-velocity removal limit (float) for these particle velocities."""
    f = lib().oracle_speed_limit
    f.restype = ctypes.c_float
    vel = _c(vel, F32)
    return float(f(vel.shape[0], _p(vel), ctypes.c_double(cfl), ctypes.c_double(dx), ctypes.c_double(frame_dt),
                   max_steps))


def remove_extreme(n, dx, pos, vel, solid, limit, max_per_cell=250):
    """Marker removal with the extreme-velocity rule on, at the given speed limit."""
    pos = _c(pos, F32).copy(); vel = _c(vel, F32).copy()
    cnt = lib().oracle_remove_extreme(n, n, n, ctypes.c_double(dx), pos.shape[0], _p(pos), _p(vel),
                                      _p(_c(solid, F32)), max_per_cell, ctypes.c_float(limit))
    return pos[:cnt].copy(), vel[:cnt].copy()


def substep(n, dx, dt, pic, cfl, g, solid, pos, vel, tol=1e-9, maxit=900, evr=None):
    """One PIC/FLIP substep.  evr = (frame_dt, max_steps) turns extreme-velocity removal on with
    the speed limit of an update of length frame_dt allowing max_steps substeps."""
    pos = _c(pos, F32).copy(); vel = _c(vel, F32).copy()
    stats = np.zeros(3, np.int32)
    err = ctypes.c_double(0)
    head = (n, n, n, ctypes.c_double(dx), ctypes.c_double(dt), ctypes.c_double(pic), cfl,
            ctypes.c_float(g[0]), ctypes.c_float(g[1]), ctypes.c_float(g[2]), _p(_c(solid, F32)),
            ctypes.c_double(tol), maxit, pos.shape[0], _p(pos), _p(vel))
    if evr is None:
        cnt = lib().oracle_substep(*head, _p(stats), ctypes.byref(err))
    else:
        cnt = lib().oracle_substep_evr(*head, ctypes.c_double(evr[0]), int(evr[1]), _p(stats), ctypes.byref(err))
    return pos[:cnt].copy(), vel[:cnt].copy(), dict(iters=int(stats[0]), success=bool(stats[1]),
                                                     fluid_cells=int(stats[2]), error=err.value)


def as_loaded(a, record_bytes=24):
    """A batch in the order the reference's load queue hands it over: a FragmentedVector of
    5e6-byte fragments whose operator[] finds element i's fragment as (int)(i * (1.0 / E)) and
    its place as i % E (fragmentedvector.h:147-152, 320); where the product rounds below an
    integer k, element k E reads the first record of fragment k - 1."""
    E = max(5000000 // record_bytes, 1)
    i = np.arange(a.shape[0], dtype=np.int64)
    node = (i.astype(np.float64) * (1.0 / E)).astype(np.int64)
    return np.ascontiguousarray(a[node * E + i % E])


def max_speed(vel):
    """FluidSimulation::_getMaximumMarkerParticleSpeed (fluidsimulation.cpp:10189-10203): the
    largest float dot(v, v), square-rooted in double."""
    v = _c(vel, F32)
    if v.shape[0] == 0:
        return 0.0
    d2 = (v[:, 0] * v[:, 0] + v[:, 1] * v[:, 1]) + v[:, 2] * v[:, 2]
    return float(np.sqrt(np.float64(d2.max())))


def update(n, dx, frame_dt, frame_index, min_steps, max_steps, pic, cfl, g, solid, pos, vel, tol=1e-9,
           maxit=900, evr=False):
    """FluidSimulation::update (fluidsimulation.cpp:10410-10543) over oracle substeps, with
    _calculateNextTimeStep (:10231-10263) for static solids and no fluid sources: the first
    substep of the first frame predicts |g| * frame_dt as the speed, later ones take the largest
    particle speed.  Returns the state, the substep lengths and each substep's statistics."""
    dt = max(frame_dt, 1e-6)
    substep_time = dt / min_steps
    remaining = dt
    glen = float(np.sqrt(np.float32(np.float32(g[0]) * np.float32(g[0]) + np.float32(g[1]) * np.float32(g[1])) +
                         np.float32(g[2]) * np.float32(g[2])))
    dts, stats = [], []
    k = 0
    while True:
        maxu = glen * dt if (frame_index == 0 and k == 0) else max_speed(vel)
        step = cfl * dx / (maxu + 1e-6)
        ts = min(dt / max(int(np.ceil(dt / step)), 1), remaining)
        if (dt - remaining) + ts > (k + 1) * substep_time:
            ts = min(substep_time, remaining)
        if k == max_steps - 1:
            ts = remaining
        remaining -= ts
        pos, vel, st = substep(n, dx, ts, pic, cfl, g, solid, pos, vel, tol, maxit,
                               evr=(dt, max_steps) if evr else None)
        dts.append(ts)
        stats.append(st)
        k += 1
        if not remaining > 1e-9:
            break
    return pos, vel, dts, stats


def p2g_apic(n, dx, pos, vel, aff9):
    """APIC transfer of all three components: [(field, valid)] as p2g."""
    pos = _c(pos, F32); vel = _c(vel, F32); aff9 = _c(aff9, F32)
    out = []
    for d in range(3):
        f = np.empty(_FSHAPE[d](n), F32); v = np.empty(_FSHAPE[d](n), U8)
        lib().oracle_p2g_apic_component(n, n, n, ctypes.c_double(dx), ctypes.c_double(radius(dx)), pos.shape[0],
                                        _p(pos), _p(vel), _p(aff9), d, _p(f), _p(v))
        out.append((f, v))
    return out


def g2p_apic(n, dx, pos, uvw):
    """APIC particle update: (velocities (N, 3), affine vectors (N, 9))."""
    pos = _c(pos, F32)
    vel = np.empty_like(pos)
    aff = np.empty((pos.shape[0], 9), F32)
    lib().oracle_g2p_apic(n, n, n, ctypes.c_double(dx), pos.shape[0], _p(pos), _p(vel), _p(aff),
                          *[_p(_c(a, F32)) for a in uvw])
    return vel, aff


def substep_apic(n, dx, dt, cfl, g, solid, pos, vel, aff9, tol=1e-9, maxit=900):
    pos = _c(pos, F32).copy(); vel = _c(vel, F32).copy(); aff9 = _c(aff9, F32).copy()
    stats = np.zeros(3, np.int32)
    err = ctypes.c_double(0)
    cnt = lib().oracle_substep_transfer(n, n, n, ctypes.c_double(dx), ctypes.c_double(dt), ctypes.c_double(0.0), cfl,
                                        ctypes.c_float(g[0]), ctypes.c_float(g[1]), ctypes.c_float(g[2]),
                                        _p(_c(solid, F32)), ctypes.c_double(tol), maxit, pos.shape[0], _p(pos),
                                        _p(vel), _p(aff9), _p(stats), ctypes.byref(err))
    return (pos[:cnt].copy(), vel[:cnt].copy(), aff9[:cnt].copy(),
            dict(iters=int(stats[0]), success=bool(stats[1]), fluid_cells=int(stats[2]), error=err.value))


def viscosity(n, dx, dt, liquid_phi, solid, visc, uvw, tol=1e-4, maxit=900, debug=False):
    """Viscosity solve (ViscositySolver) on (u, v, w).  visc: (n+1)^3 grid or a constant.
    Returns (u, v, w), stats dict and, with debug, the volumes, system, factor and solution."""
    u, v, w = [_c(a, F32).copy() for a in uvw]
    if np.isscalar(visc):
        visc = np.full((n + 1, n + 1, n + 1), visc, F32)
    nf = u.size + v.size + w.size
    stats = np.zeros(3, np.int32)
    err = ctypes.c_float(0)
    dbg = {}
    if debug:
        n1 = n + 1
        dbg = {"vol": np.zeros(n ** 3 + 3 * n * n * n1 + 3 * n * n1 * n1, F32), "index": np.zeros(nf, np.int32),
               "rowstart": np.zeros(nf + 1, np.uint32), "col": np.zeros(15 * nf, np.uint32),
               "val": np.zeros(15 * nf, F32), "rhs": np.zeros(nf, F32), "ic_invdiag": np.zeros(nf, F32),
               "ic_colstart": np.zeros(nf + 1, np.uint32), "ic_rowindex": np.zeros(15 * nf, np.uint32),
               "ic_value": np.zeros(15 * nf, F32), "soln": np.zeros(nf, F32)}
    g = lambda k: _p(dbg[k]) if debug else None
    lib().oracle_viscosity(n, n, n, ctypes.c_double(dx), ctypes.c_double(dt), _p(_c(liquid_phi, F32)),
                           _p(_c(solid, F32)), _p(_c(visc, F32)), ctypes.c_double(tol), maxit, _p(u), _p(v), _p(w),
                           _p(stats), ctypes.byref(err), g("vol"), g("index"), g("rowstart"), g("col"), g("val"),
                           g("rhs"), g("ic_invdiag"), g("ic_colstart"), g("ic_rowindex"), g("ic_value"), g("soln"))
    st = dict(n=int(stats[0]), iters=int(stats[1]), success=bool(stats[2]), error=err.value)
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
        sizes = [n ** 3, n * n * (n + 1), n * n * (n + 1), n * n * (n + 1), n * (n + 1) ** 2, n * (n + 1) ** 2,
                 n * (n + 1) ** 2]
        parts = np.split(dbg["vol"], np.cumsum(sizes)[:-1])
        n1 = n + 1
        shapes = [(n, n, n), (n, n, n1), (n, n1, n), (n1, n, n), (n1, n1, n), (n1, n, n1), (n, n1, n1)]
        dbg["vol"] = dict(zip(["center", "u", "v", "w", "eu", "ev", "ew"], [p.reshape(s) for p, s in zip(parts, shapes)]))
    return (u, v, w), st, dbg


def substep_visc(n, dx, dt, pic, cfl, g, solid, pos, vel, visc, tol=1e-9, maxit=900):
    """One FLIP substep with the viscosity solve (constant viscosity) after the body force."""
    pos = _c(pos, F32).copy(); vel = _c(vel, F32).copy()
    stats = np.zeros(3, np.int32)
    err = ctypes.c_double(0)
    cnt = lib().oracle_substep_full(n, n, n, ctypes.c_double(dx), ctypes.c_double(dt), ctypes.c_double(pic), cfl,
                                    ctypes.c_float(g[0]), ctypes.c_float(g[1]), ctypes.c_float(g[2]),
                                    _p(_c(solid, F32)), ctypes.c_double(tol), maxit, pos.shape[0], _p(pos), _p(vel),
                                    None, ctypes.c_double(visc), _p(stats), ctypes.byref(err))
    return pos[:cnt].copy(), vel[:cnt].copy(), dict(iters=int(stats[0]), success=bool(stats[1]),
                                                     fluid_cells=int(stats[2]), error=err.value)


def curvature_grid(n, dx, phi):
    """Surface curvature grid (ParticleLevelSet::calculateCurvatureGrid): (surface_phi, curvature)."""
    phi = _c(phi, F32)
    surf = np.empty((n, n, n), F32)
    k = np.empty((n, n, n), F32)
    lib().oracle_curvature_grid(n, n, n, ctypes.c_double(dx), _p(phi), _p(surf), _p(k))
    return surf, k


def pressure_solve_tension(n, dx, dt, phi, weights, uvw, curvature, k_st, tol=1e-9, maxit=900, float_scalars=True):
    """pressure_solve with the surface tension term (curvature grid, tension constant)."""
    pr = np.empty((n, n, n), F32)
    stats = np.zeros(2, np.int32)
    err = ctypes.c_double(0)
    args = [_c(phi, F32)] + [_c(a, F32) for a in weights] + [_c(a, F32) for a in uvw]
    nf = lib().oracle_pressure_solve_tension(n, n, n, ctypes.c_double(dx), ctypes.c_double(dt), *[_p(a) for a in args],
                                             _p(_c(curvature, F32)), ctypes.c_double(k_st), ctypes.c_double(tol), maxit,
                                             1 if float_scalars else 0, _p(pr), _p(stats), ctypes.byref(err))
    return pr, int(stats[0]), bool(stats[1]), err.value, nf


def apply_pressure_tension(n, dx, dt, phi, weights, pressure, uvw, curvature, k_st):
    """Pressure application with the surface tension term in the ghost pressure."""
    u, v, w = [_c(a, F32).copy() for a in uvw]
    vu = np.empty(u.shape, np.uint8); vv = np.empty(v.shape, np.uint8); vw = np.empty(w.shape, np.uint8)
    args = [_c(phi, F32)] + [_c(a, F32) for a in weights] + [_c(pressure, F32), _c(curvature, F32)]
    lib().oracle_apply_pressure_tension(n, n, n, ctypes.c_double(dx), ctypes.c_double(dt), *[_p(a) for a in args],
                                        ctypes.c_double(k_st), _p(u), _p(v), _p(w), _p(vu), _p(vv), _p(vw))
    return (u, v, w), (vu, vv, vw)


def substep_tension(n, dx, dt, pic, cfl, g, solid, pos, vel, tension, tol=1e-9, maxit=900):
    """One FLIP substep with surface tension (curvature grid + ghost-fluid tension term)."""
    pos = _c(pos, F32).copy(); vel = _c(vel, F32).copy()
    stats = np.zeros(3, np.int32)
    err = ctypes.c_double(0)
    cnt = lib().oracle_substep_tension(n, n, n, ctypes.c_double(dx), ctypes.c_double(dt), ctypes.c_double(pic), cfl,
                                       ctypes.c_float(g[0]), ctypes.c_float(g[1]), ctypes.c_float(g[2]),
                                       _p(_c(solid, F32)), ctypes.c_double(tol), maxit, pos.shape[0], _p(pos),
                                       _p(vel), None, ctypes.c_double(0.0), ctypes.c_double(tension), _p(stats),
                                       ctypes.byref(err))
    return pos[:cnt].copy(), vel[:cnt].copy(), dict(iters=int(stats[0]), success=bool(stats[1]))


def solid_level_set(n, dx, objects=(), jitter=None):
    """Solid level set of the closed domain and static mesh obstacles (FluidSimulation::
    _addStaticObjectsToSDF).  objects: (vertices (V, 3), triangles (T, 3), flags, expansion) with
    flags bit0 inverted, bit1 disabled.  jitter: (K, 3) line offsets of the first K inside tests."""
    nv = np.array([len(o[0]) for o in objects] or [0], np.int32)
    nt = np.array([len(o[1]) for o in objects] or [0], np.int32)
    verts = _c(np.concatenate([np.asarray(o[0], np.float32).reshape(-1, 3) for o in objects])
               if objects else np.zeros((1, 3)), F32)
    tris = _c(np.concatenate([np.asarray(o[1], np.int32).reshape(-1, 3) for o in objects])
              if objects else np.zeros((1, 3)), np.int32)
    flags = np.array([o[2] for o in objects] or [0], np.int32)
    exp = np.array([o[3] for o in objects] or [0.0], np.float32)
    jit = None if jitter is None else _c(np.asarray(jitter, np.float32).reshape(-1, 3), F32)
    phi = np.empty((n + 1, n + 1, n + 1), F32)
    lib().oracle_solid_level_set(n, n, n, ctypes.c_double(dx), len(objects), _p(nv), _p(nt), _p(verts), _p(tris),
                                 _p(flags), _p(exp), 0 if jit is None else jit.shape[0], _p(jit), _p(phi))
    return phi


def mesh_objects(d):
    """The obstacles of a mesh golden fixture as solid_level_set's `objects`."""
    out, vo, to = [], 0, 0
    for nv, nt, fl, e in zip(d["nverts"], d["ntris"], d["flags"], d["expansion"]):
        out.append((d["verts"][vo:vo + nv], d["tris"][to:to + nt], int(fl), float(e)))
        vo += int(nv)
        to += int(nt)
    return out


def ffp3(n, dx, surface, pos, vel, ids, flags, amount, boundary_width=1, surface_width=0.90):
    """FFP3 fluid-particle output (FluidSimulation::_generateFluidParticleDataFFP3 and its file
    data): (types, {"pos", "id", "vel", "speed"} -> bytes)."""
    pos, vel = _c(pos, F32), _c(vel, F32)
    ids = _c(ids, np.uint16)
    np_ = pos.shape[0]
    cap = 16 + 12 * 65536 + 12 * np_
    outs = [np.zeros(cap, np.uint8) for _ in range(4)]
    types = np.zeros(np_, np.uint8)
    sizes = np.zeros(4, np.int64)
    lib().oracle_ffp3(n, n, n, ctypes.c_double(dx), _p(_c(surface, F32)), np_, _p(pos), _p(vel), _p(ids),
                      int(boundary_width), ctypes.c_float(surface_width), ctypes.c_double(amount), int(flags),
                      _p(types), *[_p(o) for o in outs], _p(sizes))
    return types, {k: o[:int(s)].copy() for k, o, s in zip(("pos", "id", "vel", "speed"), outs, sizes)}


def surface_level_set(n, dx, solid, pos):
    """The liquid level set of the particles (post-processed against the solid) and its surface
    level set, as FluidSimulation::_outputFluidParticles recomputes them."""
    phi = postprocess_sdf(n, dx, solid, liquid_sdf(n, dx, pos))
    return curvature_grid(n, dx, phi)[0]
