"""FP64 model of one substep's particle-state map (x0, v0) -> (x1, v1) (tests only).

The discrete structure is frozen at the base state the model is built from: liquid level
set and cell classification, valid flags, extrapolation layers, pressure cells (see
csrc/adjoint_kernels.cu).  Within it the map is affine in v0 and smooth in x0 (P2G kernel
weights, trilinear sampling, RK3).  This module builds it in float64 with numpy/scipy from
the same discrete structure the engine uses, so that:
  - finite differences through it are exact up to FP64 rounding, and
  - its transpose gives the reference gradient (sparse LU, or a dense solve on small grids).
It follows the reference formulas: transfer kernel velocityadvector.cpp:467-536,
extrapolation gridutils.h:43-163, system pressuresolver.cpp:624-867, projection
pressuresolver.cpp:1047-1205, sampling macvelocityfield.cpp:519-645, PIC/FLIP blend
fluidsimulation.cpp:6771-6789, RK3 fluidsimulation.cpp:7616-7623 (no particle in the
test scenes reaches a collision).
"""
import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

import oracle_api as O


def _fshape(n, c):
    return (n + (c == 2), n + (c == 1), n + (c == 0))     # (d, h, w) of face grid c


def _fidx(n, c, i, j, k):
    w = n + (c == 0); h = n + (c == 1)
    return i + w * (j + h * k)


def _kernel_parts(n, dx, r, x, c):
    """P2G kernel weights w_pf and their gradients dw_pf/dx_p (a = x, y, z) as sparse
    (faces x particles) matrices, for face component c at particle positions x."""
    off = np.full(3, 0.5 * dx); off[c] = 0.0
    s = x - off
    base = np.floor(s / dx).astype(np.int64)
    d, h, w = _fshape(n, c)
    rows, cols, vals, grads = [], [], [], [[], [], []]
    for oz in (-1, 0, 1, 2):
        for oy in (-1, 0, 1, 2):
            for ox in (-1, 0, 1, 2):
                f = base + np.array([ox, oy, oz])
                ok = (f[:, 0] >= 0) & (f[:, 1] >= 0) & (f[:, 2] >= 0) & (f[:, 0] < w) & (f[:, 1] < h) & (f[:, 2] < d)
                vec = f * dx - s                      # face - particle
                d2 = (vec ** 2).sum(1)
                ok &= d2 < r * r
                wgt = 1.0 - (4 / 9) * d2 ** 3 / r ** 6 + (17 / 9) * d2 ** 2 / r ** 4 - (22 / 9) * d2 / r ** 2
                dw = -3 * (4 / 9) * d2 ** 2 / r ** 6 + 2 * (17 / 9) * d2 / r ** 4 - (22 / 9) / r ** 2
                idx = np.nonzero(ok)[0]
                rows.append(_fidx(n, c, f[idx, 0], f[idx, 1], f[idx, 2]))
                cols.append(idx)
                vals.append(wgt[idx])
                for a in range(3):
                    grads[a].append((-2.0 * dw * vec[:, a])[idx])
    nf = d * h * w
    R, C = np.concatenate(rows), np.concatenate(cols)
    M = sp.csr_matrix((np.concatenate(vals), (R, C)), shape=(nf, x.shape[0]))
    G = [sp.csr_matrix((np.concatenate(grads[a]), (R, C)), shape=(nf, x.shape[0])) for a in range(3)]
    return M, G


def _interp_parts(n, dx, x, c):
    """Trilinear sampling of face component c at points x (zero outside the domain): the
    (points x faces) matrix and its derivatives with respect to the point (a = x, y, z)."""
    d, h, w = _fshape(n, c)
    inside = np.all((x >= 0) & (x < n * dx), axis=1)
    off = np.full(3, 0.5 * dx); off[c] = 0.0
    s = x - off
    b = np.floor(s / dx).astype(np.int64)
    t = s / dx - b
    rows, cols, vals, ders = [], [], [], [[], [], []]
    for dk in (0, 1):
        for dj in (0, 1):
            for di in (0, 1):
                f = b + np.array([di, dj, dk])
                ok = inside & (f[:, 0] >= 0) & (f[:, 1] >= 0) & (f[:, 2] >= 0) & (f[:, 0] < w) & (f[:, 1] < h) & (f[:, 2] < d)
                fx = t[:, 0] if di else 1 - t[:, 0]
                fy = t[:, 1] if dj else 1 - t[:, 1]
                fz = t[:, 2] if dk else 1 - t[:, 2]
                sx, sy, sz = (1.0 if di else -1.0) / dx, (1.0 if dj else -1.0) / dx, (1.0 if dk else -1.0) / dx
                idx = np.nonzero(ok)[0]
                rows.append(idx); cols.append(_fidx(n, c, f[idx, 0], f[idx, 1], f[idx, 2]))
                vals.append((fx * fy * fz)[idx])
                ders[0].append((sx * fy * fz)[idx]); ders[1].append((fx * sy * fz)[idx]); ders[2].append((fx * fy * sz)[idx])
    R, C = np.concatenate(rows), np.concatenate(cols)
    shape = (x.shape[0], d * h * w)
    I = sp.csr_matrix((np.concatenate(vals), (R, C)), shape=shape)
    D = [sp.csr_matrix((np.concatenate(ders[a]), (R, C)), shape=shape) for a in range(3)]
    return I, D


class SubstepModel:
    def __init__(self, n, pos0, vel0, solid, dt=1 / 240, pic=0.05, cfl=5, g=(0.0, -9.81, 0.0), dense=None):
        self.n, self.dx, self.dt, self.pic = n, 1.0 / n, dt, pic
        self.pos = np.asarray(pos0, np.float64)
        self.np_ = self.pos.shape[0]
        self.layers = O.layers(cfl)
        dx = self.dx
        self.r = 0.5 * dx * np.sqrt(3.0)
        # discrete structure from the oracle (reference arithmetic)
        self.weights = O.face_weights(n, solid)
        self.phi = O.postprocess_sdf(n, dx, solid, O.liquid_sdf(n, dx, pos0))
        p2g = O.p2g(n, dx, pos0, vel0)
        self.valid1 = [v.astype(bool).ravel() for _, v in p2g]
        self.S = [self._p2g_matrix(c) for c in range(3)]
        self.lay1 = [self._layers(c, self.valid1[c]) for c in range(3)]
        self.E1 = [self._extrap_ops(c, self.valid1[c], self.lay1[c]) for c in range(3)]
        self.gdt = [float(np.float32(np.float64(np.float32(gc)) * dt)) for gc in g]
        self._build_projection(dense if dense is not None else n <= 20)
        self.I = [self._g2p_matrix(c) for c in range(3)]
        self.E2 = [self._extrap_ops(c, self._valid2(c), self._layers(c, self._valid2(c))) for c in range(3)]

    # ---- P2G (FP64 weights, global frame) ----
    def _p2g_matrix(self, c):
        n, dx, r = self.n, self.dx, self.r
        off = np.full(3, 0.5 * dx); off[c] = 0.0
        s = self.pos - off
        base = np.floor(s / dx).astype(np.int64)
        rows, cols, vals = [], [], []
        d, h, w = _fshape(n, c)
        for oz in (-1, 0, 1, 2):
            for oy in (-1, 0, 1, 2):
                for ox in (-1, 0, 1, 2):
                    f = base + np.array([ox, oy, oz])
                    ok = (f[:, 0] >= 0) & (f[:, 1] >= 0) & (f[:, 2] >= 0) & (f[:, 0] < w) & (f[:, 1] < h) & (f[:, 2] < d)
                    d2 = ((f * dx - s) ** 2).sum(1)
                    ok &= d2 < r * r
                    wgt = 1.0 - (4 / 9) * d2 ** 3 / r ** 6 + (17 / 9) * d2 ** 2 / r ** 4 - (22 / 9) * d2 / r ** 2
                    idx = np.nonzero(ok)[0]
                    rows.append(_fidx(n, c, f[idx, 0], f[idx, 1], f[idx, 2]))
                    cols.append(idx)
                    vals.append(wgt[idx])
        nf = d * h * w
        M = sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(nf, self.np_))
        W = np.asarray(M.sum(axis=1)).ravel()
        scale = np.where(W > 1e-6, 1.0 / np.where(W > 0, W, 1.0), 1.0)
        return sp.diags(scale) @ M

    # ---- extrapolation: layer at which each cell is filled (gridutils.cpp:99-170) ----
    def _layers(self, c, valid):
        d, h, w = _fshape(self.n, c)
        v = np.asarray(valid).reshape(d, h, w)
        border = np.zeros((d, h, w), bool)
        border[0] = border[-1] = True; border[:, 0] = border[:, -1] = True; border[:, :, 0] = border[:, :, -1] = True
        st = np.where(border, 3, np.where(v, 2, 0)).astype(np.int8)
        lay = np.full((d, h, w), 255, np.int32)
        for L in range(self.layers):
            known = st == 2
            nbk = np.zeros_like(known)
            nbk[1:] |= known[:-1]; nbk[:-1] |= known[1:]
            nbk[:, 1:] |= known[:, :-1]; nbk[:, :-1] |= known[:, 1:]
            nbk[:, :, 1:] |= known[:, :, :-1]; nbk[:, :, :-1] |= known[:, :, 1:]
            waiting = (st == 0) & nbk
            st[known] = 3
            lay[waiting] = L
            st[waiting] = 2
        return lay.ravel()

    def _extrap_ops(self, c, valid, lay):
        d, h, w = _fshape(self.n, c)
        N = d * h * w
        flat = np.arange(N)   # flat index i + w*(j + h*k)
        ii = flat % w; jj = (flat // w) % h; kk = flat // (w * h)
        border = (ii == 0) | (jj == 0) | (kk == 0) | (ii == w - 1) | (jj == h - 1) | (kk == d - 1)
        ops = []
        for L in range(self.layers):
            tgt = np.nonzero(lay == L)[0]
            done = border | valid | (lay < L)
            rows, cols, vals = [], [], []
            keep = np.ones(N, bool); keep[tgt] = False
            ident = np.nonzero(keep)[0]
            rows.append(ident); cols.append(ident); vals.append(np.ones(ident.size))
            nb = [(1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1)]
            cnt = np.zeros(tgt.size)
            cand = []
            for (a, b, cc) in nb:
                m = tgt + a + w * (b + h * cc)
                ok = done[m]
                cnt += ok
                cand.append((m, ok))
            for m, ok in cand:
                rows.append(tgt[ok]); cols.append(m[ok]); vals.append(1.0 / cnt[ok])
            ops.append(sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(N, N)))
        return ops

    @staticmethod
    def _apply(ops, x):
        for M in ops:
            x = M @ x
        return x

    @staticmethod
    def _apply_T(ops, x):
        for M in reversed(ops):
            x = M.T @ x
        return x

    # ---- projection ----
    def _build_projection(self, dense):
        n, dx, dt = self.n, self.dx, self.dt
        phi = self.phi
        fl = np.zeros((n, n, n), bool)
        fl[1:-1, 1:-1, 1:-1] = phi[1:-1, 1:-1, 1:-1] < 0
        self.cells = np.argwhere(fl)            # (k, j, i), k-j-i order
        key = -np.ones((n, n, n), np.int64)
        key[fl] = np.arange(self.cells.shape[0])
        nc = self.cells.shape[0]
        mfac = dt / (dx * dx)
        wg = self.weights
        A_r, A_c, A_v = [], [], []
        D_r, D_c, D_v = [[], [], []], [[], [], []], [[], [], []]
        for q, (k, j, i) in enumerate(self.cells):
            vols = [wg[0][k, j, i + 1], wg[0][k, j, i], wg[1][k, j + 1, i], wg[1][k, j, i], wg[2][k + 1, j, i], wg[2][k, j, i]]
            nbs = [(k, j, i + 1), (k, j, i - 1), (k, j + 1, i), (k, j - 1, i), (k + 1, j, i), (k - 1, j, i)]
            diag = sum(float(v) for v in vols) * mfac
            pc = float(phi[k, j, i])
            for (kk, jj, ii), vol in zip(nbs, vols):
                pn = float(phi[kk, jj, ii])
                if pn < 0:
                    if key[kk, jj, ii] >= 0:
                        A_r.append(q); A_c.append(key[kk, jj, ii]); A_v.append(-float(vol) * mfac)
                else:
                    th = np.clip(pn / (pc + 1e-9), -25, 25)
                    diag -= float(vol) * mfac * th
            A_r.append(q); A_c.append(q); A_v.append(max(diag, 0.0))
            # b = -(1/dx)(w_r u_r - w_l u_l + ...)
            for c, (hi, lo) in enumerate([((i + 1, j, k), (i, j, k)), ((i, j + 1, k), (i, j, k)), ((i, j, k + 1), (i, j, k))]):
                D_r[c] += [q, q]
                D_c[c] += [_fidx(n, c, *hi), _fidx(n, c, *lo)]
                w_hi = wg[c][hi[2], hi[1], hi[0]]; w_lo = wg[c][lo[2], lo[1], lo[0]]
                D_v[c] += [-float(w_hi) / dx, float(w_lo) / dx]
        self.A = sp.csr_matrix((A_v, (A_r, A_c)), shape=(nc, nc))
        self.D = [sp.csr_matrix((D_v[c], (D_r[c], D_c[c])), shape=(nc, np.prod(_fshape(n, c)))) for c in range(3)]
        self.Ad = self.A.toarray() if dense else None
        self.lu = None if dense else spla.splu(self.A.tocsc())
        # faces: u_p = mask * (u_b - factor (p2~ - p1~)), untouched faces pass through
        factor = float(np.float32(dt / dx))
        self.G, self.mask = [], []
        for c in range(3):
            d, h, w = _fshape(n, c)
            N = d * h * w
            mask = np.zeros(N); gr, gc_, gv = [], [], []
            na = n
            for f in range(N):
                i = f % w; j = (f // w) % h; k = f // (w * h)
                ax = (i, j, k)[c]
                if ax == 0 or ax == na - 1:
                    mask[f] = 1.0
                    continue
                c1 = (k - (c == 2), j - (c == 1), i - (c == 0))
                in2 = ax < na
                c2 = (k, j, i) if in2 else c1
                f1 = phi[c1] < 0
                f2 = in2 and phi[c2] < 0
                if not (wg[c].ravel()[f] > 0 and (f1 or f2)):
                    continue
                mask[f] = 1.0
                k1 = key[c1]; k2 = key[c2] if in2 else -1
                eps = np.float32(1e-6)
                if f1 and f2:
                    terms = [(k1, -1.0), (k2, 1.0)]
                elif f1:
                    th = np.float32(np.float32(phi[c2] if in2 else 1.0) / np.float32(phi[c1] + eps))
                    th = float(np.clip(th, -25, 25)); terms = [(k1, th - 1.0)]
                else:
                    th = np.float32(np.float32(phi[c1]) / np.float32(phi[c2] + eps))
                    th = float(np.clip(th, -25, 25)); terms = [(k2, 1.0 - th)]
                for kc, v in terms:
                    if kc >= 0:
                        gr.append(f); gc_.append(kc); gv.append(factor * v)
            self.mask.append(mask)
            self.G.append(sp.csr_matrix((gv, (gr, gc_)), shape=(N, nc)))

    def _solve(self, rhs):
        if rhs.size == 0:
            return rhs
        if self.Ad is not None:
            return np.linalg.solve(self.Ad, rhs)
        return self.lu.solve(rhs)

    def _project(self, ub):
        b = sum(self.D[c] @ ub[c] for c in range(3))
        p = self._solve(b) if np.abs(b).max(initial=0) >= 1e-12 else np.zeros_like(b)
        return [self.mask[c] * (ub[c] - self.G[c] @ p) for c in range(3)]

    def _project_T(self, gup):
        gp = -sum(self.G[c].T @ (self.mask[c] * gup[c]) for c in range(3))
        gb = self._solve(gp)          # A is symmetric
        return [self.mask[c] * gup[c] + self.D[c].T @ gb for c in range(3)]

    # ---- G2P (trilinear, MAC offsets, zero outside) ----
    def _g2p_matrix(self, c):
        n, dx = self.n, self.dx
        d, h, w = _fshape(n, c)
        p = self.pos.copy()
        inside = np.all((p >= 0) & (p < n * dx), axis=1)
        off = np.full(3, 0.5 * dx); off[c] = 0.0
        s = p - off
        b = np.floor(s / dx).astype(np.int64)
        t = s / dx - b
        rows, cols, vals = [], [], []
        for dk in (0, 1):
            for dj in (0, 1):
                for di in (0, 1):
                    f = b + np.array([di, dj, dk])
                    ok = inside & (f[:, 0] >= 0) & (f[:, 1] >= 0) & (f[:, 2] >= 0) & (f[:, 0] < w) & (f[:, 1] < h) & (f[:, 2] < d)
                    wt = (t[:, 0] if di else 1 - t[:, 0]) * (t[:, 1] if dj else 1 - t[:, 1]) * (t[:, 2] if dk else 1 - t[:, 2])
                    idx = np.nonzero(ok)[0]
                    rows.append(idx); cols.append(_fidx(n, c, f[idx, 0], f[idx, 1], f[idx, 2])); vals.append(wt[idx])
        return sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(self.np_, d * h * w))

    # ---- the map and its transpose ----
    def forward(self, v0):
        v0 = np.asarray(v0, np.float64)
        ue = [self._apply(self.E1[c], self.S[c] @ v0[:, c]) for c in range(3)]
        saved = [ue[c].copy() for c in range(3)]
        ub = [ue[c] + self.gdt[c] for c in range(3)]
        up = self._project(ub)
        lay2 = [self._layers(c, self._valid2(c)) for c in range(3)]
        self.E2 = [self._extrap_ops(c, self._valid2(c), lay2[c]) for c in range(3)]
        uc = [self._apply(self.E2[c], up[c]) for c in range(3)]
        wg = [self.weights[c].ravel() for c in range(3)]
        uc = [np.where(wg[c] == 0, 0.0, uc[c]) for c in range(3)]
        sc = [np.where(wg[c] == 0, 0.0, saved[c]) for c in range(3)]
        a, b = self.pic, 1.0 - self.pic
        v1 = np.stack([a * (self.I[c] @ uc[c]) + b * (v0[:, c] + self.I[c] @ uc[c] - self.I[c] @ sc[c]) for c in range(3)], 1)
        return v1

    def _valid2(self, c):
        # faces set valid by the projection: active faces (not the untouched ones)
        n = self.n
        d, h, w = _fshape(n, c)
        f = np.arange(d * h * w)
        ax = (f % w, (f // w) % h, f // (w * h))[c]
        return (self.mask[c] > 0) & (ax != 0) & (ax != n - 1)

    def vjp(self, g1):
        """dL/dv0 for dL/dv1 = g1 (forward() must have run: it fixes the second extrapolation)."""
        g1 = np.asarray(g1, np.float64)
        a, b = self.pic, 1.0 - self.pic
        wg = [self.weights[c].ravel() for c in range(3)]
        g0 = b * g1
        gc = [np.where(wg[c] == 0, 0.0, (a + b) * (self.I[c].T @ g1[:, c])) for c in range(3)]
        gs = [np.where(wg[c] == 0, 0.0, -b * (self.I[c].T @ g1[:, c])) for c in range(3)]
        gup = [self._apply_T(self.E2[c], gc[c]) for c in range(3)]
        gub = self._project_T(gup)
        ge = [gub[c] + gs[c] for c in range(3)]
        for c in range(3):
            g0[:, c] += self.S[c].T @ self._apply_T(self.E1[c], ge[c])
        return g0


    # ---- the state map (x0, v0) -> (x1, v1) and its transpose ----
    def _fields(self, x, v):
        """P2G outputs (before extrapolation) with their normalisation and kernel parts, and
        the constrained current / saved fields, at state (x, v) with the frozen structure."""
        n, dx = self.n, self.dx
        us, scale, parts = [], [], []
        for c in range(3):
            M, G = _kernel_parts(n, dx, self.r, x, c)
            W = np.asarray(M.sum(axis=1)).ravel()
            scl = np.where(self.valid1[c], 1.0 / np.where(W > 0, W, 1.0), 1.0)
            us.append(scl * (M @ v[:, c])); scale.append(scl); parts.append((M, G))
        ue = [self._apply(self.E1[c], us[c]) for c in range(3)]
        up = self._project([ue[c] + self.gdt[c] for c in range(3)])
        wg = [self.weights[c].ravel() for c in range(3)]
        uc = [np.where(wg[c] == 0, 0.0, self._apply(self.E2[c], up[c])) for c in range(3)]
        sc = [np.where(wg[c] == 0, 0.0, ue[c]) for c in range(3)]
        return us, scale, parts, uc, sc

    def _sample_all(self, x, fields):
        """Velocity sampled at points x from three face fields, (N, 3), and its Jacobian
        J[p, c, a] = d u_c / d x_a, (N, 3, 3)."""
        val = np.zeros((x.shape[0], 3))
        J = np.zeros((x.shape[0], 3, 3))
        for c in range(3):
            I, D = _interp_parts(self.n, self.dx, x, c)
            val[:, c] = I @ fields[c]
            for a in range(3):
                J[:, c, a] = D[a] @ fields[c]
        return val, J

    def forward_xv(self, x0, v0, record=False):
        """(x1, v1) from (x0, v0); record=True keeps the linearisation for vjp_xv."""
        x0 = np.asarray(x0, np.float64)
        v0 = np.asarray(v0, np.float64)
        us, scale, parts, uc, sc = self._fields(x0, v0)
        a, b = self.pic, 1.0 - self.pic
        U0, J0 = self._sample_all(x0, uc)
        S0, Js = self._sample_all(x0, sc)
        v1 = a * U0 + b * (v0 + U0 - S0)
        h1, h2, h3 = 0.5 * self.dt, 0.75 * self.dt, self.dt / 9.0
        p2 = x0 + h1 * U0
        U2, J2 = self._sample_all(p2, uc)
        p3 = x0 + h2 * U2
        U3, J3 = self._sample_all(p3, uc)
        x1 = x0 + h3 * (2.0 * U0 + 3.0 * U2 + 4.0 * U3)
        if record:
            self._lin = dict(x0=x0, v0=v0, us=us, scale=scale, parts=parts, J0=J0, Js=Js, J2=J2, J3=J3, p2=p2, p3=p3)
        return x1, v1

    def vjp_xv(self, gx1, gv1):
        """(dL/dx0, dL/dv0) from (dL/dx1, dL/dv1) at the state recorded by forward_xv."""
        L = self._lin
        n, dx = self.n, self.dx
        a, b = self.pic, 1.0 - self.pic
        h1, h2, h3 = 0.5 * self.dt, 0.75 * self.dt, self.dt / 9.0
        gx1 = np.asarray(gx1, np.float64)
        gv1 = np.asarray(gv1, np.float64)
        jt = lambda J, g: np.einsum("pca,pc->pa", J, g)
        gk3 = 4.0 * h3 * gx1
        gp3 = jt(L["J3"], gk3)
        gk2 = 3.0 * h3 * gx1 + h2 * gp3
        gp2 = jt(L["J2"], gk2)
        gk1 = 2.0 * h3 * gx1 + h1 * gp2
        wc = gk1 + (a + b) * gv1
        ws = -b * gv1
        gx0 = gx1 + jt(L["J0"], wc) + gp2 + gp3 + jt(L["Js"], ws)
        gv0 = b * gv1
        wg = [self.weights[c].ravel() for c in range(3)]
        gc, gs = [], []
        for c in range(3):
            I0, _ = _interp_parts(n, dx, L["x0"], c)
            I2, _ = _interp_parts(n, dx, L["p2"], c)
            I3, _ = _interp_parts(n, dx, L["p3"], c)
            gcc = I0.T @ wc[:, c] + I2.T @ gk2[:, c] + I3.T @ gk3[:, c]
            gc.append(np.where(wg[c] == 0, 0.0, gcc))
            gs.append(np.where(wg[c] == 0, 0.0, I0.T @ ws[:, c]))
        gup = [self._apply_T(self.E2[c], gc[c]) for c in range(3)]
        gub = self._project_T(gup)
        ge = [self._apply_T(self.E1[c], gub[c] + gs[c]) for c in range(3)]
        for c in range(3):
            M, G = L["parts"][c]
            t1 = L["scale"][c] * ge[c]
            t2 = t1 * self.valid1[c] * L["us"][c]
            gv0[:, c] += M.T @ t1
            for ax in range(3):
                gx0[:, ax] += L["v0"][:, c] * (G[ax].T @ t1) - G[ax].T @ t2
        return gx0, gv0


class RolloutModel:
    """k substeps of SubstepModel, each with its structure frozen at its own base state.

    Without anchors the base states are the model's own FP64 trajectory from (pos0, vel0).
    With anchors (k + 1 states (x, v), e.g. the oracle's trajectory in reference arithmetic),
    substep i is frozen and linearised at anchors[i] and shifted by the constant
    anchors[i + 1] - F_i(anchors[i]), so that the chain passes exactly through the anchors: its
    derivatives are the FP64 linearisation along that trajectory, and finite differences of
    the chain stay consistent with its transpose."""

    def __init__(self, n, pos0, vel0, solid, k, anchors=None, **kw):
        self.steps, self.shift = [], []
        x, v = np.asarray(pos0, np.float64), np.asarray(vel0, np.float64)
        for i in range(k):
            if anchors is not None:
                x, v = np.asarray(anchors[i][0], np.float64), np.asarray(anchors[i][1], np.float64)
            m = SubstepModel(n, x.astype(np.float32), v.astype(np.float32), solid, **kw)
            x, v = m.forward_xv(x, v, record=True)
            if anchors is not None:
                dx_, dv_ = anchors[i + 1][0] - x, anchors[i + 1][1] - v
                x, v = x + dx_, v + dv_
            else:
                dx_, dv_ = 0.0, 0.0
            self.steps.append(m)
            self.shift.append((dx_, dv_))
        self.xk, self.vk = x, v

    def forward(self, x0, v0):
        x, v = np.asarray(x0, np.float64), np.asarray(v0, np.float64)
        for m, (dx_, dv_) in zip(self.steps, self.shift):
            x, v = m.forward_xv(x, v)
            x, v = x + dx_, v + dv_
        return x, v

    def vjp(self, gxk, gvk):
        gx, gv = np.asarray(gxk, np.float64), np.asarray(gvk, np.float64)
        for m in reversed(self.steps):
            gx, gv = m.vjp_xv(gx, gv)
        return gx, gv


def loss_vy2(v1, mask):
    m = int(mask.sum())
    return float((v1[mask, 1] ** 2).sum() / m) if m else 0.0


def loss_grad_vy2(v1, mask):
    g = np.zeros_like(v1)
    m = int(mask.sum())
    if m:
        g[mask, 1] = 2.0 * v1[mask, 1] / m
    return g
