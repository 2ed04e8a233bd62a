"""CPU k-eigenvalue solve of the pure-upwind SN problem -- TEST/BASELINE INFRASTRUCTURE ONLY.

The reference solves SN k-eigenproblems by assembling R and F over (cell, group,
direction) and handing them to SLEPc (Krylov-Schur, shift-and-invert with a sparse LU of
R; SNSolver.cxx:344-670, petsc.cxx:175-204).  Its matrix for the 64x64x32 S8 workload
holds about 6.8e9 nonzeros (some 82 GB), which no host here can factor, so this module
restates the eigen-solve in the form that scales: the same operator, solved by power
iteration in scalar-flux space with GMRES over transport sweeps (oracle/cpu_sweep.c) for
the inner systems.  With pure upwind faces (mixed-face-interpolation 1.0) and no LS
boundary correction a sweep inverts the streaming + collision rows of R exactly
(SNSolver.cxx:397, 445-597), so the fixed point is the reference operator's eigenpair;
the tests check it against the oracle's direct solve (pampa_oracle.run_input) on small
meshes.  The outputs are normalised as SNSolver::calculateScalarFlux, normalizeScalarFlux
and normalizeAngularFlux do (SNSolver.cxx:272-341, NeutronicSolver.cxx:46-116).

Used by tests (checker at sizes the direct solve cannot reach), by bench.py's CPU legs
(cpu_baseline and --impl reference) and by bench.py's parity check after its timed
region.  The product never imports it.
"""

from __future__ import annotations

import ctypes as C
import math
import os
import subprocess
import time

import numpy as np

from . import pampa_oracle as po

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
LIB = os.path.join(REF_DIR, "libcpu_sweep.so")


def build() -> str:
    os.makedirs(REF_DIR, exist_ok=True)
    src = os.path.join(HERE, "cpu_sweep.c")
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(src) or _foreign(LIB):
        subprocess.run(["gcc", "-O3", "-fopenmp", "-shared", "-fPIC", src, "-o", LIB], check=True)
    return LIB


def _foreign(path: str) -> bool:
    """True when the library was built for another machine architecture."""
    import platform
    stamp = path + ".arch"
    ok = os.path.exists(stamp) and open(stamp).read().strip() == platform.machine()
    if not ok:
        with open(stamp, "w") as fh:
            fh.write(platform.machine())
    return not ok


_L = None


def _lib():
    global _L
    if _L is None:
        L = C.CDLL(build())
        L.cpu_sweep_threads.restype = C.c_int
        L.cpu_upwind_order.restype = C.c_int
        L.cpu_sub_norm.restype = C.c_double
        L.cpu_norm.restype = C.c_double
        _L = L
    return _L


def _p(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


class SNCpu:
    """Operator data of one pure-upwind SN problem for the CPU sweeps and eigen-solve."""

    def __init__(self, prob: po.Problem, threads: int | None = None):
        if prob.solver != "sn":
            raise ValueError("not an SN problem")
        if prob.delta != 1.0 or prob.ls:
            raise ValueError("the sweep solve needs mixed-face-interpolation 1.0 and no LS correction")
        L = _lib()
        self.threads = threads or L.cpu_sweep_threads()
        self.prob = prob
        mesh = prob.mesh
        n, F, G = mesh.n, mesh.F, prob.G
        dirs, w, refl = po.quadrature(prob.order)
        M = len(w)
        st, nsf, ksf, chi, ss, D = po._material_tables(prob)
        self.n, self.F, self.G, self.M = n, F, G, M
        self.dirs, self.w = np.ascontiguousarray(dirs), np.ascontiguousarray(w)
        self.st, self.nsf, self.ksf, self.chi, self.ss = st, nsf, ksf, chi, ss
        self.ss_c, self.chi_c, self.nsf_c = (np.ascontiguousarray(a, dtype=np.float64) for a in (ss, chi, nsf))
        self.mat = mesh.materials.astype(np.int32)
        self.vol = mesh.volumes.astype(np.float64)
        gc = po.gauss_coefs(mesh, prob.delta)
        bcs = prob.boundary_conditions()
        kind = np.full((F, n), 3, dtype=np.int32)
        nbr = np.full((F, n), -1, dtype=np.int32)
        rslot = np.full((F, n), -1, dtype=np.int32)
        slot_cell, slot_face = [], []
        for f in range(F):
            has = f < mesh.num_faces
            nb = mesh.neighbors[:, f]
            inter = has & (nb >= 0) & (nb < po.PAD)
            kind[f, inter] = 0
            nbr[f, inter] = nb[inter]
            for c in np.nonzero(has & (nb < 0))[0]:
                t = bcs.get(int(-nb[c]), po.BoundaryCondition()).type
                if t == po.BC_VACUUM:
                    kind[f, c] = 1
                elif t == po.BC_REFLECTIVE:
                    kind[f, c] = 2
                    rslot[f, c] = len(slot_cell)
                    slot_cell.append(int(c))
                    slot_face.append(f)
                else:
                    raise ValueError("boundary condition not supported by the sweep")
        self.nf = mesh.num_faces.astype(np.int32)
        self.kind, self.nbr, self.rslot = kind, nbr, rslot
        self.area = np.ascontiguousarray(mesh.areas.T)
        self.nrm = np.ascontiguousarray(np.transpose(mesh.normals, (1, 0, 2)))
        self.gauss = np.ascontiguousarray(np.transpose(gc, (1, 0, 2)))
        # directions grouped by their upwind pattern over the interior faces; one upwind
        # cell order per pattern
        inter_nf = (np.arange(F)[None, :] < mesh.num_faces[:, None]) & (mesh.neighbors >= 0) & \
            (mesh.neighbors < po.PAD)
        mu_all = np.einsum("nfd,md->mnf", mesh.normals, dirs)
        keys, pats = {}, []
        pat_of_dir = np.zeros(M, dtype=np.int64)
        for m in range(M):
            key = ((mu_all[m] < 0.0) & inter_nf).tobytes()
            if key not in keys:
                keys[key] = len(pats)
                pats.append([])
            pat_of_dir[m] = keys[key]
            pats[keys[key]].append(m)
        self.npat = len(pats)
        self.pat_dirs_ptr = np.cumsum([0] + [len(v) for v in pats]).astype(np.int32)
        self.pat_dirs = np.array([m for v in pats for m in v], dtype=np.int32)
        self.order = np.zeros((self.npat, n), dtype=np.int32)
        for p, v in enumerate(pats):
            if L.cpu_upwind_order(n, F, _p(self.nf), _p(self.kind), _p(self.nbr), _p(self.nrm),
                                  _p(np.ascontiguousarray(dirs[v[0]])), _p(self.order[p])):
                raise ValueError("the upwind graph of a direction has a cycle")
        # reflective inflow: slot s, incoming direction m (mu < 0) reads the outgoing
        # angular flux of the reflected direction in the same cell.  SNSolver.cxx:539-543
        # picks the axis from the normal of face f of cells 0, 1, 2 (the loop index
        # shadows the cell); that is kept.
        self.nrefl = len(slot_cell)
        e_slot, e_m, e_m2 = [], [], []
        for s, (c, f) in enumerate(zip(slot_cell, slot_face)):
            ax = -1
            for a in range(3):
                if abs(float(mesh.normals[a, f, a])) > 1.0 - 1e-6:
                    ax = a
            for m in range(M):
                if float(dirs[m] @ mesh.normals[c, f]) < 0.0:
                    if ax < 0:
                        raise ValueError("reflected direction not found")
                    e_slot.append(s)
                    e_m.append(m)
                    e_m2.append(int(refl[m, ax]))
        self.e_slot = np.array(e_slot, dtype=np.int64)
        self.e_m = np.array(e_m, dtype=np.int64)
        self.e_m2 = np.array(e_m2, dtype=np.int64)
        self.e_cell = np.array(slot_cell, dtype=np.int64)[self.e_slot] if e_slot else np.zeros(0, np.int64)
        # upwind source of each face, cell-major: neighbour, -(slot + 2) or -1
        upw = np.where(kind == 0, nbr, -1)
        upw = np.where(kind == 2, -(rslot + 2), upw)
        self.upw = np.ascontiguousarray(upw.T.astype(np.int32))
        # cells with equal material, volume and face data share their sweep coefficients
        # (the same rows of R): per pattern a table [class][g][1 + F][directions] of rd and a_f
        win = np.where(kind == 0, self.gauss[:, :, 3] * self.area, np.where(kind == 2, self.area, 0.0))
        wout = np.where(kind == 0, self.gauss[:, :, 0] * self.area, np.where(kind == 3, 0.0, self.area))
        key = np.concatenate([self.mat[:, None].astype(np.float64), self.vol[:, None], kind.T.astype(np.float64),
                              self.nrm.transpose(1, 0, 2).reshape(n, -1), wout.T, win.T], axis=1)
        _, rep, cls = np.unique(key, axis=0, return_index=True, return_inverse=True)
        self.ncls = len(rep)
        self.cls = np.ascontiguousarray(cls.reshape(-1).astype(np.int32))
        mu = np.einsum("fcd,md->cfm", self.nrm[:, rep], dirs)                  # (ncls, F, M)
        kr = kind[:, rep].T[:, :, None]                                        # (ncls, F, 1)
        out = np.sum(np.where(mu > 0.0, mu * wout[:, rep].T[:, :, None], 0.0), axis=1)   # (ncls, M)
        den = st[self.mat[rep]][:, :, None] * self.vol[rep][:, None, None] + out[:, None, :]  # (ncls, G, M)
        rd = 1.0 / den
        ain = np.where((mu <= 0.0) & ((kr == 0) | (kr == 2)), -(mu * win[:, rep].T[:, :, None]), 0.0)  # (ncls,F,M)
        coef = np.zeros((self.ncls, G, 1 + F, M))                              # [c][g][k][m]
        coef[:, :, 0, :] = rd
        coef[:, :, 1:, :] = ain[:, None, :, :] * rd[:, :, None, :]
        self.pat_nd = np.diff(self.pat_dirs_ptr).astype(np.int32)
        tabs, tbase, tb = [], [], 0
        fmask = np.zeros((self.npat, self.ncls), dtype=np.int32)
        for p in range(self.npat):
            dl = self.pat_dirs[self.pat_dirs_ptr[p]:self.pat_dirs_ptr[p + 1]]
            t = np.ascontiguousarray(coef[:, :, :, dl])
            tabs.append(t.reshape(-1))
            tbase.append(tb)
            tb += t.size
            nzf = np.any(t[:, :, 1:, :] != 0.0, axis=(1, 3))                   # (ncls, F)
            fmask[p] = np.sum(nzf * (1 << np.arange(F))[None, :], axis=1)
        self.tab = np.concatenate(tabs)
        self.tbase = np.array(tbase, dtype=np.int64)
        self.fmask = np.ascontiguousarray(fmask)
        # (group, pattern) blocks of psi and of the reflective inflow
        nb = G * self.npat
        nd_b = np.tile(self.pat_nd.astype(np.int64), G)
        self.pbase = np.concatenate([[0], np.cumsum(nd_b * n)[:-1]]).astype(np.int64)
        self.bbase = np.concatenate([[0], np.cumsum(nd_b * max(self.nrefl, 1))[:-1]]).astype(np.int64)
        # position of direction m inside its pattern
        self.pat_of = np.zeros(M, dtype=np.int64)
        self.pos_of = np.zeros(M, dtype=np.int64)
        for p in range(self.npat):
            for d, m in enumerate(self.pat_dirs[self.pat_dirs_ptr[p]:self.pat_dirs_ptr[p + 1]]):
                self.pat_of[m], self.pos_of[m] = p, d
        self.wpat = np.ascontiguousarray(w[self.pat_dirs])
        gg = np.arange(G)[None, :]
        blk = gg * self.npat
        # packed inflow entry (e, g) <-> bnd position; outgoing psi it is taken from
        self.bidx = (self.bbase[blk + self.pat_of[self.e_m][:, None]] +
                     self.e_slot[:, None] * self.pat_nd[self.pat_of[self.e_m]][:, None] +
                     self.pos_of[self.e_m][:, None]).reshape(-1)
        self.xidx = (self.pbase[blk + self.pat_of[self.e_m2][:, None]] +
                     self.e_cell[:, None] * self.pat_nd[self.pat_of[self.e_m2]][:, None] +
                     self.pos_of[self.e_m2][:, None]).reshape(-1)
        self.nG = n * G
        self.len = self.nG + len(e_slot) * G
        self.psi = np.zeros(G * n * M)
        self.bnd = np.zeros(max(self.nrefl, 1) * G * M)
        self.sweeps = 0

    # ---- building blocks -------------------------------------------------------------
    def sweep(self, q: np.ndarray, xb: np.ndarray | None) -> np.ndarray:
        """psi (per (group, pattern) blocks) of one sweep with isotropic source q and the
        packed reflective inflow xb."""
        bnd = None
        if self.nrefl:
            self.bnd[self.bidx] = xb
            bnd = self.bnd
        q = np.ascontiguousarray(q, dtype=np.float64)
        _lib().cpu_sweep_pat(self.n, self.G, self.F, self.npat, self.ncls, _p(self.pat_nd), _p(self.pbase),
                             _p(self.tbase), _p(self.bbase), _p(self.upw), _p(self.cls), _p(self.fmask),
                             _p(self.tab), _p(self.order), _p(q), _p(bnd) if bnd is not None else None,
                             _p(self.psi), self.threads)
        self.sweeps += 1
        return self.psi

    def moment(self, psi: np.ndarray) -> np.ndarray:
        phi0 = np.zeros(self.nG)
        _lib().cpu_moment_pat(self.n, self.G, self.npat, _p(self.pat_nd), _p(self.pbase), _p(self.wpat),
                              _p(psi), _p(phi0), self.threads)
        return phi0

    def extract(self, psi: np.ndarray) -> np.ndarray:
        """Packed reflective inflow [entry][g] of the current psi."""
        return psi[self.xidx] if self.nrefl else np.zeros(0)

    def angular(self, psi: np.ndarray) -> np.ndarray:
        """psi in the reference's layout [i][g][m]."""
        n, G, M = self.n, self.G, self.M
        out = np.zeros((n, G, M))
        for g in range(G):
            for p in range(self.npat):
                nd = int(self.pat_nd[p])
                b = int(self.pbase[g * self.npat + p])
                dl = self.pat_dirs[self.pat_dirs_ptr[p]:self.pat_dirs_ptr[p + 1]]
                out[:, g, dl] = psi[b:b + n * nd].reshape(n, nd)
        return out.reshape(-1)

    def source(self, phi0: np.ndarray, b: np.ndarray | None, lam: float) -> np.ndarray:
        """q[i,g] = V sum_g2 (sigma_s(g2->g) + lam chi_g nu_sigma_f(g2)) phi0[i,g2] (+ b)."""
        q = np.zeros(self.nG)
        _lib().cpu_source(self.n, self.G, _p(self.mat), _p(self.vol), _p(self.ss_c), _p(self.chi_c),
                          _p(self.nsf_c), C.c_double(lam), _p(np.ascontiguousarray(phi0)),
                          _p(np.ascontiguousarray(b)) if b is not None else None, _p(q), self.threads)
        return q

    def T(self, x: np.ndarray, b: np.ndarray | None, lam: float) -> np.ndarray:
        """[phi0' | inflow'] after one sweep driven by x's scalar flux and inflow."""
        psi = self.sweep(self.source(x[:self.nG], b, lam), x[self.nG:])
        return np.concatenate([self.moment(psi), self.extract(psi)])

    def fission(self, phi0: np.ndarray) -> np.ndarray:
        return self.vol * np.sum(self.nsf[self.mat] * phi0.reshape(self.n, self.G), axis=1)

    # ---- eigen-solve -----------------------------------------------------------------
    def solve(self, tol_k: float = 1e-10, tol_flux: float = 1e-9, shift: float = 0.05, eta: float = 0.2,
              restart: int = 30, max_outer: int = 5000, power: float | None = None,
              shift_when_dk: float = 0.1) -> dict:
        """Power iteration with Wielandt shift and GMRES(restart) over sweeps, in FP64 (the
        GPU solver's algorithm: the shift starts after three outer iterations once
        |dk| < shift_when_dk)."""
        t0 = time.perf_counter()
        self.sweeps = 0
        nG, n, G = self.nG, self.n, self.G
        x = np.zeros(self.len)
        x[:nG] = 1.0
        fs = self.fission(x[:nG])
        S = fs.sum()
        if not S > 0.0:
            raise ValueError("no fission source in the initial flux")
        k_prev, lam = 1.0, 0.0
        f = fs / S
        fs_old = f.copy()
        b = (self.chi[self.mat] * f[:, None]).reshape(-1)
        x /= S
        outer = inner = 0
        converged = False
        for outer in range(1, max_outer + 1):
            x *= 1.0 / (1.0 / k_prev - lam)
            r = self.T(x, b, lam) - x
            scale = self._norm(x)
            rnorm = self._norm(r)
            if rnorm > 1e-14 * scale:
                d, it = self._gmres(r, lam, eta, 1e-14 * scale, restart)
                x += d
                inner += it
            fs = self.fission(x[:nG])
            S = fs.sum()
            k = 1.0 / (lam + 1.0 / S)
            x /= S
            f = fs / S
            change = math.sqrt(np.sum((f - fs_old) ** 2) / np.sum(f * f))
            fs_old = f
            b = (self.chi[self.mat] * f[:, None]).reshape(-1)
            dk = abs(k - k_prev)
            k_prev = k
            if dk < tol_k and change < tol_flux:
                converged = True
                break
            if outer >= 3 and dk < shift_when_dk and shift > 0.0:
                lam = 1.0 / max(k * (1.0 + shift), k + 50.0 * dk)
        if not converged:
            raise RuntimeError("CPU SN power iteration did not converge")
        k = k_prev
        # psi from the converged state: one sweep with the eigen-equation's source
        psi = self.sweep(self.source(x[:nG], None, 1.0 / k), x[nG:]).copy()
        phi0 = self.moment(psi)
        pw = self.prob.power if power is None else power
        p0 = float(np.sum(phi0.reshape(n, G) * self.ksf[self.mat] * self.vol[:, None]))
        fnorm = pw / p0
        # phi = 4 pi phi0 (SNSolver.cxx:272-299) scaled to sum phi kappa_sigma_f V = power
        # (NeutronicSolver.cxx:46-78): the 4 pi cancels
        phi = phi0 * fnorm
        psi_ref = self.angular(psi) * fnorm   # SNSolver.cxx:302-341
        q = np.sum(phi.reshape(n, G) * self.ksf[self.mat] * self.vol[:, None], axis=1)
        P = np.sum(phi.reshape(n, G) * self.nsf[self.mat] * self.vol[:, None] / k, axis=1)
        return dict(keff=k, phi=phi, psi=psi_ref, q=q, P=P, power=float(q.sum()), outer_iterations=outer,
                    inner_iterations=inner, sweeps=self.sweeps, seconds=time.perf_counter() - t0,
                    threads=self.threads)

    # Gram-Schmidt products in C with the sweeps' OpenMP threads (a threaded BLAS next to
    # them would contend for the same cores)
    def _dots(self, V: np.ndarray, nv: int, w: np.ndarray) -> np.ndarray:
        h = np.zeros(nv)
        _lib().cpu_dots(C.c_longlong(self.len), nv, _p(V), _p(w), _p(h), self.threads)
        return h

    def _norm(self, x: np.ndarray) -> float:
        x = np.ascontiguousarray(x)
        return _lib().cpu_norm(C.c_longlong(x.size), _p(x), self.threads)

    def _sub_norm(self, V: np.ndarray, nv: int, h: np.ndarray, w: np.ndarray) -> float:
        return _lib().cpu_sub_norm(C.c_longlong(self.len), nv, _p(V), _p(np.ascontiguousarray(h)), _p(w),
                                   self.threads)

    def _gmres(self, r: np.ndarray, lam: float, rtol: float, atol: float, m: int):
        """GMRES(m) with classical Gram-Schmidt twice on (I - T_lam) d = r, d from zero."""
        L = self.len
        V = np.zeros((m + 1, L))
        d = np.zeros(L)
        total = 0
        beta0 = self._norm(r)
        tol = max(rtol * beta0, atol)
        res = beta0
        first = True
        while True:
            if first:
                V[0] = r
                first = False
            else:
                V[0] = r - (d - self.T(d, None, lam))
            beta = self._norm(V[0])
            res = beta
            if beta <= tol:
                break
            V[0] /= beta
            H = np.zeros((m + 1, m))
            g = np.zeros(m + 1)
            g[0] = beta
            cs, sn = np.zeros(m), np.zeros(m)
            j = 0
            while j < m:
                wv = V[j] - self.T(V[j], None, lam)
                # classical Gram-Schmidt, a second pass only when the norm fell below half
                # its value before the first (cancellation), as the GPU solve does
                w0 = self._norm(wv)
                h = self._dots(V, j + 1, wv)
                hn = self._sub_norm(V, j + 1, h, wv)
                if not hn >= 0.5 * w0:
                    h2 = self._dots(V, j + 1, wv)
                    hn = self._sub_norm(V, j + 1, h2, wv)
                    h += h2
                H[:j + 1, j] = h
                H[j + 1, j] = hn
                total += 1
                if hn > 0.0:
                    V[j + 1] = wv / hn
                for i in range(j):
                    a = cs[i] * H[i, j] + sn[i] * H[i + 1, j]
                    H[i + 1, j] = -sn[i] * H[i, j] + cs[i] * H[i + 1, j]
                    H[i, j] = a
                rr = math.hypot(H[j, j], H[j + 1, j])
                cs[j], sn[j] = H[j, j] / rr, H[j + 1, j] / rr
                H[j, j], H[j + 1, j] = rr, 0.0
                g[j + 1] = -sn[j] * g[j]
                g[j] = cs[j] * g[j]
                res = abs(g[j + 1])
                j += 1
                if res <= tol or hn == 0.0:
                    break
            y = np.linalg.solve(np.triu(H[:j, :j]), g[:j])
            self._sub_norm(V, j, -y, d)
            if res <= tol:
                break
        return d, total


def solve_input(path: str, threads: int | None = None, **kw) -> dict:
    """The CPU sweep solve of a .pmp input (pure upwind SN problems only)."""
    return SNCpu(po.read_problem(path), threads).solve(**kw)
