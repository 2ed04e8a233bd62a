"""CPU oracle for the pampa k-eigenvalue hot path -- TEST INFRASTRUCTURE ONLY.

This module is a numpy/scipy restatement of the reference code's steady-state
(n = 0) neutronics path.  It is imported only by ``tests/``,
``__graft_entry__.smoke()`` and the CPU legs of ``bench.py`` as the checker; the
product (``pampa_gb300``) never imports it and has no CPU fallback.

What it restates (paths are relative to the reference project's ``src/``):

* ``.pmp`` tokenizer ............ input.cxx:4-62 (clean / get_next_line)
* materials ..................... Material.cxx:18-131, ConstantNuclearData.cxx:4-177,
                                  PrecursorData.cxx:4-56 (beta_total)
* Cartesian mesh ................ CartesianMesh.cxx:4-414 (face order -y,+x,+y,-x,-z,+z)
* unstructured extruded mesh .... UnstructuredExtrudedMesh.cxx:4-364, math.cxx:4-79
* split / BC-material removal ... Mesh.cxx:8-204
* diffusion R and F ............. DiffusionSolver.cxx:88-320 (n = 0 branch)
* SN quadrature ................. AngularQuadratureSet.cxx:4-209
* SN gradient schemes ........... SNSolver.cxx:127-269 (Gauss weights, LS boundary weights,
                                  including the transposed d(jg, f) indexing)
* SN R and F .................... SNSolver.cxx:344-631 (n = 0 branch, incl. the reflective
                                  normal lookup through cells 0..2)
* eigen-solve ................... petsc.cxx:175-204 (Krylov-Schur + shift-and-invert at 0 with
                                  a direct LU) -> here ARPACK on R^-1 F with a SuperLU factor
* normalisation / power ......... NeutronicSolver.cxx:46-116, SNSolver.cxx:272-341

Parity pin: ``tests/test_oracle_known_answers.py`` checks this module against the nine
keff values printed in the reference's golden output (test/check_ref.txt).  Flux vectors
are not printed by the reference, so flux parity rests on this restatement.
"""

from __future__ import annotations

import math
import os
from dataclasses import dataclass, field

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

# --------------------------------------------------------------------------------------
# Tokenizer (input.cxx:4-62)
# --------------------------------------------------------------------------------------


def _clean(s: str) -> str:
    if not s:
        return ""
    # input.cxx:14-15 replaces a tab *and the following character* with one space.
    while True:
        i = s.find("\t")
        if i < 0:
            break
        s = s[:i] + " " + s[i + 2:]
    while "  " in s:
        s = s.replace("  ", " ")
    if s == " ":
        return ""
    s = s.strip(" ")
    if s.startswith("#"):
        return ""
    return s


class Tokens:
    """Line reader with the reference's `get_next_line` semantics."""

    def __init__(self, path: str):
        self.path = path
        with open(path, "r") as fh:
            self.lines = fh.read().split("\n")
        self.pos = 0

    def next_line(self) -> list[str]:
        while self.pos < len(self.lines):
            line = _clean(self.lines[self.pos].rstrip("\r"))
            self.pos += 1
            if line:
                return line.split(" ")
        return []

    def read_values(self, n: int, cast=float) -> list:
        out = []
        while len(out) < n:
            line = self.next_line()
            if not line:
                raise ValueError(f"{self.path}: missing data")
            for w in line:
                if len(out) >= n:
                    raise ValueError(f"{self.path}: out-of-bounds data")
                out.append(cast(w))
        return out

    def read_rows(self, n: int, m: int | None, cast=float) -> list[list]:
        rows = []
        while len(rows) < n:
            line = self.next_line()
            if not line:
                raise ValueError(f"{self.path}: missing data")
            if m is not None and len(line) != m:
                raise ValueError(f"{self.path}: wrong row length")
            rows.append([cast(w) for w in line])
        return rows


def _resolve(path: str, base_dir: str) -> str:
    if os.path.isabs(path) or os.path.exists(path):
        return path
    return os.path.join(base_dir, path)


# --------------------------------------------------------------------------------------
# Boundary conditions (utils.hxx:96-117, input.cxx:364-404, Function.hxx:34-51)
# --------------------------------------------------------------------------------------

BC_NONE, BC_VACUUM, BC_REFLECTIVE, BC_ROBIN, BC_DIRICHLET, BC_ADIABATIC, BC_CONVECTION = range(7)
_BC_NAMES = {"vacuum": BC_VACUUM, "reflective": BC_REFLECTIVE, "robin": BC_ROBIN,
             "dirichlet": BC_DIRICHLET, "adiabatic": BC_ADIABATIC, "convection": BC_CONVECTION}


@dataclass
class BoundaryCondition:
    type: int = BC_NONE
    values: list = field(default_factory=list)  # single-valued functions only (steady state)


def _read_bc(line: list[str], i: int, tok: Tokens) -> BoundaryCondition:
    name = line[i]
    if name not in _BC_NAMES:
        raise ValueError("wrong boundary-condition type")
    bc = BoundaryCondition(_BC_NAMES[name])
    i += 1
    nvals = 1 if bc.type in (BC_ROBIN, BC_DIRICHLET) else 2 if bc.type == BC_CONVECTION else 0
    if nvals:
        if len(line) == i + nvals:
            bc.values = [float(v) for v in line[i:i + nvals]]
        elif len(line) == i + 2 and line[i + 1] == "{":
            # time-dependent table: steady state uses the first value (Function.hxx:37-38)
            n = int(line[i])
            tok.read_values(n)
            vals = [tok.read_values(n) for _ in range(nvals)]
            tok.next_line()
            bc.values = [v[0] for v in vals]
        else:
            raise ValueError("wrong number of function arguments")
    return bc


# --------------------------------------------------------------------------------------
# Materials (Material.cxx, ConstantNuclearData.cxx, PrecursorData.cxx)
# --------------------------------------------------------------------------------------

NU_DEFAULT = 2.4355
KAPPA_DEFAULT = 3.2e-11


@dataclass
class Material:
    name: str
    bc: bool = False
    split: bool = False
    fuel: bool = False
    G: int = 0
    has_nd: bool = False
    st: np.ndarray | None = None
    nsf: np.ndarray | None = None
    ksf: np.ndarray | None = None
    ss: np.ndarray | None = None      # ss[g_from, g_to]
    D: np.ndarray | None = None
    chi: np.ndarray | None = None     # effective fission spectrum
    beta_total: float = 0.0
    lam: np.ndarray | None = None     # precursor decay constants (precursor-data)
    beta: np.ndarray | None = None    # delayed-neutron fractions per precursor group
    chi_p: np.ndarray | None = None   # prompt fission spectrum
    chi_d: np.ndarray | None = None   # delayed fission spectrum
    vel: np.ndarray | None = None     # neutron velocities
    tref: list = field(default_factory=list)   # feedback data: reference temperatures
    sets: list = field(default_factory=list)   # feedback data: one Material per temperature

    def read(self, tok: Tokens):
        nd = {}
        while True:
            line = tok.next_line()
            if not line or line[0] == "}":
                break
            key = line[0]
            if key == "nuclear-data":
                if line[1] != "{":
                    raise ValueError("missing '{'")
                nd = self._read_nd(tok)
                self.has_nd = True
            elif key == "nuclear-data-set":
                # FeedbackNuclearData::read (FeedbackNuclearData.cxx): reference temperatures
                # and one constant data set per temperature
                if line[1] != "{":
                    raise ValueError("missing '{'")
                self.tref, sets = [], []
                while True:
                    l2 = tok.next_line()
                    if not l2 or l2[0] == "}":
                        break
                    if l2[0] == "temperature":
                        self.tref = list(tok.read_values(int(l2[1])))
                    elif l2[0] == "nuclear-data":
                        sets.append(self._read_nd(tok))
                    else:
                        raise ValueError(f"unrecognized keyword {l2[0]}")
                if not sets or len(sets) != len(self.tref):
                    raise ValueError("one nuclear-data set per reference temperature")
                self.has_nd = True
                nd = sets
            elif key == "precursor-data":
                while True:
                    l2 = tok.next_line()
                    if not l2 or l2[0] == "}":
                        break
                    if l2[0] == "precursor-groups":
                        npg = int(l2[1])
                    elif l2[0] == "lambda":
                        self.lam = np.array(tok.read_values(npg), dtype=np.float64)
                    elif l2[0] == "beta":
                        beta = tok.read_values(npg)
                        self.beta = np.array(beta, dtype=np.float64)
                        bt = 0.0
                        for b in beta:          # PrecursorData.cxx:44-45 (sequential sum)
                            bt += b
                        self.beta_total = bt
                    else:
                        raise ValueError(f"unrecognized keyword {l2[0]}")
            elif key == "thermal-properties":
                pass
            elif key == "fuel":
                self.fuel = bool(int(line[1]))
            elif key == "bc":
                self.bc = bool(int(line[1]))
            elif key == "split":
                self.split = bool(int(line[1]))
            else:
                raise ValueError(f"unrecognized keyword '{key}'")
        if self.has_nd and isinstance(nd, list):
            self.sets = []
            for one in nd:          # FeedbackNuclearData::check(beta_total)
                sub = Material(name=self.name, beta_total=self.beta_total, G=self.G)
                sub._check(one)
                self.sets.append(sub)
            self._copy_from(self.sets[0])
        elif self.has_nd:
            self._check(nd)

    def _read_nd(self, tok: Tokens) -> dict:
        nd = {}
        G = -1
        while True:
            line = tok.next_line()
            if not line or line[0] == "}":
                break
            k = line[0]
            if k == "energy-groups":
                G = int(line[1])
            elif k == "sigma-scattering":
                nd[k] = np.array(tok.read_rows(G, G), dtype=np.float64)
            elif k in ("sigma-total", "nu-sigma-fission", "kappa-sigma-fission", "sigma-transport",
                       "diffusion-coefficient", "fission-spectrum", "fission-spectrum-prompt",
                       "fission-spectrum-delayed", "neutron-velocity"):
                if k == "fission-spectrum":
                    k = "fission-spectrum-prompt"
                nd[k] = np.array(tok.read_values(G), dtype=np.float64)
            else:
                raise ValueError(f"unrecognized keyword '{k}'")
        self.G = G
        return nd

    def _check(self, nd: dict):
        """ConstantNuclearData::check(beta_total), ConstantNuclearData.cxx:129-177."""
        G = self.G
        nsf = nd.get("nu-sigma-fission")
        chi_p = nd.get("fission-spectrum-prompt")
        if nsf is not None or chi_p is not None:
            if nsf is None or chi_p is None:
                raise ValueError("fissile material needs nu-fission and fission spectrum")
        if nsf is None:
            nsf = np.zeros(G)
        ksf = nd.get("kappa-sigma-fission")
        if ksf is None:
            f = KAPPA_DEFAULT / NU_DEFAULT
            ksf = nsf * f
        if chi_p is None:
            chi_p = np.zeros(G)
        chi_d = nd.get("fission-spectrum-delayed", chi_p)
        bt = self.beta_total
        if bt > 0.0:
            chi = (1.0 - bt) * chi_p + bt * chi_d
        else:
            chi = chi_p.copy()
        D = nd.get("diffusion-coefficient")
        if "sigma-transport" in nd:
            if D is not None:
                raise ValueError("transport XS only without diffusion coefficients")
            D = 1.0 / (3.0 * nd["sigma-transport"])
        self.st = nd.get("sigma-total")
        self.nsf, self.ksf, self.chi, self.D = nsf, ksf, chi, D
        self.ss = nd.get("sigma-scattering")
        self.chi_p, self.chi_d = chi_p, chi_d
        self.vel = nd.get("neutron-velocity")

    _FIELDS = ("st", "nsf", "ksf", "ss", "D", "chi", "chi_p", "chi_d", "vel")

    def _copy_from(self, other: "Material"):
        for f in self._FIELDS:
            setattr(self, f, getattr(other, f))

    def at(self, T: float) -> "Material":
        """The material's data at temperature T (FeedbackNuclearData::interpolate and
        its getters, FeedbackNuclearData.hxx:60-140): below the first reference
        temperature the first set, above the last the last, else linear between the two
        sets around T.  The reference reads the set before the first when T equals the
        first reference value; the first set is used there."""
        if not self.sets:
            return self
        tref = self.tref
        if T < tref[0]:
            i1 = i2 = 0
            f = 0.0
        elif T > tref[-1]:
            i1 = i2 = len(tref) - 1
            f = 0.0
        else:
            i2 = int(np.searchsorted(tref, T, side="left"))
            if i2 == 0:
                i1, f = 0, 0.0
            else:
                i1 = i2 - 1
                f = (T - tref[i1]) / (tref[i2] - tref[i1])
        a, b = self.sets[i1], self.sets[i2]
        out = Material(name=self.name, G=self.G, has_nd=True, beta_total=self.beta_total, lam=self.lam,
                       beta=self.beta)
        for fld in self._FIELDS:
            x, y = getattr(a, fld), getattr(b, fld)
            setattr(out, fld, None if x is None else (1.0 - f) * x + f * y)
        return out

    def check_for_solver(self, G: int, diffusion: bool):
        if not self.has_nd:
            raise ValueError("missing nuclear data")
        if self.G != G:
            raise ValueError("wrong number of energy groups")
        if self.st is None or self.ss is None:
            raise ValueError("missing cross sections")
        if diffusion and self.D is None:
            raise ValueError("missing diffusion coefficients")


# --------------------------------------------------------------------------------------
# Mesh
# --------------------------------------------------------------------------------------


@dataclass
class Mesh:
    num_dims: int = 0
    volumes: np.ndarray = None       # (n,)
    centroids: np.ndarray = None     # (n, 3)
    materials: np.ndarray = None     # (n,) 0-based material index
    num_faces: np.ndarray = None     # (n,)
    areas: np.ndarray = None         # (n, F)
    fcent: np.ndarray = None         # (n, F, 3)
    normals: np.ndarray = None       # (n, F, 3)
    neighbors: np.ndarray = None     # (n, F): >=0 cell, <0 -(boundary index)-1, pad = huge
    boundaries: list = field(default_factory=list)
    bcs: dict = field(default_factory=dict)   # 1-based boundary index -> BoundaryCondition
    has_bcs: bool = False

    @property
    def n(self) -> int:
        return len(self.volumes)

    @property
    def F(self) -> int:
        return self.areas.shape[1]


PAD = np.iinfo(np.int64).max // 4


def read_cartesian(path: str) -> tuple[Mesh, dict]:
    """CartesianMesh::read (CartesianMesh.cxx:4-143)."""
    tok = Tokens(path)
    st = dict(nx=0, ny=0, nz=0, dx=[], dy=[], dz=[], num_dims=0, boundaries=[], bcs={},
              has_bcs=False, mats=None)
    while True:
        line = tok.next_line()
        if not line:
            break
        k = line[0]
        if k in ("dx", "dy", "dz"):
            n = int(line[1])
            if n > 0:
                d = tok.read_values(n)
            else:
                d = tok.read_values(1) * (-n)
                n = -n
            ax = k[1]
            st["n" + ax] = n
            st[k] = d
            if k == "dx" or n > 1:
                st["num_dims"] += 1
            st["boundaries"] += ["-" + ax, "+" + ax]
        elif k == "bc":
            st["has_bcs"] = True
            ibc = st["boundaries"].index(line[1])
            st["bcs"][ibc + 1] = _read_bc(line, 2, tok)
        elif k == "materials":
            nx, ny, nz = st["nx"], max(st["ny"], 1), max(st["nz"], 1)
            st["mats"] = np.array(tok.read_values(nx * ny * nz, int), dtype=np.int64) - 1
        elif k == "nodal-indices":
            nx, ny, nz = st["nx"], max(st["ny"], 1), max(st["nz"], 1)
            tok.read_values(nx * ny * nz, int)
        else:
            raise ValueError(f"unrecognized keyword '{k}'")
    return _build_cartesian(st), st


def _build_cartesian(st: dict) -> Mesh:
    """CartesianMesh::build (CartesianMesh.cxx:146-414)."""
    nx, ny, nz = st["nx"], st["ny"], st["nz"]
    dx = np.array(st["dx"], dtype=np.float64)
    dy = np.array(st["dy"], dtype=np.float64) if ny > 0 else np.zeros(1)
    dz = np.array(st["dz"], dtype=np.float64) if nz > 0 else np.zeros(1)
    # The reference reads dy(0)/dz(0) of an empty array for missing axes; the same value enters
    # every cell and face centroid, so only differences matter and 0 is used here.
    def axis(d, n):
        c = np.zeros(n + 1)
        for i in range(n):
            c[i + 1] = c[i] + d[i]
        return c
    x = axis(dx, nx)
    y = axis(dy, ny)
    z = axis(dz, nz)
    NY, NZ = max(ny, 1), max(nz, 1)
    mats = st["mats"].reshape(NZ, NY, nx)
    phys = mats != -1
    for k in range(1, NZ):
        if np.any(phys[k] != phys[0]):
            raise ValueError("wrong material definition")
    cid = -np.ones((NZ, NY, nx), dtype=np.int64)
    cid[phys] = np.arange(int(phys.sum()))
    kk, jj, ii = np.nonzero(phys)
    n = len(ii)
    if ny > 0 and nz > 0:
        vol = dx[ii] * dy[jj] * dz[kk]
    elif ny > 0:
        vol = dx[ii] * dy[jj]
    else:
        vol = dx[ii].copy()
    cent = np.stack([x[ii] + 0.5 * dx[ii], y[jj] + 0.5 * dy[jj], z[kk] + 0.5 * dz[kk]], axis=1)
    B = st["boundaries"]
    dirs = ["-x", "+x"] + (["-y", "+y"] if ny > 0 else []) + (["-z", "+z"] if nz > 0 else [])
    bidx = {d: B.index(d) for d in dirs}
    F = 6 if nz > 0 else 4 if ny > 0 else 2
    areas = np.zeros((n, F))
    fc = np.zeros((n, F, 3))
    nrm = np.zeros((n, F, 3))
    nbr = np.zeros((n, F), dtype=np.int64)
    cx, cy, cz = cent[:, 0], cent[:, 1], cent[:, 2]

    def neighbor(di, dj, dk, name):
        i2, j2, k2 = ii + di, jj + dj, kk + dk
        out = np.full(n, -bidx[name] - 1, dtype=np.int64)
        ok = (i2 >= 0) & (i2 < nx) & (j2 >= 0) & (j2 < NY) & (k2 >= 0) & (k2 < NZ)
        c = np.full(n, -1, dtype=np.int64)
        c[ok] = cid[k2[ok], j2[ok], i2[ok]]
        out[c >= 0] = c[c >= 0]
        return out

    f = 0
    specs = []
    if ny > 0:
        specs.append(("-y", (0, -1, 0)))
    specs.append(("+x", (1, 0, 0)))
    if ny > 0:
        specs.append(("+y", (0, 1, 0)))
    specs.append(("-x", (-1, 0, 0)))
    if nz > 0:
        specs += [("-z", (0, 0, -1)), ("+z", (0, 0, 1))]
    for name, (di, dj, dk) in specs:
        ax = name[1]
        if ax == "x":
            areas[:, f] = (dy[jj] * dz[kk]) if nz > 0 else (dy[jj] if ny > 0 else 1.0)
            fc[:, f] = np.stack([x[ii] + (dx[ii] if di > 0 else 0.0), cy, cz], axis=1)
        elif ax == "y":
            areas[:, f] = (dx[ii] * dz[kk]) if nz > 0 else dx[ii]
            fc[:, f] = np.stack([cx, y[jj] + (dy[jj] if dj > 0 else 0.0), cz], axis=1)
        else:
            areas[:, f] = dx[ii] * dy[jj]
            fc[:, f] = np.stack([cx, cy, z[kk] + (dz[kk] if dk > 0 else 0.0)], axis=1)
        nrm[:, f] = np.array([di, dj, dk], dtype=np.float64)
        nbr[:, f] = neighbor(di, dj, dk, name)
        f += 1
    m = Mesh(num_dims=st["num_dims"], volumes=vol, centroids=cent, materials=mats[phys].copy(),
             num_faces=np.full(n, F, dtype=np.int64), areas=areas, fcent=fc, normals=nrm,
             neighbors=nbr, boundaries=list(B), bcs=dict(st["bcs"]), has_bcs=st["has_bcs"])
    return m


def read_unstructured(path: str) -> Mesh:
    """UnstructuredExtrudedMesh::read/build (UnstructuredExtrudedMesh.cxx:4-364)."""
    tok = Tokens(path)
    pts = None
    cells = None
    nz = 0
    dz = []
    num_dims = 0
    boundaries: list[str] = []
    xy_bnames: list[str] = []
    xy_bpoints: list[list[int]] = []
    default_b = -1
    bcs = {}
    has_bcs = False
    mats = None
    while True:
        line = tok.next_line()
        if not line:
            break
        k = line[0]
        if k == "points":
            npnt = int(line[1])
            pts = np.array(tok.read_rows(npnt, 2), dtype=np.float64)
        elif k == "cells":
            ncell = int(line[1])
            cells = tok.read_rows(ncell, None, int)
            num_dims += 2
        elif k == "dz":
            n = int(line[1])
            if n > 0:
                dz = tok.read_values(n)
            else:
                dz = tok.read_values(1) * (-n)
                n = -n
            nz = n
            if nz > 1:
                num_dims += 1
            boundaries += ["-z", "+z"]
        elif k == "boundary":
            name = line[1]
            boundaries.append(name)
            xy_bnames.append(name)
            nb = int(line[2])
            if nb > 0:
                xy_bpoints.append(tok.read_values(nb, int))
            else:
                default_b = len(xy_bpoints)
                xy_bpoints.append([])
        elif k == "bc":
            has_bcs = True
            ibc = boundaries.index(line[1])
            bcs[ibc + 1] = _read_bc(line, 2, tok)
        elif k == "materials":
            nxy = len(cells)
            mats = np.array(tok.read_values(nxy * max(nz, 1), int), dtype=np.int64) - 1
        elif k == "nodal-indices":
            tok.read_values(len(cells) * max(nz, 1), int)
        else:
            raise ValueError(f"unrecognized keyword '{k}'")

    nxy = len(cells)
    npnt = len(pts)
    dz = np.array(dz, dtype=np.float64) if nz > 0 else np.zeros(1)
    zc = np.zeros(nz + 1)
    for kk in range(nz):
        zc[kk + 1] = zc[kk] + dz[kk]

    def area(ids):
        a = 0.0
        nn = len(ids)
        for q in range(nn):
            p1, p2 = pts[ids[q]], pts[ids[(q + 1) % nn]]
            a += p1[0] * p2[1] - p2[0] * p1[1]
        return a * 0.5

    def centroid(ids, a):
        c0 = c1 = 0.0
        nn = len(ids)
        for q in range(nn):
            p1, p2 = pts[ids[q]], pts[ids[(q + 1) % nn]]
            da = p1[0] * p2[1] - p2[0] * p1[1]
            c0 += (p1[0] + p2[0]) * da
            c1 += (p1[1] + p2[1]) * da
        s = 1.0 / (6.0 * a)
        return c0 * s, c1 * s

    xy_area = np.array([area(c) for c in cells])
    xy_cent = np.array([centroid(c, a) for c, a in zip(cells, xy_area)])

    # point -> (cells, then boundaries), UnstructuredExtrudedMesh.cxx:227-251
    pcells: list[list[int]] = [[] for _ in range(npnt)]
    for i, c in enumerate(cells):
        for p in c:
            pcells[p].append(i)
    for b, name in enumerate(xy_bnames):
        bi = boundaries.index(name)
        for p in xy_bpoints[b]:
            pcells[p].append(-bi - 1)
    xy_nbr = []
    for i, c in enumerate(cells):
        nn = len(c)
        row = []
        for f in range(nn):
            ip1, ip2 = c[f], c[(f + 1) % nn]
            found = None
            s2 = pcells[ip2]
            for i1 in pcells[ip1]:
                for i2 in s2:
                    if i1 == i2 and i1 != i:
                        if found is not None and found > 0:
                            raise ValueError("wrong mesh connectivity")
                        found = i1
            if found is None and default_b >= 0:
                found = -default_b - 1
            if found is None:
                raise ValueError("wrong mesh connectivity")
            row.append(found)
        xy_nbr.append(row)

    NZ = max(nz, 1)
    n = nxy * NZ
    nfxy = np.array([len(c) for c in cells])
    F = int(nfxy.max()) + (2 if nz > 0 else 0)
    vol = np.zeros(n)
    cent = np.zeros((n, 3))
    nf = np.zeros(n, dtype=np.int64)
    areas = np.zeros((n, F))
    fc = np.zeros((n, F, 3))
    nrm = np.zeros((n, F, 3))
    nbr = np.full((n, F), PAD, dtype=np.int64)
    bz = [boundaries.index("-z"), boundaries.index("+z")] if nz > 0 else []
    ic = 0
    for kk in range(NZ):
        zmid = zc[kk] + 0.5 * dz[kk] if nz > 0 else 0.0
        for i, c in enumerate(cells):
            nn = len(c)
            a = xy_area[i]
            vol[ic] = a * dz[kk] if nz > 0 else a
            cent[ic] = (xy_cent[i][0], xy_cent[i][1], zmid)
            nf[ic] = nn + 2 if nz > 0 else nn
            for f in range(nn):
                p1, p2 = pts[c[f]], pts[c[(f + 1) % nn]]
                d = math.sqrt((p2[0] - p1[0]) ** 2 + (p2[1] - p1[1]) ** 2)
                areas[ic, f] = d * dz[kk] if nz > 0 else d
                fc[ic, f] = (0.5 * (p1[0] + p2[0]), 0.5 * (p1[1] + p2[1]), zmid)
                nx_, ny_ = p2[1] - p1[1], p1[0] - p2[0]
                nr = math.sqrt(nx_ * nx_ + ny_ * ny_)
                nrm[ic, f] = (nx_ / nr, ny_ / nr, 0.0)
                j = xy_nbr[i][f]
                nbr[ic, f] = j + kk * nxy if j >= 0 else j
            if nz > 0:
                f = nn
                areas[ic, f] = a
                fc[ic, f] = (xy_cent[i][0], xy_cent[i][1], zc[kk])
                nrm[ic, f] = (0.0, 0.0, -1.0)
                nbr[ic, f] = -bz[0] - 1 if kk == 0 else ic - nxy
                f += 1
                areas[ic, f] = a
                fc[ic, f] = (xy_cent[i][0], xy_cent[i][1], zc[kk] + dz[kk])
                nrm[ic, f] = (0.0, 0.0, 1.0)
                nbr[ic, f] = -bz[1] - 1 if kk == nz - 1 else ic + nxy
            ic += 1
    return Mesh(num_dims=num_dims, volumes=vol, centroids=cent, materials=mats, num_faces=nf,
                areas=areas, fcent=fc, normals=nrm, neighbors=nbr, boundaries=boundaries,
                bcs=bcs, has_bcs=has_bcs)


def split_materials(mesh: Mesh, materials: list[Material]):
    """Mesh::splitMaterials (Mesh.cxx:24-60): connected regions of split materials."""
    for i in range(mesh.n):
        im = int(mesh.materials[i])
        mat = materials[im]
        if mat.split:
            new = len(materials)
            stack = [i]
            mesh.materials[i] = new
            while stack:
                c = stack.pop()
                for f in range(mesh.num_faces[c]):
                    c2 = int(mesh.neighbors[c, f])
                    if 0 <= c2 < PAD and mesh.materials[c2] == im:
                        mesh.materials[c2] = new
                        stack.append(c2)
            nsub = getattr(mat, "_nsub", 0)
            name = f"{mat.name}-{nsub}"
            mat._nsub = nsub + 1
            sub = Material(**{k: getattr(mat, k) for k in mat.__dataclass_fields__})
            sub.name = name
            sub.split = False
            if mat.bc:
                mesh.boundaries.append(name)
            materials.append(sub)


def remove_bc_materials(mesh: Mesh, materials: list[Material]) -> Mesh:
    """Mesh::removeBCMaterials (Mesh.cxx:63-204)."""
    isbc = np.array([materials[m].bc for m in mesh.materials])
    keep = ~isbc
    newid = -np.ones(mesh.n, dtype=np.int64)
    newid[keep] = np.arange(int(keep.sum()))
    matb = {i: mesh.boundaries.index(m.name) for i, m in enumerate(materials) if m.bc}
    nbr = mesh.neighbors[keep].copy()
    valid = (nbr >= 0) & (nbr < PAD)
    for (r, f) in zip(*np.nonzero(valid)):
        c2 = int(nbr[r, f])
        if isbc[c2]:
            nbr[r, f] = -matb[int(mesh.materials[c2])] - 1
        else:
            nbr[r, f] = newid[c2]
    nf = mesh.num_faces[keep]
    F = int(nf.max())
    return Mesh(num_dims=mesh.num_dims, volumes=mesh.volumes[keep], centroids=mesh.centroids[keep],
                materials=mesh.materials[keep], num_faces=nf, areas=mesh.areas[keep][:, :F],
                fcent=mesh.fcent[keep][:, :F], normals=mesh.normals[keep][:, :F],
                neighbors=nbr[:, :F], boundaries=list(mesh.boundaries), bcs=dict(mesh.bcs),
                has_bcs=mesh.has_bcs)


# --------------------------------------------------------------------------------------
# Problem (Parser.cxx:4-260)
# --------------------------------------------------------------------------------------


@dataclass
class Problem:
    mesh: Mesh
    materials: list
    solver: str            # "diffusion" | "sn"
    G: int
    power: float = 1.0
    bcs: dict = field(default_factory=dict)
    has_bcs: bool = False
    order: int = -1
    delta: float = 0.1
    ls: bool = False
    dt: list = field(default_factory=list)
    T: np.ndarray | None = None   # the "temperature" field per cell (zero when not set)

    def boundary_conditions(self) -> dict:
        # DiffusionSolver.cxx:91 / SNSolver.cxx:346: solver BCs if any were given, else mesh BCs
        return self.bcs if self.has_bcs else self.mesh.bcs


def read_problem(path: str) -> Problem:
    base = os.path.dirname(os.path.abspath(path))
    state = dict(mesh=None, materials=[], solvers=[], dt=[], ready=False)
    _parse(path, base, state)
    if len(state["solvers"]) != 1:
        raise ValueError("exactly one neutronic solver block expected")
    s = state["solvers"][0]
    s.mesh = state["mesh"]
    s.dt = state["dt"]
    return s


def _parse(path: str, base: str, state: dict):
    tok = Tokens(path)
    while True:
        line = tok.next_line()
        if not line:
            break
        k = line[0]
        if k == "mesh":
            p = _resolve(line[2], base)
            if line[1] == "cartesian":
                state["mesh"], _ = read_cartesian(p)
            elif line[1] == "unstructured":
                state["mesh"] = read_unstructured(p)
            else:
                raise ValueError("mesh type outside the k-eigen path")
        elif k == "material":
            mat = Material(line[1])
            if line[2] == "{":
                mat.read(tok)
            else:
                mat.read(Tokens(_resolve(line[2], base)))
            if mat.bc:
                state["mesh"].boundaries.append(mat.name)
            state["materials"].append(mat)
        elif k == "solver":
            if not state["ready"]:
                mats = state["materials"]
                if any(m.split for m in mats):
                    split_materials(state["mesh"], mats)
                if any(m.bc for m in mats):
                    state["mesh"] = remove_bc_materials(state["mesh"], mats)
                state["ready"] = True
            kind = line[1]
            if kind not in ("diffusion", "sn"):
                raise ValueError("solver outside the k-eigen path")
            prob = Problem(mesh=None, materials=state["materials"], solver=kind, G=-1)
            if line[2] == "{":
                _read_solver(prob, tok, state["mesh"])
            else:
                _read_solver(prob, Tokens(_resolve(line[2], base)), state["mesh"])
            state["solvers"].append(prob)
        elif k == "dt":
            n = int(line[1])
            state["dt"] = tok.read_values(n) if n > 0 else tok.read_values(1) * (-n)
        elif k in ("vtk", "petsc"):
            pass
        elif k == "include":
            _parse(_resolve(line[1], base), base, state)
        else:
            raise ValueError(f"unrecognized keyword '{k}'")


def _read_solver(prob: Problem, tok: Tokens, mesh: Mesh):
    """DiffusionSolver::read (DiffusionSolver.cxx:4-85), SNSolver::read (SNSolver.cxx:8-124)."""
    while True:
        line = tok.next_line()
        if not line or line[0] == "}":
            break
        k = line[0]
        if k == "energy-groups":
            prob.G = int(line[1])
        elif k == "bc":
            prob.has_bcs = True
            ibc = mesh.boundaries.index(line[1])
            prob.bcs[ibc + 1] = _read_bc(line, 2, tok)
        elif k == "power":
            prob.power = float(line[1])
        elif k == "convergence":
            pass
        elif k == "order" and prob.solver == "sn":
            prob.order = int(line[1])
        elif k == "mixed-face-interpolation" and prob.solver == "sn":
            prob.delta = float(line[1])
        elif k == "least-squares-boundary-interpolation" and prob.solver == "sn":
            prob.ls = bool(int(line[1]))
        else:
            raise ValueError(f"unrecognized keyword '{k}'")


# --------------------------------------------------------------------------------------
# Helpers (math.cxx:150-161)
# --------------------------------------------------------------------------------------


def surface_leakage_factor(p1: np.ndarray, p2: np.ndarray, n: np.ndarray) -> np.ndarray:
    dp = p2 - p1
    num = dp[..., 0] * n[..., 0] + dp[..., 1] * n[..., 1] + dp[..., 2] * n[..., 2]
    den = dp[..., 0] * dp[..., 0] + dp[..., 1] * dp[..., 1] + dp[..., 2] * dp[..., 2]
    return num / den


def _material_tables(prob: Problem):
    """Per-material tables (constant data; a feedback material contributes its first set)."""
    return _tables_of(prob.materials, prob.G)


def _cell_materials(prob: Problem):
    """The data every cell sees: its material at the cell's temperature when the material
    has feedback data.  Returns (materials, index per cell); without feedback data the
    problem's materials and the mesh's material indices."""
    mats = prob.materials
    if not any(m.sets for m in mats):
        return mats, prob.mesh.materials
    T = prob.T if prob.T is not None else np.zeros(prob.mesh.n)
    eff, index, cell = [], {}, np.zeros(prob.mesh.n, dtype=np.int64)
    for i, m in enumerate(prob.mesh.materials):
        t = float(T[i]) if mats[m].sets else 0.0
        key = (int(m), t)
        if key not in index:
            index[key] = len(eff)
            eff.append(mats[m].at(t))
        cell[i] = index[key]
    return eff, cell


def _tables_of(mats: list, G: int):
    st = np.array([m.st for m in mats])
    nsf = np.array([m.nsf for m in mats])
    ksf = np.array([m.ksf for m in mats])
    chi = np.array([m.chi for m in mats])
    ss = np.array([m.ss for m in mats])
    D = np.array([m.D if m.D is not None else np.zeros(G) for m in mats])
    return st, nsf, ksf, chi, ss, D


# --------------------------------------------------------------------------------------
# Diffusion assembly (DiffusionSolver.cxx:88-320, n = 0)
# --------------------------------------------------------------------------------------


def assemble_diffusion(prob: Problem):
    mesh = prob.mesh
    G = prob.G
    for m in prob.materials:
        m.check_for_solver(G, True)
    eff, mat = _cell_materials(prob)
    st, nsf, ksf, chi, ss, D = _tables_of(eff, G)
    orig = mesh.materials
    Tc = prob.T if prob.T is not None else np.zeros(mesh.n)
    bcs = prob.boundary_conditions()
    n = mesh.n
    V = mesh.volumes
    rows, cols, vals = [], [], []
    frows, fcols, fvals = [], [], []
    diag = np.zeros((n, G))
    cell = np.arange(n)
    for g in range(G):
        diag[:, g] = st[mat, g] * V
        for g2 in range(G):
            term = -ss[mat, g2, g] * V
            if g2 == g:
                diag[:, g] += term
            else:
                rows.append(cell * G + g)
                cols.append(cell * G + g2)
                vals.append(term)
            frows.append(cell * G + g)
            fcols.append(cell * G + g2)
            fvals.append(chi[mat, g] * nsf[mat, g2] * V)
    # faces, in face order so the diagonal accumulates in the reference's order
    for f in range(mesh.F):
        has = f < mesh.num_faces
        nb = mesh.neighbors[:, f]
        A = mesh.areas[:, f]
        for g in range(G):
            Dg = D[mat, g]
            # boundaries
            bmask = has & (nb < 0)
            if bmask.any():
                for c in np.nonzero(bmask)[0]:
                    bc = bcs.get(int(-nb[c]), BoundaryCondition())
                    if bc.type == BC_VACUUM:
                        w = surface_leakage_factor(mesh.centroids[c], mesh.fcent[c, f], mesh.normals[c, f])
                        diag[c, g] += w * Dg[c] * A[c]
                    elif bc.type == BC_REFLECTIVE:
                        pass
                    elif bc.type == BC_ROBIN:
                        diag[c, g] -= bc.values[0] * A[c]
                    else:
                        raise ValueError("boundary condition not implemented")
            imask = has & (nb >= 0) & (nb < PAD)
            c = np.nonzero(imask)[0]
            if len(c) == 0:
                continue
            c2 = nb[c]
            same = orig[c2] == orig[c]
            r = np.empty(len(c))
            cs = c[same]
            w = surface_leakage_factor(mesh.centroids[cs], mesh.centroids[c2[same]], mesh.normals[cs, f])
            r[same] = -w * Dg[cs] * A[cs]
            cd = c[~same]
            cd2 = c2[~same]
            w1 = surface_leakage_factor(mesh.centroids[cd], mesh.fcent[cd, f], mesh.normals[cd, f])
            w1 = w1 * (Dg[cd] * A[cd])
            w2 = surface_leakage_factor(mesh.centroids[cd2], mesh.fcent[cd, f], mesh.normals[cd, f])
            # the neighbour's coefficient at this cell's temperature (DiffusionSolver.cxx:270-273)
            Dn = np.array([prob.materials[orig[b]].at(float(Tc[a])).D[g] if prob.materials[orig[b]].sets
                           else prob.materials[orig[b]].D[g] for a, b in zip(cd, cd2)])
            w2 = w2 * (-Dn * A[cd])
            r[~same] = -(w1 * w2) / (w1 + w2)
            diag[c, g] -= r
            rows.append(c * G + g)
            cols.append(c2 * G + g)
            vals.append(r)
    N = n * G
    rows.append(np.arange(N))
    cols.append(np.arange(N))
    vals.append(diag.reshape(-1))
    R = sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(N, N))
    Fm = sp.csr_matrix((np.concatenate(fvals), (np.concatenate(frows), np.concatenate(fcols))), shape=(N, N))
    return R, Fm


# --------------------------------------------------------------------------------------
# SN quadrature (AngularQuadratureSet.cxx:4-209)
# --------------------------------------------------------------------------------------


def quadrature(order: int):
    M = order * (order + 2)
    d = np.zeros((M, 3))
    w = np.zeros(M)
    if order == 2:
        d[0] = [1.0 / math.sqrt(3.0)] * 3
        w[0] = 1.0 / 8.0
    elif order == 4:
        mu = [0.3500212, 0.8688903]
        d[0:3] = [[mu[0], mu[0], mu[1]], [mu[0], mu[1], mu[0]], [mu[1], mu[0], mu[0]]]
        w[0:3] = (1.0 / 3.0) / 8.0
    elif order == 6:
        mu = [0.2666355, 0.6815076, 0.9261808]
        ww = [0.1761263, 0.1572071]
        d[0:6] = [[mu[0], mu[0], mu[2]], [mu[0], mu[2], mu[0]], [mu[2], mu[0], mu[0]],
                  [mu[0], mu[1], mu[1]], [mu[1], mu[0], mu[1]], [mu[1], mu[1], mu[0]]]
        w[0:3] = ww[0] / 8.0
        w[3:6] = ww[1] / 8.0
    elif order == 8:
        mu = [0.2182179, 0.5773503, 0.7867958, 0.9511897]
        ww = [0.1209877, 0.0907407, 0.0925926]
        d[0:10] = [[mu[0], mu[0], mu[3]], [mu[0], mu[3], mu[0]], [mu[3], mu[0], mu[0]],
                   [mu[0], mu[1], mu[2]], [mu[0], mu[2], mu[1]], [mu[1], mu[0], mu[2]],
                   [mu[1], mu[2], mu[0]], [mu[2], mu[0], mu[1]], [mu[2], mu[1], mu[0]],
                   [mu[1], mu[1], mu[1]]]
        w[0:3] = ww[0] / 8.0
        w[3:9] = ww[1] / 8.0
        w[9] = ww[2] / 8.0
    else:
        raise ValueError("SN order not implemented")
    m8 = M // 8
    for o in range(1, 8):
        for m in range(m8):
            l = o * m8 + m
            d[l, 0] = -d[m, 0] if (o & 1) else d[m, 0]
            d[l, 1] = -d[m, 1] if (o & 2) else d[m, 1]
            d[l, 2] = -d[m, 2] if (o & 4) else d[m, 2]
            w[l] = w[m]
    axes = np.eye(3)
    refl = -np.ones((M, 3), dtype=np.int64)
    for a in range(3):
        for m in range(M):
            av = -2.0 * float(d[m] @ axes[a])
            r = av * axes[a] + d[m]
            for m2 in range(M):
                if float(d[m2] @ r) > 1.0 - 1e-6:
                    if refl[m, a] != -1:
                        raise ValueError("multiple reflected directions found")
                    refl[m, a] = m2
            if refl[m, a] == -1:
                raise ValueError("reflected direction not found")
    return d, w, refl


# --------------------------------------------------------------------------------------
# SN gradient schemes (SNSolver.cxx:127-269)
# --------------------------------------------------------------------------------------


def boundary_cells(mesh: Mesh) -> np.ndarray:
    nb = mesh.neighbors
    has = np.arange(mesh.F)[None, :] < mesh.num_faces[:, None]
    isb = np.any(has & (nb < 0), axis=1)
    ic = -np.ones(mesh.n, dtype=np.int64)
    ic[isb] = np.arange(int(isb.sum()))
    return ic


def gauss_coefs(mesh: Mesh, delta: float) -> np.ndarray:
    """coefs(i, f, 0..3) of SNSolver::buildGaussGradientScheme for interior faces."""
    nb = mesh.neighbors
    c = np.zeros((mesh.n, mesh.F, 4))
    for f in range(mesh.F):
        ok = (f < mesh.num_faces) & (nb[:, f] >= 0) & (nb[:, f] < PAD)
        i = np.nonzero(ok)[0]
        i2 = nb[i, f]
        fcnt = mesh.fcent[i, f]
        r_if = np.sqrt(np.sum((mesh.centroids[i] - fcnt) ** 2, axis=1))
        r_i2f = np.sqrt(np.sum((mesh.centroids[i2] - fcnt) ** 2, axis=1))
        r_ii2 = np.sqrt(np.sum((mesh.centroids[i2] - mesh.centroids[i]) ** 2, axis=1))
        c[i, f, 0] = (r_i2f + delta * r_if) / r_ii2
        c[i, f, 1] = (1.0 - delta) * r_if / r_ii2
        c[i, f, 2] = (1.0 - delta) * r_i2f / r_ii2
        c[i, f, 3] = (r_if + delta * r_i2f) / r_ii2
    return c


# Starting values of the LS Gram matrix G.  The reference declares `Eigen::MatrixXd
# G(num_dims, num_dims)` per boundary cell and accumulates into it without initialising it
# (SNSolver.cxx:247-252).  "zero" is its evident intent and what the product implements.
# The "heap-*" models restate what glibc's allocator leaves there when G's chunk is freed
# at the end of one boundary cell and handed back, last-in first-out, to the next: G(0,0)
# holds the free-list pointer (a denormal, taken as 0) and G(0,1), G(1,1) the previous
# cell's final values; "heap-key-kept" also carries G(1,0), which glibc before 2.29 (no
# tcache key) leaves untouched (32-byte-aligned Eigen allocations carry G(0,0) as well,
# which moves keff by 4e-8 more), "heap-key-cleared" sets it to 0 as glibc 2.29+ does
# when it hands a chunk out.  The first boundary cell
# starts from zero in both: what its chunk held before is not determined by the input.
LS_GRAM_START = "zero"


def ls_coefs(mesh: Mesh, ic_to_ibc: np.ndarray) -> np.ndarray:
    """SNSolver::buildLSGradientScheme for boundary cells (SNSolver.cxx:211-269).

    Reproduces the reference exactly: d is a (faces x dims) row-major array, and d(jg, f)
    reads its flat element jg*dims + f; G starts from LS_GRAM_START (zero by default).
    """
    nd = mesh.num_dims
    nbc = int((ic_to_ibc >= 0).sum())
    coefs = np.zeros((nbc, mesh.F, 3))
    carry = LS_GRAM_START != "zero" and nd == 2
    prev = np.zeros((nd, nd))
    for i in np.nonzero(ic_to_ibc >= 0)[0]:
        ic = ic_to_ibc[i]
        nf = int(mesh.num_faces[i])
        ci = mesh.centroids[i]
        d = np.zeros((nf, nd))
        for f in range(nf):
            i2 = int(mesh.neighbors[i, f])
            c2 = mesh.fcent[i, f] if i2 < 0 else mesh.centroids[i2]
            for a in range(nd):
                d[f, a] = c2[a] - ci[a]
        flat = d.reshape(-1)
        Gm = np.zeros((nd, nd))
        if carry:
            Gm[0, 1], Gm[1, 1] = prev[0, 1], prev[1, 1]
            if LS_GRAM_START == "heap-key-kept":
                Gm[1, 0] = prev[1, 0]
        for jg in range(nd):
            for ig in range(nd):
                for f in range(nf):
                    Gm[jg, ig] += flat[jg * nd + f] * d[f, ig]
        prev = Gm.copy()
        Ginv = np.linalg.inv(Gm)
        for f in range(nf):
            for a in range(nd):
                for b in range(nd):
                    coefs[ic, f, a] += Ginv[a, b] * flat[b * nd + f]
    return coefs


# --------------------------------------------------------------------------------------
# SN assembly (SNSolver.cxx:344-631, n = 0)
# --------------------------------------------------------------------------------------


def assemble_sn(prob: Problem):
    mesh = prob.mesh
    G = prob.G
    for m in prob.materials:
        m.check_for_solver(G, False)
    eff, mat_c = _cell_materials(prob)
    st, nsf, ksf, chi, ss, D = _tables_of(eff, G)
    dirs, w, refl = quadrature(prob.order)
    M = len(w)
    bcs = prob.boundary_conditions()
    n = mesh.n
    mat = mat_c
    V = mesh.volumes
    gc = gauss_coefs(mesh, prob.delta)
    ic_to_ibc = boundary_cells(mesh)
    lsc = ls_coefs(mesh, ic_to_ibc) if prob.ls else None
    GM = G * M
    N = n * GM
    cell = np.arange(n)
    rows, cols, vals = [], [], []
    frows, fcols, fvals = [], [], []
    # in-cell scattering (all (g2, m2), including the diagonal) and collision
    for g in range(G):
        for m in range(M):
            l = cell * GM + g * M + m
            rows.append(l)
            cols.append(l)
            vals.append(st[mat, g] * V)
            for g2 in range(G):
                for m2 in range(M):
                    l2 = cell * GM + g2 * M + m2
                    rows.append(l)
                    cols.append(l2)
                    vals.append(-ss[mat, g2, g] * w[m2] * V)
                    frows.append(l)
                    fcols.append(l2)
                    fvals.append(chi[mat, g] * nsf[mat, g2] * w[m2] * V)
    nb = mesh.neighbors
    for f in range(mesh.F):
        has = f < mesh.num_faces
        A = mesh.areas[:, f]
        mu = mesh.normals[:, f] @ dirs.T          # (n, M)
        inter = has & (nb[:, f] >= 0) & (nb[:, f] < PAD)
        ci = np.nonzero(inter)[0]
        c2 = nb[ci, f]
        for m in range(M):
            wm = mu[ci, m]
            out = wm > 0.0
            w_i = np.where(out, gc[ci, f, 0], gc[ci, f, 2])
            w_i2 = np.where(out, gc[ci, f, 1], gc[ci, f, 3])
            for g in range(G):
                l = ci * GM + g * M + m
                rows.append(l)
                cols.append(l)
                vals.append(w_i * wm * A[ci])
                rows.append(l)
                cols.append(c2 * GM + g * M + m)
                vals.append(w_i2 * wm * A[ci])
        bmask = has & (nb[:, f] < 0)
        for c in np.nonzero(bmask)[0]:
            bc = bcs.get(int(-nb[c, f]), BoundaryCondition())
            Af = A[c]
            for m in range(M):
                wm = mu[c, m]
                if bc.type == BC_VACUUM:
                    if wm > 0.0:
                        for g in range(G):
                            l = c * GM + g * M + m
                            rows.append(l); cols.append(l); vals.append(wm * Af)
                        if prob.ls:
                            dp = mesh.fcent[c, f] - mesh.centroids[c]
                            ibc = ic_to_ibc[c]
                            for f2 in range(int(mesh.num_faces[c])):
                                i3 = int(nb[c, f2])
                                if i3 >= 0:
                                    w3 = dp[0] * lsc[ibc, f2, 0] + dp[1] * lsc[ibc, f2, 1] + dp[2] * lsc[ibc, f2, 2]
                                    for g in range(G):
                                        l = c * GM + g * M + m
                                        rows.append(l); cols.append(l); vals.append(-w3 * wm * Af)
                                        rows.append(l); cols.append(i3 * GM + g * M + m)
                                        vals.append(w3 * wm * Af)
                elif bc.type == BC_REFLECTIVE:
                    if wm > 0.0:
                        for g in range(G):
                            l = c * GM + g * M + m
                            rows.append(l); cols.append(l); vals.append(wm * Af)
                    else:
                        # SNSolver.cxx:539-543: the loop index shadows the cell, so the normal
                        # of face f of cells 0, 1 and 2 is tested against the x, y and z axes.
                        m2 = -1
                        for a in range(3):
                            dd = float(mesh.normals[a, f, a])
                            if abs(dd) > 1.0 - 1e-6:
                                m2 = int(refl[m, a])
                        if m2 == -1:
                            raise ValueError("reflected direction not found")
                        for g in range(G):
                            l = c * GM + g * M + m
                            rows.append(l); cols.append(c * GM + g * M + m2); vals.append(wm * Af)
                else:
                    raise ValueError("boundary condition not implemented")
    R = sp.csr_matrix((np.concatenate([np.atleast_1d(v) for v in vals]),
                       (np.concatenate([np.atleast_1d(v) for v in rows]),
                        np.concatenate([np.atleast_1d(v) for v in cols]))), shape=(N, N))
    Fm = sp.csr_matrix((np.concatenate(fvals), (np.concatenate(frows), np.concatenate(fcols))),
                       shape=(N, N))
    return R, Fm, w


# --------------------------------------------------------------------------------------
# Eigen-solve and post-processing
# --------------------------------------------------------------------------------------


def solve_eigen(R: sp.csr_matrix, Fm: sp.csr_matrix, tol: float = 1e-13):
    """Dominant k of R x = (1/k) F x: Arnoldi on R^-1 F with an LU of R (petsc.cxx:175-204)."""
    N = R.shape[0]
    lu = spla.splu(R.tocsc(), permc_spec="MMD_AT_PLUS_A")
    op = spla.LinearOperator((N, N), matvec=lambda v: lu.solve(Fm @ v), dtype=np.float64)
    v0 = np.ones(N)
    vals, vecs = spla.eigs(op, k=1, which="LM", v0=v0, tol=tol, maxiter=100000,
                           ncv=min(N - 1, 40))
    k = float(np.real(vals[0]))
    x = np.real(vecs[:, 0])
    return k, x


def _kappa_nu_tables(prob: Problem):
    eff, mat = _cell_materials(prob)
    st, nsf, ksf, chi, ss, D = _tables_of(eff, prob.G)
    return ksf[mat], nsf[mat]


def normalize_scalar_flux(prob: Problem, phi: np.ndarray) -> np.ndarray:
    """NeutronicSolver::normalizeScalarFlux (NeutronicSolver.cxx:46-78)."""
    ksf, _ = _kappa_nu_tables(prob)
    V = prob.mesh.volumes
    phi2 = phi.reshape(prob.mesh.n, prob.G)
    p0 = float(np.sum(phi2 * ksf * V[:, None]))
    out = phi * (prob.power / p0)
    if np.any(out < 0.0):
        raise ValueError("negative values in the scalar-flux solution")
    return out


def power_and_production(prob: Problem, phi: np.ndarray, keff: float):
    """NeutronicSolver::calculatePowerAndProductionRate (NeutronicSolver.cxx:81-116)."""
    ksf, nsf = _kappa_nu_tables(prob)
    V = prob.mesh.volumes
    phi2 = phi.reshape(prob.mesh.n, prob.G)
    q = np.sum(phi2 * ksf * V[:, None], axis=1)
    P = np.sum(phi2 * nsf * V[:, None] / keff, axis=1)
    return q, P, float(np.sum(q))


def solve_problem(prob: Problem, tol: float = 1e-13) -> dict:
    """Steady-state solve: keff, normalised fluxes, power and production-rate fields."""
    if prob.solver == "diffusion":
        R, Fm = assemble_diffusion(prob)
        k, x = solve_eigen(R, Fm, tol)
        phi = normalize_scalar_flux(prob, x)
        q, P, ptot = power_and_production(prob, phi, k)
        return dict(keff=k, phi=phi, q=q, P=P, power=ptot, R=R, F=Fm)
    R, Fm, w = assemble_sn(prob)
    k, x = solve_eigen(R, Fm, tol)
    n, G, M = prob.mesh.n, prob.G, len(w)
    psi = x.reshape(n, G, M)
    phi = 4.0 * math.pi * np.einsum("igm,m->ig", psi, w).reshape(-1)   # SNSolver.cxx:272-299
    phi = normalize_scalar_flux(prob, phi)
    ksf, _ = _kappa_nu_tables(prob)
    V = prob.mesh.volumes
    p0 = float(np.sum(np.einsum("igm,m->ig", psi, w) * ksf * V[:, None]))  # SNSolver.cxx:302-341
    psi_n = x * (prob.power / p0)
    if np.any(psi_n < 0.0):
        raise ValueError("negative values in the angular-flux solution")
    q, P, ptot = power_and_production(prob, phi, k)
    return dict(keff=k, phi=phi, psi=psi_n, q=q, P=P, power=ptot, R=R, F=Fm, weights=w)


def run_input(path: str, tol: float = 1e-13) -> dict:
    return solve_problem(read_problem(path), tol)


def diffusion_transient_system(prob: Problem, R0: sp.csr_matrix, dt: float, keff: float, phi0: np.ndarray,
                               S: np.ndarray):
    """R and b of DiffusionSolver::buildMatrices for a time step n > 0
    (DiffusionSolver.cxx:108-175): R = R(n=0) + V/(v_g dt) on the diagonal
    - (1 - beta) chi_p,g nu_sigma_f,g2 V / keff in the cell's (g, g2) block;
    b = chi_d,g S_i + V/(v_g dt) phi0.  R0 is the n = 0 operator of assemble_diffusion."""
    mesh, G = prob.mesh, prob.G
    n = mesh.n
    eff, mat = _cell_materials(prob)
    V = mesh.volumes
    for m in eff:
        if m.vel is None:
            raise ValueError("missing neutron velocities")
    vel = np.array([m.vel for m in eff])
    chip = np.array([(1.0 - m.beta_total) * m.chi_p for m in eff])
    chid = np.array([m.chi_d for m in eff])
    st, nsf, ksf, chi, ss, D = _tables_of(eff, G)
    d = (V[:, None] / (vel[mat] * dt)).reshape(-1)
    cell = np.arange(n)
    rows, cols, vals = [], [], []
    for g in range(G):
        for g2 in range(G):
            rows.append(cell * G + g)
            cols.append(cell * G + g2)
            vals.append(-chip[mat, g] * nsf[mat, g2] * V / keff)
    N = n * G
    Rp = sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(N, N))
    R = (R0 + sp.diags(d) + Rp).tocsr()
    b = (chid[mat] * S[:, None]).reshape(-1) + d * phi0
    return R, b


def run_transient(path: str, delayed_source_scale: float = 1.0, tol: float = 1e-13) -> list[dict]:
    """The C front end's time loop (c/main.c:16-29) for a diffusion input with time steps:
    the steady state, then every step of the input's dt list with a direct solve of the
    step's linear system (the reference solves it with KSP, petsc.cxx:147-172).  The
    delayed source S = beta P of calculatePowerAndProductionRate (NeutronicSolver.cxx:81-116)
    is scaled by delayed_source_scale after the steady state, as a coupled caller setting
    the "delayed-source" field would.  Returns per step keff (steady state), phi, q, P and the
    total power."""
    prob = read_problem(path)
    if prob.solver != "diffusion":
        raise ValueError("transients are restated for diffusion only")
    res = solve_problem(prob, tol)
    keff = res["keff"]
    ksf, nsf = _kappa_nu_tables(prob)
    V = prob.mesh.volumes
    beta = np.array([m.beta_total for m in prob.materials])[prob.mesh.materials]
    out = [dict(keff=keff, phi=res["phi"], q=res["q"], P=res["P"], power=res["power"])]
    phi = res["phi"]
    S = beta * res["P"] * delayed_source_scale
    t = 0.0
    for dt in prob.dt:
        t += dt
        R, b = diffusion_transient_system(prob, res["R"], dt, keff, phi, S)
        phi = spla.spsolve(R.tocsc(), b)
        ph2 = phi.reshape(prob.mesh.n, prob.G)
        q = np.sum(ph2 * ksf * V[:, None], axis=1)
        P = np.sum(ph2 * nsf * V[:, None] / keff, axis=1)
        S = beta * P
        out.append(dict(dt=dt, t=t, phi=phi, q=q, P=P, power=float(np.sum(q))))
    return out



def precursor_step(prob: Problem, npg: int, P: np.ndarray, C0: np.ndarray | None, dt: float):
    """PrecursorSolver::solve (PrecursorSolver.cxx:59-127): C = beta/lambda P (steady
    state, C0 None) or (C0 + dt beta P) / (1 + dt lambda); S = sum_g lambda C."""
    n = prob.mesh.n
    C = np.zeros((n, npg))
    S = np.zeros(n)
    for i in range(n):
        m = prob.materials[prob.mesh.materials[i]]
        if m.lam is None:
            continue
        for g in range(npg):
            if C0 is None:
                C[i, g] = (m.beta[g] / m.lam[g]) * P[i]
            else:
                C[i, g] = (C0[i, g] + dt * m.beta[g] * P[i]) / (1.0 + dt * m.lam[g])
            S[i] += m.lam[g] * C[i, g]
    return C, S


def run_coupled_transient(prob: Problem, npg: int, tol: float = 1e-12, max_iter: int = 200,
                          precursor_scale: float = 1.0) -> list[dict]:
    """Diffusion coupled to the precursor solver by implicit fixed-point iteration
    (CouplingSolver.cxx:77-145) over the steady state and every time step of prob.dt:
    diffusion solve, production rate to the precursors, their delayed source back to the
    diffusion solve, until the power and the delayed source stop changing (relative
    2-norm below tol).  The precursor populations are scaled by precursor_scale after the
    steady state, as a caller setting the "precursors" field would.  Returns per step phi,
    q, P, C, S and the total power."""
    res = solve_problem(prob)
    keff = res["keff"]
    ksf, nsf = _kappa_nu_tables(prob)
    V = prob.mesh.volumes
    C, S = precursor_step(prob, npg, res["P"], None, 0.0)
    out = [dict(keff=keff, phi=res["phi"], q=res["q"], P=res["P"], C=C, S=S, power=res["power"])]
    phi = res["phi"]
    C = C * precursor_scale
    for dt in prob.dt:
        phi_prev, C0 = phi.copy(), C.copy()
        q_old = S_old = None
        for _ in range(max_iter):
            R, b = diffusion_transient_system(prob, res["R"], dt, keff, phi_prev, S)
            phi = spla.spsolve(R.tocsc(), b)
            ph2 = phi.reshape(prob.mesh.n, prob.G)
            q = np.sum(ph2 * ksf * V[:, None], axis=1)
            P = np.sum(ph2 * nsf * V[:, None] / keff, axis=1)
            C, S = precursor_step(prob, npg, P, C0, dt)
            if q_old is not None and np.linalg.norm(q - q_old) < tol * np.linalg.norm(q) and \
                    np.linalg.norm(S - S_old) < tol * np.linalg.norm(S):
                break
            q_old, S_old = q, S
        out.append(dict(dt=dt, phi=phi, q=q, P=P, C=C, S=S, power=float(np.sum(q))))
    return out
