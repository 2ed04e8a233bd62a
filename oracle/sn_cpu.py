"""CPU sweep baseline -- TEST/BASELINE INFRASTRUCTURE ONLY.

Builds the inputs of ``oracle/cpu_sweep.c`` (upwind sweep of the reference's SN operator,
pure upwind, no LS) from the oracle's own mesh and quadrature, and times sweeps on the
host cores.  Only ``bench.py``'s CPU legs use it.
"""

from __future__ import annotations

import ctypes as C
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


def _lib():
    L = C.CDLL(build())
    L.cpu_sweep_threads.restype = C.c_int
    return L


def sweep_inputs(prob: po.Problem) -> dict:
    """Face data, quadrature and per-pattern level schedules for the upwind sweep."""
    mesh = prob.mesh
    n, F, G = mesh.n, mesh.F, prob.G
    dirs, w, refl = po.quadrature(prob.order)
    M = len(w)
    gc = po.gauss_coefs(mesh, prob.delta)
    bcs = prob.boundary_conditions()
    kind = np.full((F, n), 3, dtype=np.int32)
    nbr = np.full((F, n), -1, dtype=np.int32)
    rslot = np.full((F, n), -1, dtype=np.int32)
    nrefl = 0
    for f in range(F):
        has = f < mesh.num_faces
        nb = mesh.neighbors[:, f]
        inter = has & (nb >= 0) & (nb < po.PAD)
        kind[f, inter] = 0
        nbr[f, inter] = nb[inter]
        for c in np.nonzero(has & (nb < 0))[0]:
            t = bcs[int(-nb[c])].type
            if t == po.BC_VACUUM:
                kind[f, c] = 1
            elif t == po.BC_REFLECTIVE:
                kind[f, c] = 2
                rslot[f, c] = nrefl
                nrefl += 1
            else:
                raise ValueError("boundary condition not supported by the sweep")
    area = np.ascontiguousarray(mesh.areas.T)
    nrm = np.ascontiguousarray(np.transpose(mesh.normals, (1, 0, 2)))
    gauss = np.ascontiguousarray(np.transpose(gc, (1, 0, 2)))
    # upwind patterns by the sign of mu on every interior face, levels by relaxation
    mu_all = np.einsum("nfd,md->mnf", mesh.normals, dirs)
    inter_nf = (np.arange(F)[None, :] < mesh.num_faces[:, None]) & (mesh.neighbors >= 0) & (mesh.neighbors < po.PAD)
    keys = {}
    pat_dirs = []
    for m in range(M):
        key = ((mu_all[m] < 0.0) & inter_nf).tobytes()
        if key not in keys:
            keys[key] = len(pat_dirs)
            pat_dirs.append([m])
        else:
            pat_dirs[keys[key]].append(m)
    pat_dirs_ptr = np.cumsum([0] + [len(v) for v in pat_dirs]).astype(np.int32)
    order, lev_ptr, pat_lev_ptr, pat_nlev = [], [], [], []
    nbr_safe = np.where(inter_nf, mesh.neighbors, 0)
    for v in pat_dirs:
        up = (mu_all[v[0]] < 0.0) & inter_nf
        level = np.zeros(n, dtype=np.int64)
        while True:
            cand = np.where(up, level[nbr_safe] + 1, 0).max(axis=1)
            new = np.maximum(level, cand)
            if np.array_equal(new, level):
                break
            level = new
        o = np.argsort(level, kind="stable")
        counts = np.bincount(level, minlength=level.max() + 1)
        pat_lev_ptr.append(sum(len(x) for x in lev_ptr))
        lev_ptr.append(np.concatenate([[0], np.cumsum(counts)]))
        pat_nlev.append(len(counts))
        order.append(o)
    return dict(n=n, G=G, M=M, F=F, nf=mesh.num_faces.astype(np.int32), kind=kind, nbr=nbr, area=area,
                nrm=nrm, gauss=gauss, rslot=rslot, mat=mesh.materials.astype(np.int32),
                vol=mesh.volumes.astype(np.float64), dirs=dirs, w=w,
                st=np.array([m.st for m in prob.materials], dtype=np.float64),
                npat=len(pat_dirs), pat_dirs_ptr=pat_dirs_ptr,
                pat_dirs=np.concatenate([np.array(v, dtype=np.int32) for v in pat_dirs]),
                pat_lev_ptr=np.array(pat_lev_ptr, dtype=np.int32), pat_nlev=np.array(pat_nlev, dtype=np.int32),
                lev_ptr=np.concatenate(lev_ptr).astype(np.int32), order=np.concatenate(order).astype(np.int32),
                nrefl=nrefl)


def time_sweeps(inp: dict, nsweeps: int, threads: int | None = None) -> tuple[float, int]:
    """Seconds per (sweep + scalar-flux moment) on the host cores, and threads used."""
    L = _lib()
    threads = threads or L.cpu_sweep_threads()
    n, G, M = inp["n"], inp["G"], inp["M"]
    rng = np.random.default_rng(0)
    q = rng.random(n * G)
    bnd = rng.random(max(inp["nrefl"], 1) * G * M)
    psi = np.zeros(n * G * M)
    phi0 = np.zeros(n * G)
    P = lambda a: a.ctypes.data_as(C.c_void_p)
    a = inp
    args = [C.c_int(n), C.c_int(G), C.c_int(M), C.c_int(a["F"]), P(a["nf"]), P(a["kind"]), P(a["nbr"]),
            P(a["area"]), P(a["nrm"]), P(a["gauss"]), P(a["rslot"]), P(a["mat"]), P(a["vol"]), P(a["dirs"]),
            P(a["st"]), C.c_int(a["npat"]), P(a["pat_dirs_ptr"]), P(a["pat_dirs"]), P(a["pat_lev_ptr"]),
            P(a["pat_nlev"]), P(a["lev_ptr"]), P(a["order"]), P(q), P(bnd) if a["nrefl"] else None, P(psi),
            C.c_int(threads)]
    L.cpu_sweep(*args)  # warm-up (page-in)
    t0 = time.perf_counter()
    for _ in range(nsweeps):
        L.cpu_sweep(*args)
        L.cpu_moment(C.c_longlong(n * G), C.c_int(M), P(a["w"]), P(psi), P(phi0), C.c_int(threads))
    return (time.perf_counter() - t0) / nsweeps, threads
