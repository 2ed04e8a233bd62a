"""Seeded synthetic k-eigenvalue workloads, written as reference-format ``.pmp`` inputs.

Each generator writes ``input.pmp``, ``mesh.pmp`` and ``mat<k>.pmp`` files into a
directory so the reference parser, the oracle and this library read identical inputs.
Cross sections are macroscopic (1/cm); the total cross section is written as
sigma_t = sigma_a + sum of out-scatter (the reference reads sigma_t directly).

Workloads (sizes are the defaults; every generator takes smaller sizes for tests):

* ``diffusion_2d``  -- 2-group diffusion on a 2D Cartesian 34x34 mesh of 5 cm cells,
  17x17 blocks of 2x2 cells, 4 materials (one non-fissile reflector), vacuum on +x/+y,
  reflective on -x/-y.
* ``sn_3d``         -- 2-group S8 discrete ordinates on a 3D Cartesian 64x64x32 mesh of
  2 cm cells with within-group scattering, pure upwind (mixed-face-interpolation 1.0),
  no LS boundary correction, vacuum on +x/+y/+z, reflective on -x/-y/-z.
* ``diffusion_3d_7g`` -- 7-group diffusion on a 3D Cartesian 256x256x128 mesh of 2 cm
  cells, 6 materials in 8x8x8-cell blocks, down-scatter g->g+1, g->g+2 and up-scatter
  g->g-1 for the three thermal groups, lognormal entries, chi on groups 1-3.
"""

from __future__ import annotations

import math
import os

import numpy as np

# cross-section ranges of the 2-group family (1/cm; D in cm)
RANGES_2G = dict(D1=(1.2, 1.5), D2=(0.3, 0.4), sa1=(0.008, 0.012), sa2=(0.05, 0.09),
                 nsf1=(0.0, 0.006), nsf2=(0.0, 0.14), s12=(0.015, 0.025))


def _u(rng, lo_hi):
    lo, hi = lo_hi
    return float(rng.uniform(lo, hi))


def materials_2g(rng, num: int, self_scatter: tuple | None = None, reflector_last: bool = True):
    """`num` 2-group materials; the last one is a non-fissile reflector."""
    mats = []
    for m in range(num):
        D = [_u(rng, RANGES_2G["D1"]), _u(rng, RANGES_2G["D2"])]
        sa = [_u(rng, RANGES_2G["sa1"]), _u(rng, RANGES_2G["sa2"])]
        nsf = [_u(rng, RANGES_2G["nsf1"]), _u(rng, RANGES_2G["nsf2"])]
        if reflector_last and m == num - 1:
            nsf = [0.0, 0.0]
        ss = np.zeros((2, 2))
        ss[0, 1] = _u(rng, RANGES_2G["s12"])
        if self_scatter is not None:
            ss[0, 0] = _u(rng, self_scatter)
            ss[1, 1] = _u(rng, self_scatter)
        mats.append(dict(G=2, D=D, sa=sa, nsf=nsf, ss=ss, chi=[1.0, 0.0]))
    return mats


def materials_multigroup(rng, num: int, G: int = 7):
    """`num` G-group materials for the 7-group family (one non-fissile)."""
    mats = []
    t = np.linspace(0.0, 1.0, G)
    for m in range(num):
        jitter = rng.uniform(0.9, 1.1, size=G)
        D = np.exp(np.log(1.35) * (1 - t) + np.log(0.35) * t) * jitter
        sa = np.exp(np.log(0.010) * (1 - t) + np.log(0.070) * t) * rng.uniform(0.8, 1.2, size=G)
        nsf = np.exp(np.log(0.003) * (1 - t) + np.log(0.12) * t) * rng.uniform(0.8, 1.2, size=G)
        if m == num - 1:
            nsf[:] = 0.0
        ss = np.zeros((G, G))
        for g in range(G):
            for g2, on in ((g + 1, True), (g + 2, True), (g - 1, g >= G - 3)):
                if on and 0 <= g2 < G:
                    med = math.exp(rng.uniform(math.log(1e-3), math.log(5e-2)))
                    ss[g, g2] = med * math.exp(rng.normal(0.0, 0.5))
        chi = np.zeros(G)
        chi[:3] = [0.6, 0.3, 0.1]
        mats.append(dict(G=G, D=list(D), sa=list(sa), nsf=list(nsf), ss=ss, chi=list(chi)))
    return mats


def _fmt(vals) -> str:
    return " ".join(f"{v:.10g}" for v in vals)


def write_material(path: str, mat: dict, diffusion: bool = True):
    G = mat["G"]
    ss = np.asarray(mat["ss"])
    st = [mat["sa"][g] + ss[g].sum() for g in range(G)]
    lines = ["nuclear-data {", f"   energy-groups {G}", "   sigma-total", "   " + _fmt(st)]
    if any(v > 0 for v in mat["nsf"]):
        lines += ["   nu-sigma-fission", "   " + _fmt(mat["nsf"]), "   fission-spectrum",
                  "   " + _fmt(mat["chi"])]
    lines += ["   sigma-scattering"] + ["   " + _fmt(ss[g]) for g in range(G)]
    if diffusion:
        lines += ["   diffusion-coefficient", "   " + _fmt(mat["D"])]
    lines += ["}"]
    with open(path, "w") as fh:
        fh.write("\n".join(lines) + "\n")


def write_cartesian_mesh(path: str, d: float, nx: int, ny: int, nz: int, layout: np.ndarray,
                         bcs: dict[str, str]):
    """layout: (nz, ny, nx) 1-based material indices (0 = void)."""
    lines = [f"dx -{nx}", f"{d:.6f}", f"dy -{ny}", f"{d:.6f}"]
    if nz > 0:
        lines += [f"dz -{nz}", f"{d:.6f}"]
    lines.append("")
    for b, t in bcs.items():
        lines.append(f"bc {b} {t}")
    lines.append("")
    ncell = layout.size
    lines.append(f"materials {ncell}")
    flat = layout.reshape(-1, nx)
    for row in flat:
        lines.append(" ".join(str(int(v)) for v in row))
    with open(path, "w") as fh:
        fh.write("\n".join(lines) + "\n")


def _block_layout(rng, shape, block, num_materials) -> np.ndarray:
    nb = [int(math.ceil(s / b)) for s, b in zip(shape, block)]
    blocks = rng.integers(1, num_materials + 1, size=nb)
    lay = blocks
    for ax, b in enumerate(block):
        lay = np.repeat(lay, b, axis=ax)
    return lay[tuple(slice(0, s) for s in shape)]


def diffusion_2d(out_dir: str, n: int = 34, cell: float = 5.0, seed: int = 1) -> str:
    """2-group 2D diffusion (34x34 of 5 cm cells by default)."""
    os.makedirs(out_dir, exist_ok=True)
    rng = np.random.default_rng(seed)
    mats = materials_2g(rng, 4)
    layout = _block_layout(rng, (1, n, n), (1, 2, 2), 4)
    write_cartesian_mesh(os.path.join(out_dir, "mesh.pmp"), cell, n, n, 0, layout,
                         {"-x": "reflective", "+x": "vacuum", "-y": "reflective", "+y": "vacuum"})
    for k, m in enumerate(mats):
        write_material(os.path.join(out_dir, f"mat{k + 1}.pmp"), m)
    lines = ["mesh cartesian mesh.pmp", ""]
    lines += [f"material mat{k + 1} mat{k + 1}.pmp" for k in range(len(mats))]
    lines += ["", "solver diffusion {", "   energy-groups 2", "}"]
    path = os.path.join(out_dir, "input.pmp")
    with open(path, "w") as fh:
        fh.write("\n".join(lines) + "\n")
    return path


def sn_3d(out_dir: str, nx: int = 64, ny: int = 64, nz: int = 32, cell: float = 2.0, order: int = 8,
          seed: int = 2, block: int = 4) -> str:
    """2-group S_N on a 3D Cartesian mesh (64x64x32 of 2 cm cells, S8 by default)."""
    os.makedirs(out_dir, exist_ok=True)
    rng = np.random.default_rng(seed)
    mats = materials_2g(rng, 4, self_scatter=(0.2, 0.5))
    layout = _block_layout(rng, (nz, ny, nx), (block, block, block), 4)
    write_cartesian_mesh(os.path.join(out_dir, "mesh.pmp"), cell, nx, ny, nz, layout,
                         {"-x": "reflective", "+x": "vacuum", "-y": "reflective", "+y": "vacuum",
                          "-z": "reflective", "+z": "vacuum"})
    for k, m in enumerate(mats):
        write_material(os.path.join(out_dir, f"mat{k + 1}.pmp"), m, diffusion=False)
    lines = ["mesh cartesian mesh.pmp", ""]
    lines += [f"material mat{k + 1} mat{k + 1}.pmp" for k in range(len(mats))]
    lines += ["", "solver sn {", "   energy-groups 2", f"   order {order}",
              "   mixed-face-interpolation 1.0", "   least-squares-boundary-interpolation 0", "}"]
    path = os.path.join(out_dir, "input.pmp")
    with open(path, "w") as fh:
        fh.write("\n".join(lines) + "\n")
    return path


def diffusion_3d_7g_data(nx: int = 256, ny: int = 256, nz: int = 128, seed: int = 3, block: int = 8,
                         G: int = 7) -> tuple[list[dict], np.ndarray]:
    """Materials and (nz, ny, nx) layout of diffusion_3d_7g's problem."""
    rng = np.random.default_rng(seed)
    mats = materials_multigroup(rng, 6, G)
    layout = _block_layout(rng, (nz, ny, nx), (block, block, block), 6)
    return mats, layout


def diffusion_3d_7g(out_dir: str, nx: int = 256, ny: int = 256, nz: int = 128, cell: float = 2.0,
                    seed: int = 3, block: int = 8, G: int = 7) -> str:
    """7-group 3D diffusion (256x256x128 of 2 cm cells by default)."""
    os.makedirs(out_dir, exist_ok=True)
    mats, layout = diffusion_3d_7g_data(nx, ny, nz, seed, block, G)
    write_cartesian_mesh(os.path.join(out_dir, "mesh.pmp"), cell, nx, ny, nz, layout,
                         {"-x": "reflective", "+x": "vacuum", "-y": "reflective", "+y": "vacuum",
                          "-z": "reflective", "+z": "vacuum"})
    for k, m in enumerate(mats):
        write_material(os.path.join(out_dir, f"mat{k + 1}.pmp"), m)
    lines = ["mesh cartesian mesh.pmp", ""]
    lines += [f"material mat{k + 1} mat{k + 1}.pmp" for k in range(len(mats))]
    lines += ["", "solver diffusion {", f"   energy-groups {G}", "}"]
    path = os.path.join(out_dir, "input.pmp")
    with open(path, "w") as fh:
        fh.write("\n".join(lines) + "\n")
    return path


def materials_4g(rng, num: int):
    """`num` 4-group materials (isotropic scattering, one non-fissile) from the 2-group ranges,
    log-interpolated between the fast and thermal values."""
    mats = []
    G = 4
    t = np.linspace(0.0, 1.0, G)
    for m in range(num):
        D1, D2 = _u(rng, RANGES_2G["D1"]), _u(rng, RANGES_2G["D2"])
        a1, a2 = _u(rng, RANGES_2G["sa1"]), _u(rng, RANGES_2G["sa2"])
        f1, f2 = _u(rng, (0.001, 0.006)), _u(rng, (0.02, 0.14))
        D = list(np.exp(np.log(D1) * (1 - t) + np.log(D2) * t))
        sa = list(np.exp(np.log(a1) * (1 - t) + np.log(a2) * t))
        nsf = list(np.exp(np.log(f1) * (1 - t) + np.log(f2) * t))
        if m == num - 1:
            nsf = [0.0] * G
        ss = np.zeros((G, G))
        for g in range(G):
            ss[g, g] = _u(rng, (0.2, 0.5))
            if g + 1 < G:
                ss[g, g + 1] = _u(rng, RANGES_2G["s12"])
        chi = [0.8, 0.2, 0.0, 0.0]
        mats.append(dict(G=G, D=D, sa=sa, nsf=nsf, ss=ss, chi=chi))
    return mats


def write_hex_prism_mesh(path: str, nq: int, nr: int, pitch: float, nz: int, dz: float, layout: np.ndarray):
    """Unstructured extruded mesh of an nq x nr lattice of flat-topped hexagons (flat-to-flat
    = pitch), CCW points, every lateral boundary edge on the default boundary 'exterior'
    (declared before dz so the default boundary keeps its own index), vacuum everywhere.
    layout: (nz, nr, nq) 1-based material indices."""
    s = pitch / math.sqrt(3.0)           # side length
    pts: dict = {}
    coords = []
    cells = []

    def pid(x, y):
        key = (round(x, 9), round(y, 9))
        if key not in pts:
            pts[key] = len(coords)
            coords.append((x, y))
        return pts[key]

    for r in range(nr):
        for q in range(nq):
            cx = 1.5 * s * q
            cy = pitch * (r + 0.5 * (q & 1))
            ids = [pid(cx + s * math.cos(math.radians(60 * k)), cy + s * math.sin(math.radians(60 * k)))
                   for k in range(6)]
            cells.append(ids)
    lines = [f"points {len(coords)}"] + [f"{x:.9f} {y:.9f}" for x, y in coords]
    lines += [f"cells {len(cells)} {6 * len(cells)}"] + [" ".join(str(i) for i in c) for c in cells]
    lines += ["boundary exterior 0", f"dz -{nz}", f"{dz:.6f}", "",
              "bc exterior vacuum", "bc -z vacuum", "bc +z vacuum", ""]
    lines.append(f"materials {layout.size}")
    for row in layout.reshape(nz, -1):
        lines.append(" ".join(str(int(v)) for v in row))
    with open(path, "w") as fh:
        fh.write("\n".join(lines) + "\n")


def sn_hex_data(nq: int = 200, nr: int = 200, nz: int = 40, seed: int = 5,
                block: int = 10) -> tuple[list[dict], np.ndarray]:
    """Materials and (nz, nr, nq) layout of sn_hex's problem."""
    rng = np.random.default_rng(seed)
    mats = materials_4g(rng, 5)
    layout = _block_layout(rng, (nz, nr, nq), (max(1, nz // 4), block, block), 5)
    return mats, layout


def sn_hex(out_dir: str, nq: int = 200, nr: int = 200, nz: int = 40, pitch: float = 2.0, dz: float = 2.0,
           order: int = 8, seed: int = 5, block: int = 10) -> str:
    """4-group S_N on a hexagonal-prism lattice (200 x 200 hexagons x 40 layers by default,
    1.6M cells), 5 materials in blocks of `block` hexagons, vacuum boundaries."""
    os.makedirs(out_dir, exist_ok=True)
    mats, layout = sn_hex_data(nq, nr, nz, seed, block)
    write_hex_prism_mesh(os.path.join(out_dir, "mesh.pmp"), nq, nr, pitch, nz, dz, layout)
    for k, m in enumerate(mats):
        write_material(os.path.join(out_dir, f"mat{k + 1}.pmp"), m, diffusion=False)
    lines = ["mesh unstructured mesh.pmp", ""]
    lines += [f"material mat{k + 1} mat{k + 1}.pmp" for k in range(len(mats))]
    lines += ["", "solver sn {", "   energy-groups 4", f"   order {order}",
              "   mixed-face-interpolation 1.0", "   least-squares-boundary-interpolation 0", "}"]
    path = os.path.join(out_dir, "input.pmp")
    with open(path, "w") as fh:
        fh.write("\n".join(lines) + "\n")
    return path


# --------------------------------------------------------------------------------------
# Operators built in memory (no .pmp round trip): for request streams whose sizes make
# file parsing the bottleneck.  Same formulas as the reference's DiffusionSolver::
# buildMatrices (DiffusionSolver.cxx:88-320) on a uniform Cartesian mesh, with the
# material values rounded as the .pmp writers above round them, so that the arrays equal
# the ones the drop-in host assembles from the same problem written to files.
# --------------------------------------------------------------------------------------

KAPPA_OVER_NU = 3.2e-11 / 2.4355  # default kappa-sigma-fission / nu-sigma-fission


def _rt(v: float) -> float:
    return float(f"{v:.10g}")


def material_arrays(mats: list[dict]) -> dict:
    """Per-material tables as the solver reads them from the written material files."""
    G = mats[0]["G"]
    D = np.array([[_rt(v) for v in m["D"]] for m in mats])
    ss = np.array([[[_rt(v) for v in row] for row in np.asarray(m["ss"], dtype=float)] for m in mats])
    st = np.array([[_rt(m["sa"][g] + np.asarray(m["ss"], dtype=float)[g].sum()) for g in range(G)] for m in mats])
    fiss = np.array([any(v > 0 for v in m["nsf"]) for m in mats])
    nsf = np.array([[_rt(v) for v in m["nsf"]] if f else [0.0] * G for m, f in zip(mats, fiss)])
    chi = np.array([[_rt(v) for v in m["chi"]] if f else [0.0] * G for m, f in zip(mats, fiss)])
    return dict(G=G, D=D, sigma_s=ss, sigma_t=st, nu_sigma_f=nsf, chi=chi, kappa_sigma_f=nsf * KAPPA_OVER_NU)


def cartesian_diffusion_operator(nx: int, ny: int, nz: int, h: float, layout: np.ndarray, mats: list[dict],
                                 reflective=("-x", "-y", "-z")) -> dict:
    """pgpu_diffusion_operator arrays of a uniform 3D Cartesian mesh (cells of side h,
    layout (nz, ny, nx) of 1-based material indices, faces -y +x +y -x -z +z, vacuum on
    every side not listed in `reflective`)."""
    t = material_arrays(mats)
    G = t["G"]
    n = nx * ny * nz
    mat = np.ascontiguousarray(layout, dtype=np.int64).reshape(-1) - 1
    V, A = h * h * h, h * h
    x = np.arange(n) % nx
    y = (np.arange(n) // nx) % ny
    z = np.arange(n) // (nx * ny)
    Dc = t["D"][mat]  # (n, G)
    self_ss = t["sigma_s"][:, np.arange(G), np.arange(G)]  # (materials, G)
    diag = t["sigma_t"][mat] * V - self_ss[mat] * V
    faces = [("-y", y > 0, -nx), ("+x", x < nx - 1, 1), ("+y", y < ny - 1, nx), ("-x", x > 0, -1),
             ("-z", z > 0, -nx * ny), ("+z", z < nz - 1, nx * ny)]
    nbr = np.full((6, n), -1, dtype=np.int32)
    off = np.zeros((6, n, G))
    for f, (side, inside, step) in enumerate(faces):
        cells = np.nonzero(inside)[0]
        nb = cells + step
        nbr[f, cells] = nb
        same = mat[nb] == mat[cells]
        Di, Dn = Dc[cells], Dc[nb]
        r = np.where(same[:, None], -(1.0 / h) * Di * A, 0.0)
        w1 = (2.0 / h) * (Di * A)
        w2 = (2.0 / h) * (Dn * A)
        r = np.where(same[:, None], r, -(w1 * w2) / (w1 + w2))
        off[f, cells] = r
        diag[cells] -= r
        bnd = np.nonzero(~inside)[0]
        if side not in reflective:
            diag[bnd] += (2.0 / h) * Dc[bnd] * A
    return dict(neighbors=nbr, offdiag=off.reshape(6, n * G), diag=diag.reshape(-1),
                materials=mat.astype(np.int32), volumes=np.full(n, V), sigma_s=t["sigma_s"], chi=t["chi"],
                nu_sigma_f=t["nu_sigma_f"], kappa_sigma_f=t["kappa_sigma_f"])


def diffusion_request(rng, nx: int, ny: int, nz: int, G: int, h: float = 2.0, perturb: float = math.log(1.05),
                      block: int = 4, nmat: int = 4) -> tuple[dict, list[dict], np.ndarray]:
    """One serving request: random block layout of `nmat` materials (2-group ranges for
    G = 2, the multigroup family otherwise) with an independent lognormal perturbation
    (sigma_ln = perturb) of every cross section.  Returns (operator, materials, layout)."""
    mats = materials_2g(rng, nmat) if G == 2 else materials_multigroup(rng, nmat, G)
    for m in mats:
        for key in ("D", "sa", "nsf"):
            m[key] = [float(v * math.exp(rng.normal(0.0, perturb))) for v in m[key]]
        ss = np.asarray(m["ss"], dtype=float)
        m["ss"] = ss * np.exp(rng.normal(0.0, perturb, size=ss.shape))
    layout = _block_layout(rng, (nz, ny, nx), (block, block, block), nmat)
    return cartesian_diffusion_operator(nx, ny, nz, h, layout, mats), mats, layout


def diffusion_request_op(spec: tuple) -> dict:
    """Operator of the serving request spec = (nx, ny, nz, G, seed): diffusion_request with
    a generator seeded by `seed` (a top-level function, so a process pool can build a
    stream of requests in parallel)."""
    nx, ny, nz, G, seed = spec
    return diffusion_request(np.random.default_rng(int(seed)), int(nx), int(ny), int(nz), int(G))[0]


def write_diffusion_input(out_dir: str, nx: int, ny: int, nz: int, h: float, layout: np.ndarray,
                          mats: list[dict]) -> str:
    """The .pmp input of a problem built by cartesian_diffusion_operator (same boundaries)."""
    os.makedirs(out_dir, exist_ok=True)
    write_cartesian_mesh(os.path.join(out_dir, "mesh.pmp"), h, nx, ny, nz, layout,
                         {"-x": "reflective", "+x": "vacuum", "-y": "reflective", "+y": "vacuum",
                          "-z": "reflective", "+z": "vacuum"})
    for k, m in enumerate(mats):
        write_material(os.path.join(out_dir, f"mat{k + 1}.pmp"), m)
    lines = ["mesh cartesian mesh.pmp", ""]
    lines += [f"material mat{k + 1} mat{k + 1}.pmp" for k in range(len(mats))]
    lines += ["", "solver diffusion {", f"   energy-groups {mats[0]['G']}", "}"]
    path = os.path.join(out_dir, "input.pmp")
    with open(path, "w") as fh:
        fh.write("\n".join(lines) + "\n")
    return path
