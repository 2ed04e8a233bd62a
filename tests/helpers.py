"""Test helpers: convert the oracle's assembled matrices into the GPU operator layouts."""
import numpy as np

from oracle import pampa_oracle as po


def rel_l2(a, b) -> float:
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def material_arrays(prob):
    st, nsf, ksf, chi, ss, D = po._material_tables(prob)
    return dict(sigma_t=st, sigma_s=ss, chi=chi, nu_sigma_f=nsf, kappa_sigma_f=ksf)


def diffusion_operator_from_oracle(prob, R):
    """pgpu_diffusion_operator arrays holding exactly the oracle's CSR matrix R."""
    mesh = prob.mesh
    n, F, G = mesh.n, mesh.F, prob.G
    R = R.tocsr()
    nbr = np.full((F, n), -1, dtype=np.int32)
    off = np.zeros((F, n * G))
    for f in range(F):
        nb = mesh.neighbors[:, f]
        ok = (f < mesh.num_faces) & (nb >= 0) & (nb < po.PAD)
        cells = np.nonzero(ok)[0]
        nbr[f, cells] = nb[cells]
        for g in range(G):
            rows = cells * G + g
            cols = nb[cells] * G + g
            off[f, rows] = np.asarray(R[rows, cols]).ravel()
    m = material_arrays(prob)
    return dict(neighbors=nbr, offdiag=off, diag=R.diagonal(), materials=mesh.materials,
                volumes=mesh.volumes, sigma_s=m["sigma_s"], chi=m["chi"], nu_sigma_f=m["nu_sigma_f"],
                kappa_sigma_f=m["kappa_sigma_f"])


def bc_split_input(d: str, solver: str = "diffusion", right: str = "reflective") -> str:
    """A 2D 10x8 input whose third material is a split boundary-condition material
    (`bc 1`, `split 1`; Mesh.cxx:24-204): its cells form two disconnected strips (x = 0 and
    x = 9), which splitting turns into the boundaries edge-0 and edge-1, and which are then
    removed from the mesh (68 cells remain).  edge-0 is vacuum, edge-1 `right`."""
    import os

    from pampa_gb300 import workloads as wl

    rng = np.random.default_rng(7)
    self_scatter = (0.2, 0.5) if solver == "sn" else None
    mats = wl.materials_2g(rng, 3, self_scatter=self_scatter)
    nx, ny = 10, 8
    lay = np.full((1, ny, nx), 2)
    lay[0, 2:6, 3:7] = 1
    lay[0, 1:7, 0] = 3
    lay[0, 1:7, nx - 1] = 3
    wl.write_cartesian_mesh(os.path.join(d, "mesh.pmp"), 5.0, nx, ny, 0, lay, {})
    for k, m in enumerate(mats):
        wl.write_material(os.path.join(d, f"mat{k + 1}.pmp"), m, solver == "diffusion")
    with open(os.path.join(d, "mat3.pmp"), "a") as fh:
        fh.write("bc 1\nsplit 1\n")
    lines = ["mesh cartesian mesh.pmp", "", "material fuel mat1.pmp", "material refl mat2.pmp",
             "material edge mat3.pmp", "", f"solver {solver} {{", "   energy-groups 2"]
    if solver == "sn":
        lines += ["   order 2", "   mixed-face-interpolation 1.0"]
    lines += ["   bc -x vacuum", "   bc +x vacuum", "   bc -y reflective", "   bc +y vacuum",
              "   bc edge-0 vacuum", f"   bc edge-1 {right}", "}"]
    with open(os.path.join(d, "input.pmp"), "w") as fh:
        fh.write("\n".join(lines) + "\n")
    return os.path.join(d, "input.pmp")


def feedback_input(d: str, solver: str = "diffusion") -> str:
    """A 2D 10x10 input whose two fuel materials carry feedback nuclear data
    (`nuclear-data-set`: 2 and 3 reference temperatures, cross sections changing with
    temperature) beside a constant reflector."""
    import os

    from pampa_gb300 import workloads as wl

    rng = np.random.default_rng(11)
    self_scatter = (0.2, 0.5) if solver == "sn" else None
    base = wl.materials_2g(rng, 3, self_scatter=self_scatter)
    diffusion = solver == "diffusion"
    temps = {0: [300.0, 900.0], 1: [300.0, 600.0, 1200.0]}
    for k in (0, 1):
        blocks = []
        for j, t in enumerate(temps[k]):
            m = dict(base[k])
            f = 1.0 + 0.15 * j                                   # hotter: less fission, more absorption
            m = dict(m, nsf=[x / f for x in m["nsf"]], sa=[x * f for x in m["sa"]],
                     D=[x * (1.0 + 0.05 * j) for x in m["D"]])
            path = os.path.join(d, f"tmp{k}{j}.pmp")
            wl.write_material(path, m, diffusion)
            blocks.append(open(path).read())
            os.remove(path)
        with open(os.path.join(d, f"mat{k + 1}.pmp"), "w") as fh:
            fh.write("nuclear-data-set {\n")
            fh.write(f"   temperature {len(temps[k])}\n   " + " ".join(str(t) for t in temps[k]) + "\n")
            for b in blocks:
                fh.write(b)
            fh.write("}\n")
    wl.write_material(os.path.join(d, "mat3.pmp"), base[2], diffusion)
    nx = ny = 10
    lay = np.full((1, ny, nx), 3)
    lay[0, 2:8, 2:5] = 1
    lay[0, 2:8, 5:8] = 2
    wl.write_cartesian_mesh(os.path.join(d, "mesh.pmp"), 5.0, nx, ny, 0, lay,
                            {"-x": "reflective", "+x": "vacuum", "-y": "reflective", "+y": "vacuum"})
    lines = ["mesh cartesian mesh.pmp", "", "material fuel1 mat1.pmp", "material fuel2 mat2.pmp",
             "material refl mat3.pmp", "", f"solver {solver} {{", "   energy-groups 2"]
    if solver == "sn":
        lines += ["   order 2", "   mixed-face-interpolation 1.0"]
    lines += ["}"]
    with open(os.path.join(d, "input.pmp"), "w") as fh:
        fh.write("\n".join(lines) + "\n")
    return os.path.join(d, "input.pmp")


def feedback_temperatures(n: int) -> np.ndarray:
    """A temperature field crossing every interpolation case: below the first reference
    temperature, between reference temperatures, on an inner one, above the last."""
    rng = np.random.default_rng(3)
    T = rng.choice([250.0, 450.0, 600.0, 750.0, 1000.0, 1500.0], size=n)
    return T


def sn_operator_from_oracle(prob, cart=(0, 0, 0)):
    """pgpu_sn_operator arrays of an SN problem read by the oracle (the layouts of
    include/pampa_gb300.h), for calls below the drop-in driver (serving)."""
    mesh = prob.mesh
    n, F, G = mesh.n, mesh.F, prob.G
    dirs, w, refl = po.quadrature(prob.order)
    gc = po.gauss_coefs(mesh, prob.delta)
    bcs = prob.boundary_conditions()
    kind = np.full((F, n), 3, dtype=np.int32)
    nbr = np.full((F, n), -1, dtype=np.int32)
    raxis = np.zeros((F, n), dtype=np.int32)
    for f in range(F):
        has = f < mesh.num_faces
        nb = mesh.neighbors[:, f]
        inter = has & (nb >= 0) & (nb < po.PAD)
        kind[f, inter] = 0
        nbr[f, inter] = nb[inter]
        # the reflection axis of face slot f: the axis of the normal of face f of cells 0, 1, 2
        # (SNSolver.cxx:539-543)
        ax = 0
        for a in range(3):
            if a < n and abs(float(mesh.normals[a, f, a])) > 1.0 - 1e-6:
                ax = a
        for c in np.nonzero(has & (nb < 0))[0]:
            t = bcs.get(int(-nb[c]), po.BoundaryCondition()).type
            kind[f, c] = 1 if t == po.BC_VACUUM else 2
            if t == po.BC_REFLECTIVE:
                raxis[f, c] = ax
    eff, mat_c = po._cell_materials(prob)
    st, nsf, ksf, chi, ss, _ = po._tables_of(eff, G)
    return dict(num_cell_faces=mesh.num_faces, face_kind=kind, neighbors=nbr, areas=mesh.areas.T,
                normals=np.transpose(mesh.normals, (1, 0, 2)), gauss=np.transpose(gc, (1, 0, 2)),
                reflect_axis=raxis, materials=mat_c, volumes=mesh.volumes, directions=dirs, weights=w,
                reflected=refl, sigma_t=st, sigma_s=ss, chi=chi, nu_sigma_f=nsf, kappa_sigma_f=ksf, cart=cart)


# --------------------------------------------------------------------------------------
# Fission operators applied on the host, for eigen-residual checks of solves too large for
# the oracle: F of DiffusionSolver::buildMatrices (DiffusionSolver.cxx:88-320: chi_g
# nu_sigma_f_g2 V in each cell's group block) and of SNSolver::buildMatrices
# (SNSolver.cxx:344-631: chi_g nu_sigma_f_g2 w_m2 V), with the material values as the
# solvers read them from the written files (workloads.material_arrays).
# --------------------------------------------------------------------------------------


def fission_source(mats, layout, phi) -> np.ndarray:
    """f[i, g] = chi_g(m_i) sum_g2 nu_sigma_f_g2(m_i) phi[i, g2] (no volume), m_i the cell's
    material from the 1-based `layout` in cell order."""
    from pampa_gb300 import workloads as wl
    t = wl.material_arrays(mats)
    G = t["G"]
    mat = np.asarray(layout).reshape(-1) - 1
    phi = np.asarray(phi, dtype=np.float64).reshape(-1, G)
    f = np.zeros_like(phi)
    for m in range(len(mats)):
        idx = np.nonzero(mat == m)[0]
        if idx.size and np.any(t["nu_sigma_f"][m]):
            f[idx] = np.outer(phi[idx] @ t["nu_sigma_f"][m], t["chi"][m])
    return f


def sn_scalar_flux(psi, weights, G: int) -> np.ndarray:
    """phi[i, g] = sum_m w_m psi[(i G + g) M + m]."""
    w = np.asarray(weights, dtype=np.float64)
    return (np.asarray(psi, dtype=np.float64).reshape(-1, w.size) @ w).reshape(-1, G)


def eigen_residual(Rx, f, M: int = 1, chunk: int = 1 << 22) -> tuple[float, float]:
    """For R x = (V/k) F' x with F' x = f broadcast over M directions: the least-squares
    scale c = <f, R x> / <f, f> (c = V/k for an eigenpair) and ||R x - c f|| / ||c f||,
    summed chunk by chunk of rows (no cancellation between the two norms)."""
    Rx = np.asarray(Rx, dtype=np.float64).reshape(-1, M)
    fv = np.asarray(f, dtype=np.float64).reshape(-1)
    num = float(fv @ Rx.sum(axis=1))
    den = float(M * (fv @ fv))
    c = num / den
    ss = 0.0
    for a in range(0, fv.size, chunk):
        r = Rx[a:a + chunk] - c * fv[a:a + chunk, None]
        ss += float(np.sum(r * r))
    return c, float(np.sqrt(ss / (c * c * den)))
