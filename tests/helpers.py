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
