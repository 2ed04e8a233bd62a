"""The host-side fission operators and the eigen-residual measure that the full-size GPU
tests use (tests/test_full_size_gpu.py), checked here against the oracle on small meshes:
the fission source equals the oracle's assembled F (DiffusionSolver.cxx:88-320,
SNSolver.cxx:344-631) applied to random vectors, the generators' layouts are the cell
order of the meshes the readers build, and the oracle's own eigenpairs have a residual at
rounding level under the same measure."""
import math

import numpy as np

from helpers import eigen_residual, fission_source, sn_scalar_flux
from oracle import pampa_oracle as po
from pampa_gb300 import workloads as wl


def test_diffusion_fission_source_and_residual_against_oracle(tmp_path):
    nx, ny, nz, h = 6, 5, 4, 2.0
    path = wl.diffusion_3d_7g(str(tmp_path), nx=nx, ny=ny, nz=nz, block=2)
    mats, layout = wl.diffusion_3d_7g_data(nx, ny, nz, block=2)
    prob = po.read_problem(path)
    assert np.array_equal(prob.mesh.materials, layout.reshape(-1) - 1)
    R, F = po.assemble_diffusion(prob)
    V = h ** 3
    x = np.random.default_rng(1).random(R.shape[0])
    ref = F @ x
    got = V * fission_source(mats, layout, x).reshape(-1)
    assert np.linalg.norm(got - ref) <= 1e-13 * np.linalg.norm(ref)
    res = po.solve_problem(prob)
    c, rel = eigen_residual(R @ res["phi"], fission_source(mats, layout, res["phi"]))
    assert abs(c * res["keff"] / V - 1.0) <= 1e-10, (c, res["keff"])
    assert rel <= 1e-10, rel


def test_sn_hex_fission_source_and_residual_against_oracle(tmp_path):
    nq, nr, nz, pitch, dz = 4, 3, 2, 2.0, 2.0
    path = wl.sn_hex(str(tmp_path), nq=nq, nr=nr, nz=nz, pitch=pitch, dz=dz)
    mats, layout = wl.sn_hex_data(nq, nr, nz)
    prob = po.read_problem(path)
    assert np.array_equal(prob.mesh.materials, layout.reshape(-1) - 1)
    V = math.sqrt(3.0) / 2.0 * pitch * pitch * dz  # regular hexagon, flat-to-flat = pitch
    assert np.allclose(prob.mesh.volumes, V, rtol=1e-8, atol=0)
    R, F, w = po.assemble_sn(prob)
    G, M = prob.G, w.size
    x = np.random.default_rng(2).random(R.shape[0])
    ref = F @ x
    f = fission_source(mats, layout, sn_scalar_flux(x, w, G))
    got = (prob.mesh.volumes[:, None, None] * np.repeat(f[:, :, None], M, axis=2)).reshape(-1)
    assert np.linalg.norm(got - ref) <= 1e-13 * np.linalg.norm(ref)
    res = po.solve_problem(prob)
    psi = res["psi"]
    c, rel = eigen_residual(R @ psi, fission_source(mats, layout, sn_scalar_flux(psi, w, G)), M)
    assert abs(c * res["keff"] / V - 1.0) <= 1e-8, (c, res["keff"])  # volumes equal to 1e-8
    assert rel <= 1e-8, rel
