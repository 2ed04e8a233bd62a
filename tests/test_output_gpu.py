"""The .vtk and PETSc binary outputs of the neutronic solvers on the GPU path
(DiffusionSolver.cxx:410-432, SNSolver.cxx:753-780): the flux and power sections hold the
solution to the 6 printed digits and match the oracle's flux, and the PETSc dump holds the
solution exactly as pampa_get_field returns it.
"""
import os

import numpy as np
import pytest

import pampa_gb300 as pg
from helpers import rel_l2
from output_files import read_ptc, read_vtk
from oracle import pampa_oracle as po

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("solver", ["diffusion", "sn"])
def test_vtk_and_dump_of_a_solve(solver, tmp_path, monkeypatch):
    from pampa_gb300 import workloads as wl
    if solver == "diffusion":
        path = wl.diffusion_2d(str(tmp_path), n=12)
    else:
        path = wl.sn_hex(str(tmp_path), nq=4, nr=3, nz=2, order=2, block=2)
    ref = po.run_input(path)
    monkeypatch.chdir(tmp_path)
    with pg.Pampa(path, "-silent", "-vtk", "-petsc_dump") as p:
        p.solve()
        phi = p.field("scalar-flux")
        q = p.field("power")
        psi = p.field("angular-flux") if solver == "sn" else None
    v = read_vtk(str(tmp_path / "output_0.vtk"))
    n, G = len(q), len(phi) // len(q)
    assert v["num_cells"] == n
    for g in range(G):
        sec = v["scalars"][f"flux_{g + 1}"]
        assert np.allclose(sec, phi[g::G], rtol=5e-6, atol=0)
        assert rel_l2(sec, ref["phi"][g::G]) <= 1e-5
    assert np.allclose(v["scalars"]["power"], q, rtol=5e-6, atol=1e-300)
    if solver == "diffusion":
        assert np.array_equal(read_ptc(str(tmp_path / "scalar_flux_0.ptc")), phi)
    else:
        M = len(psi) // (n * G)
        assert np.array_equal(read_ptc(str(tmp_path / "angular_flux_0.ptc")), psi)
        assert np.allclose(v["scalars"][f"flux_1_{M}"], psi[M - 1::G * M], rtol=5e-6, atol=1e-300)
        # hexagonal prisms: 12 points per cell (VTK hexagonal prism)
        assert set(v["types"]) == {16}
    assert os.path.exists(tmp_path / "output_0.vtk")
