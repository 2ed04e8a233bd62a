"""The .vtk and PETSc binary outputs (vtk.cxx:28-170, petsc.cxx:491-511) written by the
drop-in driver, on the precursor golden case, which runs without a GPU (the precursor
solver is host bookkeeping): the mesh section must hold the grid's points and every
physical cell's 8 points in gmsh order (their mean is the oracle's cell centroid), the
cell types and the materials; each precursor group's section and the PETSc dump must hold
the printed populations, steady state C = beta/lambda P with the uniform production rate.
"""
import os
import subprocess

import numpy as np

from conftest import ROOT, materialize_case
from output_files import read_ptc, read_vtk
from oracle import pampa_oracle as po


def test_vtk_and_petsc_dump_of_the_precursor_case(tmp_path):
    import pampa_gb300.build as b
    lib = b.build()
    libdir = os.path.dirname(lib)
    exe = str(tmp_path / "pampa")
    subprocess.run(["gcc", "-O2", "-std=c99", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "frontend", "pampa_main.c"), "-L", libdir, "-lpampa_gb300",
                    f"-Wl,-rpath,{libdir}", "-o", exe], check=True)
    path = materialize_case("pwr-iaea-benchmark/cartesian-precursors-3d", str(tmp_path))
    d = os.path.dirname(path)
    res = subprocess.run([exe, "input.pmp", "-silent", "-vtk", "-vtk_interval", "2", "-petsc_dump"], cwd=d,
                         capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stdout[-2000:]
    files = sorted(os.listdir(d))
    # steps 0..4 with interval 2: files for n = 0, 2, 4 named by n / 2
    assert [f for f in files if f.endswith(".vtk")] == ["output_0.vtk", "output_1.vtk", "output_2.vtk"]
    assert all(f"precursors_{n}.ptc" in files for n in range(5))
    mesh, _ = po.read_cartesian(os.path.join(d, "mesh.pmp"))
    v = read_vtk(os.path.join(d, "output_0.vtk"))
    n = len(mesh.volumes)
    assert v["num_cells"] == n and len(v["cells"]) == n
    assert len(v["points"]) == 35 * 35 * 35
    assert all(len(c) == 8 for c in v["cells"]) and set(v["types"]) == {12}
    cent = np.array([v["points"][c].mean(axis=0) for c in v["cells"]])
    assert np.allclose(cent, mesh.centroids, rtol=0, atol=1e-9)
    assert np.array_equal(v["scalars"]["materials"], mesh.materials + 1)
    # precursor populations: beta_g / lambda_g / n in fuel, 0 elsewhere (6 groups)
    C = read_ptc(os.path.join(d, "precursors_0.ptc")).reshape(n, 6)
    fuel = C.max(axis=1) > 0
    assert f"{C.max():.3e}" == "1.424e-06"
    for g in range(6):
        sec = v["scalars"][f"precursor_{g + 1}"]
        assert np.allclose(sec, C[:, g], rtol=1e-6, atol=0)
    assert np.array_equal(read_ptc(os.path.join(d, "precursors_4.ptc")).reshape(n, 6) > 0, np.repeat(fuel[:, None], 6, 1))
