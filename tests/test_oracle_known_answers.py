"""Pin the CPU oracle to the reference's own known answers (test/check_ref.txt).

The reference prints keff with 6 decimals; a restatement that reproduces its algorithm
must print the same digits.  Seven of the nine cases do.  The two 2D SN cases
(pwr-iaea-benchmark/cartesian-sn and unstructured-sn) use the least-squares boundary
gradient, whose 2x2 Gram matrix the reference accumulates into an uninitialised Eigen
matrix (SNSolver.cxx:247-252); in 1D that matrix is 1x1 and the leftover heap word is a
free-list pointer (a denormal, effectively 0), in 2D its other entries are undefined.  The
oracle starts the Gram matrix at zero and lands 4.7 pcm above the printed value; that gap
is asserted here so any other change in the SN operator still shows up.
"""
import os

import numpy as np
import pytest

from conftest import known_answers
from oracle import pampa_oracle as po

EXACT = ["slabs/reflected-diffusion", "slabs/reflected-s2", "slabs/reflected-s4",
         "pwr-iaea-benchmark/cartesian-diffusion", "pwr-iaea-benchmark/unstructured-diffusion",
         "pwr-iaea-benchmark/cartesian-diffusion-3d", "pwr-iaea-benchmark/unstructured-diffusion-3d"]
UB_LS_2D = ["pwr-iaea-benchmark/cartesian-sn", "pwr-iaea-benchmark/unstructured-sn"]


@pytest.mark.parametrize("case", EXACT)
def test_oracle_reproduces_printed_keff(case, case_input):
    ref = known_answers()[case]
    res = po.run_input(case_input(case))
    assert round(res["keff"], 6) == pytest.approx(ref, abs=1e-12), (case, res["keff"], ref)
    assert res["power"] == pytest.approx(1.0, rel=1e-12)
    assert np.all(res["phi"] >= 0.0)


@pytest.mark.parametrize("case", UB_LS_2D)
def test_oracle_2d_ls_sn_gap(case, case_input):
    ref = known_answers()[case]
    res = po.run_input(case_input(case))
    assert res["keff"] - ref == pytest.approx(4.724e-5, abs=2e-7), (case, res["keff"], ref)


@pytest.mark.parametrize("start,gap", [("heap-key-cleared", 2.9e-5), ("heap-key-kept", 0.9e-5)])
def test_heap_models_of_the_uninitialised_gram_matrix(start, gap, case_input, monkeypatch):
    """Starting each boundary cell's Gram matrix from what the allocator leaves there (the
    previous boundary cell's final entries, see pampa_oracle.LS_GRAM_START) moves the
    oracle from 4.7 pcm toward the printed keff of the 2D LS case: 2.9 pcm with glibc's
    list key cleared, 0.9 pcm with it kept.  Not exact: the first boundary cell's chunk
    held values no input determines."""
    case = "pwr-iaea-benchmark/cartesian-sn"
    ref = known_answers()[case]
    monkeypatch.setattr(po, "LS_GRAM_START", start)
    res = po.run_input(case_input(case))
    assert res["keff"] - ref == pytest.approx(gap, abs=1e-6), (start, res["keff"], ref)


def test_cartesian_and_unstructured_meshes_agree(case_input):
    """The PWR geometry written as quads gives the same operator as the Cartesian mesh."""
    a = po.read_problem(case_input("pwr-iaea-benchmark/cartesian-diffusion"))
    b = po.read_problem(case_input("pwr-iaea-benchmark/unstructured-diffusion"))
    Ra, Fa = po.assemble_diffusion(a)
    Rb, Fb = po.assemble_diffusion(b)
    assert Ra.shape == Rb.shape
    assert abs(Ra - Rb).max() < 1e-12
    assert abs(Fa - Fb).max() < 1e-15


def test_reflective_symmetry_matches_full_core(tmp_path):
    """Quarter core with reflective symmetry planes == full core with vacuum (pure upwind,
    no LS), which exercises the reflected-direction mapping of the SN operator."""
    from pampa_gb300 import workloads as wl
    rng = np.random.default_rng(5)
    mats = wl.materials_2g(rng, 2, self_scatter=(0.2, 0.5))
    q = np.array([[[1, 1, 2], [1, 1, 2], [2, 2, 2]]])  # (1, 3, 3) quarter layout
    full = np.concatenate([q[:, ::-1, :], q], axis=1)
    full = np.concatenate([full[:, :, ::-1], full], axis=2)
    out = {}
    for name, lay, bcs in (("quarter", q, {"-x": "reflective", "+x": "vacuum", "-y": "reflective", "+y": "vacuum"}),
                           ("full", full, {"-x": "vacuum", "+x": "vacuum", "-y": "vacuum", "+y": "vacuum"})):
        d = tmp_path / name
        d.mkdir()
        ny, nx = lay.shape[1:]
        wl.write_cartesian_mesh(str(d / "mesh.pmp"), 3.0, nx, ny, 0, lay, bcs)
        for k, m in enumerate(mats):
            wl.write_material(str(d / f"m{k}.pmp"), m, diffusion=False)
        (d / "input.pmp").write_text("mesh cartesian mesh.pmp\nmaterial a m0.pmp\nmaterial b m1.pmp\n"
                                     "solver sn {\n energy-groups 2\n order 4\n mixed-face-interpolation 1.0\n}\n")
        out[name] = po.run_input(str(d / "input.pmp"))["keff"]
    assert out["quarter"] == pytest.approx(out["full"], abs=1e-10)
