"""GPU parity of the discrete-ordinates k-eigenvalue path against the CPU oracle.

Bars as for diffusion: |k_gpu - k_oracle| <= 1e-6 and relative L2 of the normalised
scalar and angular flux <= 1e-5 (FP64); mixed precision within 1 pcm and 1e-4.
"""
import numpy as np
import pytest

import pampa_gb300 as pg
from conftest import known_answers
from helpers import rel_l2
from oracle import pampa_oracle as po

pytestmark = pytest.mark.gpu

K_TOL = 1e-6
FLUX_TOL = 1e-5

KNOWN = ["slabs/reflected-s2", "slabs/reflected-s4", "pwr-iaea-benchmark/cartesian-sn",
         "pwr-iaea-benchmark/unstructured-sn"]


@pytest.mark.parametrize("case", ["slabs/reflected-s4", "pwr-iaea-benchmark/unstructured-sn"])
def test_sn_operator_matches_oracle_matrix(case, case_input):
    path = case_input(case)
    prob = po.read_problem(path)
    R, F, w = po.assemble_sn(prob)
    rng = np.random.default_rng(1)
    with pg.Pampa(path, "-silent") as p:
        for _ in range(2):
            x = rng.standard_normal(R.shape[0])
            assert rel_l2(p.apply_operator(x), R @ x) <= 1e-13


@pytest.mark.parametrize("case", KNOWN)
def test_dropin_sn_known_answers(case, case_input):
    path = case_input(case)
    ref = po.run_input(path)
    with pg.Pampa(path, "-silent") as p:
        p.solve()
        k = p.keff
        phi = p.field("scalar-flux")
        psi = p.field("angular-flux")
        q = p.field("power")
    assert abs(k - ref["keff"]) <= K_TOL, (k, ref["keff"])
    if case.startswith("slabs"):
        assert round(k, 6) == pytest.approx(known_answers()[case], abs=1e-12)
    assert rel_l2(phi, ref["phi"]) <= FLUX_TOL
    assert rel_l2(psi, ref["psi"]) <= FLUX_TOL
    assert q.sum() == pytest.approx(1.0, rel=1e-12)


@pytest.mark.parametrize("shape,order", [((6, 6, 4), 4), ((4, 4, 3), 8),     # level-set sweeps
                                         ((4, 4, 4), 8), ((12, 8, 8), 2),    # dataflow, 4x4x4 tiles
                                         ((8, 8, 4), 4), ((16, 8, 4), 4),    # dataflow, 8x8x4 tiles
                                         ((16, 16, 8), 2)])
def test_synthetic_sn_3d_reflective(shape, order, tmp_path):
    from pampa_gb300 import workloads as wl
    nx, ny, nz = shape
    path = wl.sn_3d(str(tmp_path), nx=nx, ny=ny, nz=nz, order=order, block=2)
    ref = po.run_input(path)
    with pg.Pampa(path, "-silent") as p:
        p.solve()
        assert abs(p.keff - ref["keff"]) <= K_TOL, (p.keff, ref["keff"])
        assert rel_l2(p.field("scalar-flux"), ref["phi"]) <= FLUX_TOL
        assert rel_l2(p.field("angular-flux"), ref["psi"]) <= FLUX_TOL


def test_sn_mixed_precision_within_one_pcm(tmp_path):
    from pampa_gb300 import workloads as wl
    path = wl.sn_3d(str(tmp_path), nx=6, ny=6, nz=4, order=4, block=2)
    ref = po.run_input(path)
    with pg.Pampa(path, "-silent", "-pgpu_precision", "mixed") as p:
        p.solve()
        assert abs(p.keff - ref["keff"]) <= 1e-5
        assert rel_l2(p.field("scalar-flux"), ref["phi"]) <= 1e-4


def _with_delta(path: str, delta: str) -> str:
    text = open(path).read().replace("mixed-face-interpolation 1.0", f"mixed-face-interpolation {delta}")
    with open(path, "w") as fh:
        fh.write(text)
    return path


def test_sn_linear_face_interpolation_angular_space(tmp_path):
    """mixed-face-interpolation < 1 couples downwind cells: the angular-space GMRES path
    must still reproduce the reference operator's eigenpair."""
    from pampa_gb300 import workloads as wl
    path = _with_delta(wl.sn_3d(str(tmp_path), nx=5, ny=4, nz=3, order=2, block=2, cell=6.0), "0.5")
    ref = po.run_input(path)
    with pg.Pampa(path, "-silent") as p:
        p.solve()
        assert abs(p.keff - ref["keff"]) <= K_TOL, (p.keff, ref["keff"])
        assert rel_l2(p.field("scalar-flux"), ref["phi"]) <= FLUX_TOL
        assert rel_l2(p.field("angular-flux"), ref["psi"]) <= FLUX_TOL


def test_sn_default_delta_negative_flux_is_an_error(tmp_path, capfd):
    """With the default mixed-face-interpolation (0.1) this coarse mesh gives negative
    angular flux; the reference stops with an error (SNSolver.cxx:329) and so must we."""
    from pampa_gb300 import workloads as wl
    path = _with_delta(wl.sn_3d(str(tmp_path), nx=5, ny=4, nz=3, order=2, block=2), "0.1")
    with pytest.raises(ValueError, match="negative"):
        po.run_input(path)
    with pg.Pampa(path, "-silent") as p:
        with pytest.raises(pg.PampaError, match="negative"):
            p.solve()


@pytest.mark.parametrize("nq,nr,nz,order", [(5, 4, 3, 2), (5, 4, 3, 4), (3, 2, 2, 8)])
def test_hex_prism_lattice(nq, nr, nz, order, tmp_path):
    """Unstructured extruded hexagonal prisms (level-set sweeps over 8-face cells)."""
    from pampa_gb300 import workloads as wl
    path = wl.sn_hex(str(tmp_path), nq=nq, nr=nr, nz=nz, order=order, block=2)
    ref = po.run_input(path)
    with pg.Pampa(path, "-silent") as p:
        p.solve()
        assert abs(p.keff - ref["keff"]) <= K_TOL, (p.keff, ref["keff"])
        assert rel_l2(p.field("scalar-flux"), ref["phi"]) <= FLUX_TOL
        assert rel_l2(p.field("angular-flux"), ref["psi"]) <= FLUX_TOL


@pytest.mark.parametrize("precision,k_tol,flux_tol", [("fp64", K_TOL, FLUX_TOL), ("mixed", 1e-5, 1e-4)])
def test_benchmark_box_full_size_against_cpu_solve(precision, k_tol, flux_tol, tmp_path):
    """The bench's default workload at its full size (S8, 2 groups, 64x64x32 cells, 21M
    angular unknowns, dataflow sweeps of 8x8x4 tiles) against the CPU sweep solve of
    oracle/sn_cpu.py, which the CPU tests pin to the oracle's direct solve."""
    from pampa_gb300 import workloads as wl
    from oracle import sn_cpu
    path = wl.sn_3d(str(tmp_path))
    ref = sn_cpu.solve_input(path)
    with pg.Pampa(path, "-silent", "-pgpu_precision", precision) as p:
        p.solve()
        assert abs(p.keff - ref["keff"]) <= k_tol, (p.keff, ref["keff"])
        assert rel_l2(p.field("scalar-flux"), ref["phi"]) <= flux_tol
        assert rel_l2(p.field("angular-flux"), ref["psi"]) <= flux_tol


@pytest.mark.parametrize("precision,k_tol,flux_tol", [("fp64", K_TOL, FLUX_TOL), ("mixed", 1e-5, 1e-4)])
def test_hex_lattice_40x40x8_s8_against_cpu_solve(precision, k_tol, flux_tol, tmp_path):
    """The hexagonal-prism workload's family at 40x40 hexagons x 8 layers, S8, 4 groups
    (4.1M angular unknowns, level-set sweeps), against the CPU sweep solve."""
    from pampa_gb300 import workloads as wl
    from oracle import sn_cpu
    path = wl.sn_hex(str(tmp_path), nq=40, nr=40, nz=8, order=8, block=10)
    ref = sn_cpu.solve_input(path)
    with pg.Pampa(path, "-silent", "-pgpu_precision", precision, "-pgpu_shift", "0.02") as p:
        p.solve()
        assert abs(p.keff - ref["keff"]) <= k_tol, (p.keff, ref["keff"])
        assert rel_l2(p.field("scalar-flux"), ref["phi"]) <= flux_tol
        assert rel_l2(p.field("angular-flux"), ref["psi"]) <= flux_tol


@pytest.mark.parametrize("shape", [(6, 5, 4), (10, 6, 5)])
def test_column_sweep_equals_level_sweep(shape, tmp_path, monkeypatch):
    """Boxes whose sides are not multiples of 4 are swept by columns (a warp per column,
    pattern and group chunk); the level-set sweep (PGPU_SWEEP_COLUMNS=0) computes the same
    updates in the same order, so both give the same eigenpair."""
    from pampa_gb300 import workloads as wl
    nx, ny, nz = shape
    path = wl.sn_3d(str(tmp_path), nx=nx, ny=ny, nz=nz, order=4, block=2)
    out = {}
    for mode in ("1", "0"):
        monkeypatch.setenv("PGPU_SWEEP_COLUMNS", mode)
        with pg.Pampa(path, "-silent") as p:
            p.solve()
            out[mode] = (p.keff, p.field("scalar-flux"), p.field("angular-flux"))
    assert abs(out["1"][0] - out["0"][0]) <= 1e-10
    assert rel_l2(out["1"][1], out["0"][1]) <= 1e-9
    assert rel_l2(out["1"][2], out["0"][2]) <= 1e-9


def test_hex_lattice_column_sweep_equals_level_sweep(tmp_path, monkeypatch):
    """A hexagonal-prism lattice is swept by pipelined columns; the level-set sweep
    (PGPU_SWEEP_COLUMNS=0) makes the same updates in the same order."""
    from pampa_gb300 import workloads as wl
    path = wl.sn_hex(str(tmp_path), nq=12, nr=10, nz=9, order=4, block=3)
    out = {}
    for mode in ("1", "0"):
        monkeypatch.setenv("PGPU_SWEEP_COLUMNS", mode)
        with pg.Pampa(path, "-silent", "-pgpu_precision", "mixed") as p:
            p.solve()
            out[mode] = (p.keff, p.field("scalar-flux"))
    assert abs(out["1"][0] - out["0"][0]) <= 1e-9
    assert rel_l2(out["1"][1], out["0"][1]) <= 1e-8
