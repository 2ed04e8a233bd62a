"""Aggregation multigrid (V-cycle) preconditioner of the diffusion inner solves: the same
eigenpair as the oracle, and far fewer inner iterations than the cell preconditioner alone.

PGPU_DIFF_MG=1 builds the hierarchy at any size (by default only operators of at least
2^17 rows get one) and PGPU_DIFF_MG=0 turns it off; the variable is read when a problem is
created.  Bars as for the other diffusion tests: FP64 |dk| <= 1e-6 and flux relative L2
<= 1e-5 against the oracle; mixed precision 1e-5 and 1e-4.
"""
import os
import sys

import numpy as np
import pytest

import pampa_gb300 as pg
from conftest import known_answers
from helpers import rel_l2
from oracle import pampa_oracle as po
from pampa_gb300 import workloads as wl

pytestmark = pytest.mark.gpu


def _tols(precision):
    return (1e-6, 1e-5) if precision == pg.PGPU_FP64 else (1e-5, 1e-4)


@pytest.mark.parametrize("G,precision,shape", [(2, pg.PGPU_FP64, (12, 10, 6)), (4, pg.PGPU_MIXED, (9, 7, 5)),
                                               (7, pg.PGPU_FP64, (12, 10, 6)), (7, pg.PGPU_MIXED, (16, 12, 8))])
def test_vcycle_solve_matches_oracle(G, precision, shape, tmp_path, monkeypatch):
    """Boxes with odd sides (aggregates of 1 to 8 cells) and every supported G."""
    monkeypatch.setenv("PGPU_DIFF_MG", "1")
    rng = np.random.default_rng(30 + G)
    nx, ny, nz = shape
    op, mats, layout = wl.diffusion_request(rng, nx, ny, nz, G, block=2)
    with pg.DiffusionProblem(**op) as dp:
        res = dp.solve(precision=precision)
        phi = dp.scalar_flux()
        again = dp.solve(precision=precision)
        assert again.keff == res.keff and np.array_equal(dp.scalar_flux(), phi)  # deterministic
    ref = po.run_input(wl.write_diffusion_input(str(tmp_path), nx, ny, nz, 2.0, layout, mats))
    k_tol, f_tol = _tols(precision)
    assert abs(res.keff - ref["keff"]) <= k_tol, (res.keff, ref["keff"])
    assert rel_l2(phi, ref["phi"]) <= f_tol


def test_vcycle_cuts_inner_iterations(monkeypatch):
    """7-group box of 24x24x12 cells: the V-cycle needs well under half the BiCGStab
    iterations of the cell preconditioner, for the same k."""
    rng = np.random.default_rng(5)
    op, _, _ = wl.diffusion_request(rng, 24, 24, 12, 7, block=4)
    out = {}
    for mg in ("0", "1"):
        monkeypatch.setenv("PGPU_DIFF_MG", mg)
        with pg.DiffusionProblem(**op) as dp:
            out[mg] = dp.solve(precision=pg.PGPU_FP64)
    assert abs(out["0"].keff - out["1"].keff) <= 1e-8
    assert out["1"].stats["inner_iterations"] * 2 < out["0"].stats["inner_iterations"], \
        (out["1"].stats["inner_iterations"], out["0"].stats["inner_iterations"])


@pytest.mark.parametrize("case", ["pwr-iaea-benchmark/unstructured-diffusion-3d",
                                  "pwr-iaea-benchmark/cartesian-diffusion-3d"])
def test_vcycle_through_the_drop_in(case, case_input, monkeypatch):
    """The reference's 3D IAEA inputs (one unstructured mesh: aggregates of prism cells)
    solved through the drop-in API with the hierarchy forced on."""
    monkeypatch.setenv("PGPU_DIFF_MG", "1")
    path = case_input(case)
    ref = po.run_input(path)
    with pg.Pampa(path, "-silent") as p:
        p.solve()
        assert abs(p.keff - ref["keff"]) <= 1e-6, (p.keff, ref["keff"])
        assert round(p.keff, 6) == pytest.approx(known_answers()[case], abs=1e-12)
        assert rel_l2(p.field("scalar-flux"), ref["phi"]) <= 1e-5


def test_vcycle_linear_solve(monkeypatch):
    """The transient step's linear solve (R - lam F) x = b with the hierarchy combined for
    lam (0.3, well below the fundamental 1/k): same solution as with the cell
    preconditioner alone."""
    rng = np.random.default_rng(8)
    op, _, _ = wl.diffusion_request(rng, 14, 12, 8, 7, block=2)
    b = rng.random(14 * 12 * 8 * 7)
    xs = {}
    for mg in ("0", "1"):
        monkeypatch.setenv("PGPU_DIFF_MG", mg)
        with pg.DiffusionProblem(**op) as dp:
            xs[mg], _ = dp.solve_linear(0.3, b, tol_flux=1e-12)
    assert rel_l2(xs["1"], xs["0"]) <= 1e-10


@pytest.mark.parametrize("precision", [pg.PGPU_FP64, pg.PGPU_MIXED])
def test_default_size_threshold_box_against_oracle_fixture(precision, monkeypatch):
    """A 7-group box of 40x40x12 cells (134,400 rows, above the 2^17 rows from which the
    solver builds the V-cycle by itself) against the oracle's direct solve, kept as a
    fixture (tests/golden/make_diffusion_7g_fixture.py: the direct solve takes minutes).
    The default path (V-cycle) and the cell preconditioner alone both reach the oracle's
    eigenpair, and the default path takes far fewer inner iterations."""
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
    import make_diffusion_7g_fixture as fx
    fix = np.load(fx.FIXTURE)
    op, _, _ = fx.problem()
    assert np.allclose(fx.checksums(op), fix["checksums"], rtol=1e-12, atol=0), "generator changed"
    k_tol, f_tol = _tols(precision)
    out = {}
    for mg in (None, "0"):
        if mg is None:
            monkeypatch.delenv("PGPU_DIFF_MG", raising=False)
        else:
            monkeypatch.setenv("PGPU_DIFF_MG", mg)
        with pg.DiffusionProblem(**op) as dp:
            res = dp.solve(precision=precision)
            phi = dp.scalar_flux()
        assert abs(res.keff - float(fix["keff"])) <= k_tol, (mg, res.keff, float(fix["keff"]))
        assert rel_l2(phi, fix["phi"]) <= f_tol, mg
        out[mg] = res.stats["inner_iterations"]
    assert out[None] * 2 < out["0"], out
