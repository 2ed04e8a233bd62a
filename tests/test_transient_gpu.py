"""Transient steps n > 0 of the diffusion solver on the GPU against the oracle.

The reference's DiffusionSolver assembles, for a time step of size dt, R with the
1/(v dt) terms on its diagonal and -(1 - beta) chi_p nu_sigma_f V / keff in each cell's
group block, and b = chi_d S + V/(v dt) phi0 (DiffusionSolver.cxx:108-175), then solves
R phi = b with KSP (petsc.cxx:147-172).  The GPU path solves the same system with
BiCGStab under FP64 residual refinement (pgpu_problem_solve_linear); the oracle solves
it directly (pampa_oracle.run_transient).  Bars: relative L2 of the flux and of the power
and production-rate fields <= 1e-7 (the linear solve stops at a relative residual of
1e-9), total power to 1e-9.
"""
import numpy as np
import pytest

import pampa_gb300 as pg
from helpers import diffusion_operator_from_oracle, rel_l2
from oracle import pampa_oracle as po

pytestmark = pytest.mark.gpu

FLUX_TOL = 1e-7


def _with_steps(path: str, steps: int, dt: float) -> str:
    with open(path, "a") as fh:
        fh.write(f"\ndt -{steps}\n{dt}\n")
    return path


def _run(path, scale):
    out = []
    with pg.Pampa(path, "-silent") as p:
        p.solve()
        if scale != 1.0:
            p.set_field("delayed-source", p.field("delayed-source") * scale)
        out.append(dict(keff=p.keff, phi=p.field("scalar-flux"), q=p.field("power")))
        t = 0.0
        for n, dt in enumerate(p.dt, start=1):
            t += dt
            p.solve(n, dt, t)
            out.append(dict(phi=p.field("scalar-flux"), q=p.field("power"), P=p.field("production-rate")))
    return out


@pytest.mark.parametrize("scale", [1.0, 0.5])
def test_transient_steps_match_oracle(scale, case_input):
    """Steady state then three steps of 10 ms on the 2D PWR benchmark geometry; with the
    delayed source scaled by 0.5 the power falls, unscaled it stays at the steady state."""
    path = _with_steps(case_input("pwr-iaea-benchmark/cartesian-diffusion"), 3, 0.01)
    ref = po.run_transient(path, delayed_source_scale=scale)
    got = _run(path, scale)
    assert len(got) == len(ref) == 4
    assert abs(got[0]["keff"] - ref[0]["keff"]) <= 1e-6
    for g, r in zip(got[1:], ref[1:]):
        assert rel_l2(g["phi"], r["phi"]) <= FLUX_TOL
        assert rel_l2(g["q"], r["q"]) <= FLUX_TOL
        assert rel_l2(g["P"], r["P"]) <= FLUX_TOL
        assert g["q"].sum() == pytest.approx(r["power"], rel=1e-9)
    if scale == 1.0:
        assert all(g["q"].sum() == pytest.approx(1.0, rel=1e-9) for g in got[1:])
    else:
        assert got[-1]["q"].sum() < 0.999


@pytest.mark.parametrize("precision", [pg.PGPU_FP64, pg.PGPU_MIXED])
def test_linear_solve_entry_point(precision, case_input):
    """pgpu_problem_solve_linear: (R - lam F) x = b against a direct solve, both precisions."""
    prob = po.read_problem(case_input("pwr-iaea-benchmark/unstructured-diffusion"))
    R, F = po.assemble_diffusion(prob)
    import scipy.sparse.linalg as spla
    rng = np.random.default_rng(3)
    b = rng.random(R.shape[0])
    lam = 0.9
    x_ref = spla.spsolve((R - lam * F).tocsc(), b)
    with pg.DiffusionProblem(**diffusion_operator_from_oracle(prob, R)) as dp:
        x, stats = dp.solve_linear(lam, b, precision=precision, tol_flux=1e-11)
        assert rel_l2(x, x_ref) <= 1e-8
        assert stats["residual"] <= 1e-11
        # from the solution as the initial guess nothing is left to do
        x2, stats2 = dp.solve_linear(lam, b, x0=x, precision=precision, tol_flux=1e-11)
        assert stats2["inner_iterations"] == 0
        assert np.array_equal(x2, x)


def test_transient_needs_the_steady_state_first(case_input, capfd):
    path = _with_steps(case_input("pwr-iaea-benchmark/cartesian-diffusion"), 1, 0.01)
    with pg.Pampa(path, "-silent") as p:
        with pytest.raises(pg.PampaError):
            p.solve(1, 0.01, 0.01)
    assert "the steady state must be solved before a transient step" in capfd.readouterr().out


def test_transient_input_without_velocities_is_rejected(case_input):
    """ConstantNuclearData::check(G, diffusion, transient) (ConstantNuclearData.cxx:180-200)
    wants neutron velocities and both fission spectra when the input has time steps; the
    slab materials have no velocities, so initialisation fails as in the reference."""
    path = _with_steps(case_input("slabs/reflected-diffusion"), 1, 0.01)
    with pytest.raises(pg.PampaError, match="pampa_initialize"):
        pg.Pampa(path, "-silent")


def test_sn_time_step_fails_as_in_the_reference(case_input):
    """The reference's SN step solves its angular-flux system into the scalar-flux vector
    (SNSolver.cxx:658-666), which PETSc rejects; the drop-in reports the same failure
    after a normal steady state."""
    path = _with_steps(case_input("pwr-iaea-benchmark/cartesian-sn"), 1, 0.01)
    with pg.Pampa(path, "-silent") as p:
        p.solve()
        assert p.keff > 0.0
        with pytest.raises(pg.PampaError, match="pampa_solve failed"):
            p.solve(1, 0.01, 0.01)
