"""Diffusion coupled to the delayed-neutron precursors (CouplingSolver + PrecursorSolver)
through the drop-in driver, steady state and transient steps, against the oracle.

The input defines `solver diffusion`, `solver precursors` and `solver coupled main` with
implicit coupling (CouplingSolver.cxx:77-145): every step iterates diffusion solve ->
production rate -> precursor update -> delayed source -> diffusion solve until the
convergence errors of the exchanged fields fall below their tolerances (1e-10 relative
2-norm here).  The oracle restates the same fixed point with direct solves
(pampa_oracle.run_coupled_transient).  Bars: k within 1e-6, fields within 1e-7 relative L2.
"""
import os

import pytest

import pampa_gb300 as pg
from helpers import rel_l2
from oracle import pampa_oracle as po

pytestmark = pytest.mark.gpu

TOL = 1e-7


def _coupled_input(case_input, steps, dt, tol="1e-10"):
    path = case_input("pwr-iaea-benchmark/cartesian-diffusion")
    d = os.path.dirname(path)
    mats = "\n".join(f"material {m} ../materials/{m}.pmp" for m in ("fuel1", "fuel2", "fuel2+rod", "reflector"))
    text = f"""mesh cartesian mesh.pmp
{mats}
solver diffusion {{
   energy-groups 2
   convergence power 2 1 {tol}
   convergence production-rate 2 1 {tol}
}}
solver precursors {{
   precursor-groups 6
   convergence precursors 2 1 {tol}
   convergence delayed-source 2 1 {tol}
}}
solver coupled main {{
   coupled-solvers 2 diffusion precursors
   implicit 1
}}
dt -{steps}
{dt}
"""
    coupled = os.path.join(d, "coupled.pmp")
    with open(coupled, "w") as fh:
        fh.write(text)
    # the oracle reads the diffusion part of the same problem
    plain = os.path.join(d, "plain.pmp")
    with open(plain, "w") as fh:
        fh.write(text.split("solver precursors")[0] + f"dt -{steps}\n{dt}\n")
    return coupled, plain


@pytest.mark.parametrize("scale", [1.0, 0.5])
def test_coupled_precursors_transient_matches_oracle(scale, case_input):
    """Unperturbed, the precursors stay in equilibrium and the power at 1; with the
    precursor populations halved after the steady state the delayed source drops and so
    does the power."""
    coupled, plain = _coupled_input(case_input, 3, 0.05)
    ref = po.run_coupled_transient(po.read_problem(plain), 6, precursor_scale=scale)
    with pg.Pampa(coupled, "-silent") as p:
        p.solve()
        assert abs(p.keff - ref[0]["keff"]) <= 1e-6
        assert rel_l2(p.field("precursors"), ref[0]["C"].reshape(-1)) <= TOL
        if scale != 1.0:
            p.set_field("precursors", p.field("precursors") * scale)
        t = 0.0
        for n, dt in enumerate(p.dt, start=1):
            t += dt
            p.solve(n, dt, t)
            r = ref[n]
            assert rel_l2(p.field("scalar-flux"), r["phi"]) <= TOL
            assert rel_l2(p.field("power"), r["q"]) <= TOL
            assert rel_l2(p.field("precursors"), r["C"].reshape(-1)) <= TOL
            assert rel_l2(p.field("delayed-source"), r["S"]) <= TOL
            assert p.field("power").sum() == pytest.approx(r["power"], rel=1e-8)
            if scale == 1.0:   # precursors in equilibrium keep the power at the steady state
                assert r["power"] == pytest.approx(1.0, rel=1e-8)
        if scale != 1.0:
            assert ref[-1]["power"] < 0.99
