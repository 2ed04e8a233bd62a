"""The in-memory diffusion operator generator (serving requests) against the oracle's
assembly of the same problem written as .pmp files: the arrays must be identical."""
import numpy as np
import pytest

from helpers import diffusion_operator_from_oracle
from oracle import pampa_oracle as po
from pampa_gb300 import workloads as wl


@pytest.mark.parametrize("shape,G", [((6, 5, 4), 2), ((5, 4, 3), 4), ((4, 4, 4), 7)])
def test_generated_operator_equals_oracle_assembly(shape, G, tmp_path):
    rng = np.random.default_rng(7 + G)
    nx, ny, nz = shape
    op, mats, layout = wl.diffusion_request(rng, nx, ny, nz, G, block=2)
    path = wl.write_diffusion_input(str(tmp_path), nx, ny, nz, 2.0, layout, mats)
    prob = po.read_problem(path)
    R, _ = po.assemble_diffusion(prob)
    ref = diffusion_operator_from_oracle(prob, R)
    for key in ("neighbors", "materials"):
        assert np.array_equal(np.asarray(op[key]), np.asarray(ref[key])), key
    for key in ("diag", "offdiag", "volumes", "sigma_s", "chi", "nu_sigma_f", "kappa_sigma_f"):
        assert np.array_equal(np.asarray(op[key], float), np.asarray(ref[key], float)), key


def test_diffusion_7g_fixture_matches_its_generator():
    """The kept oracle answer of the 7-group 40x40x12 box (used by the GPU multigrid test)
    belongs to the operator the seeded generator builds today, and its flux is normalised
    as the oracle normalises (positive, finite)."""
    import os
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
    import make_diffusion_7g_fixture as fx
    fix = np.load(fx.FIXTURE)
    op, _, _ = fx.problem()
    assert np.allclose(fx.checksums(op), fix["checksums"], rtol=1e-12, atol=0)
    phi = fix["phi"]
    assert phi.size == 40 * 40 * 12 * 7 and np.all(np.isfinite(phi)) and phi.min() >= 0
    assert 0.3 < float(fix["keff"]) < 1.5
