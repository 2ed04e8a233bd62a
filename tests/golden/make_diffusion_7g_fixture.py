"""Oracle answer for a 7-group diffusion box above the multigrid size threshold.

The oracle's direct solve (SuperLU factor of R + ARPACK on R^-1 F) of a 7-group problem
of 134,400 rows takes minutes on one core, too long for a test run, so its answer is kept
as a fixture: diffusion_7g_40x40x12.npz holds keff, the normalised scalar flux (float32:
its rounding, 6e-8 relative, is far below the tests' 1e-5 bar) and checksums of the
operator the seeded generator builds, so a changed generator is caught before the
comparison.

The problem: pampa_gb300.workloads.diffusion_request(numpy.random.default_rng(SEED), 40,
40, 12, 7, block=4) -- 4 materials of the 7-group family in 4x4x4-cell blocks, every cross
section perturbed by a lognormal factor (sigma_ln = ln 1.05), 2 cm cells, reflective
-x/-y/-z and vacuum +x/+y/+z.  19,200 cells x 7 groups = 134,400 rows, above the 2^17 rows
from which the diffusion solver builds its aggregation V-cycle by default.

Usage: python tests/golden/make_diffusion_7g_fixture.py   (about 3 minutes)
"""
from __future__ import annotations

import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

SEED = 77
SHAPE = (40, 40, 12)
GROUPS = 7
FIXTURE = os.path.join(HERE, "diffusion_7g_40x40x12.npz")


def problem():
    """(operator, materials, layout) of the fixture's problem."""
    from pampa_gb300 import workloads as wl
    nx, ny, nz = SHAPE
    return wl.diffusion_request(np.random.default_rng(SEED), nx, ny, nz, GROUPS, block=4)


def checksums(op: dict) -> np.ndarray:
    """Sums of the operator arrays: diagonal, face couplings, neighbour indices, nu-sigma-f."""
    return np.array([np.sum(op["diag"]), np.sum(op["offdiag"]), float(np.sum(op["neighbors"])),
                     np.sum(op["nu_sigma_f"])], dtype=np.float64)


def main() -> None:
    from oracle import pampa_oracle as po
    from pampa_gb300 import workloads as wl
    op, mats, layout = problem()
    nx, ny, nz = SHAPE
    with tempfile.TemporaryDirectory() as d:
        ref = po.run_input(wl.write_diffusion_input(d, nx, ny, nz, 2.0, layout, mats))
    np.savez_compressed(FIXTURE, keff=np.float64(ref["keff"]), phi=ref["phi"].astype(np.float32),
                        checksums=checksums(op))
    print(f"wrote {FIXTURE}: keff {ref['keff']:.12f}, {ref['phi'].size} flux values")


if __name__ == "__main__":
    main()
