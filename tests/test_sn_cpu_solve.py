"""The CPU sweep solve (oracle/sn_cpu.py + oracle/cpu_sweep.c) against the oracle's direct
solve.

sn_cpu restates the reference's SN eigen-solve as power iteration with GMRES over
transport sweeps; it is the checker of the GPU result at sizes where the direct solve
(SuperLU + ARPACK on the assembled R and F, pampa_oracle.run_input) cannot run, and the
CPU baseline the bench times.  So it is pinned here first: same k within 1e-6 and same
normalised scalar and angular flux, power and production rate within 1e-5 relative L2, on
Cartesian boxes (reflective -x/-y/-z faces, vacuum +x/+y/+z) and hexagonal-prism lattices
(vacuum, unstructured extruded mesh).
"""
import pytest

from helpers import rel_l2
from oracle import pampa_oracle as po, sn_cpu

K_TOL = 1e-6
FLUX_TOL = 1e-5


def _check(path):
    ref = po.run_input(path)
    cpu = sn_cpu.solve_input(path, threads=2)
    assert abs(cpu["keff"] - ref["keff"]) <= K_TOL, (cpu["keff"], ref["keff"])
    for key in ("phi", "psi", "q", "P"):
        assert rel_l2(cpu[key], ref[key]) <= FLUX_TOL, key
    assert cpu["power"] == pytest.approx(1.0, rel=1e-12)
    return cpu


@pytest.mark.parametrize("shape,order", [((6, 6, 4), 4), ((16, 8, 4), 2), ((8, 8, 4), 4)])
def test_cpu_sweep_solve_cartesian(shape, order, tmp_path):
    from pampa_gb300 import workloads as wl
    nx, ny, nz = shape
    _check(wl.sn_3d(str(tmp_path), nx=nx, ny=ny, nz=nz, order=order, block=2))


@pytest.mark.parametrize("nq,nr,nz,order", [(5, 4, 3, 2), (5, 4, 3, 4)])
def test_cpu_sweep_solve_hex_lattice(nq, nr, nz, order, tmp_path):
    from pampa_gb300 import workloads as wl
    _check(wl.sn_hex(str(tmp_path), nq=nq, nr=nr, nz=nz, order=order, block=2))


def test_cpu_sweep_solve_does_not_depend_on_threads(tmp_path):
    """Threads own whole (group, pattern) sweeps; only the order of the GMRES sums changes
    with the thread count, so the answers agree to rounding."""
    from pampa_gb300 import workloads as wl
    path = wl.sn_3d(str(tmp_path), nx=8, ny=8, nz=4, order=4, block=2)
    a = sn_cpu.solve_input(path, threads=1)
    b = sn_cpu.solve_input(path, threads=3)
    assert abs(a["keff"] - b["keff"]) <= 1e-12
    assert rel_l2(a["phi"], b["phi"]) <= 1e-10


def test_cpu_sweep_rejects_operators_it_cannot_sweep(tmp_path):
    from pampa_gb300 import workloads as wl
    path = wl.sn_3d(str(tmp_path), nx=4, ny=4, nz=4, order=2, block=2)
    text = open(path).read().replace("mixed-face-interpolation 1.0", "mixed-face-interpolation 0.5")
    open(path, "w").write(text)
    with pytest.raises(ValueError, match="mixed-face-interpolation 1.0"):
        sn_cpu.SNCpu(po.read_problem(path))
