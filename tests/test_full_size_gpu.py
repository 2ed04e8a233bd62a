"""The benchmarked workloads at their full sizes, where the oracle's direct solve cannot
run: the 7-group diffusion box of 256x256x128 cells (58.7M unknowns) and the S8 SN
hexagonal-prism lattice of 200x200 hexagons x 40 layers (512M angular unknowns).

Both are checked through a property that holds at any size: the converged pair is an
eigenpair of the operator the drop-in assembled from the input.  R x is applied by the
library's operator (pinned to the oracle's assembled matrix on the reference's inputs,
tests/test_diffusion_gpu.py and tests/test_sn_gpu.py), F x is formed on the host from the
generator's materials (pinned to the oracle's F, tests/test_residual_cpu.py), and

    c = <F'x, Rx> / <F'x, F'x>  must equal V / k,     ||Rx - c F'x|| / ||c F'x||  must be small,

with F'x the fission source without the (uniform) cell volume V.  The mixed-precision
solves are also compared with the FP64 solve of the same operator: |dk| <= 1e-5 (1 pcm)
and flux relative L2 <= 1e-4.  Measured on a GB300 (residual, |c k / V - 1|): 7-group FP64
1.6e-12, 8.7e-13; 7-group mixed 6.0e-12, 3.0e-12 (|dk| vs FP64 1.4e-12, flux L2 1.3e-10);
hexagonal mixed 2.3e-10, 1.1e-11.  The bars below sit at least 30 times above those values.
"""
import ctypes as C
import math

import numpy as np
import pytest

import pampa_gb300 as pg
from helpers import eigen_residual, fission_source, rel_l2, sn_scalar_flux
from oracle import pampa_oracle as po
from pampa_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

K_REL = 1e-9          # |c k / V - 1|
RESIDUAL_DIFF = 2e-10  # ||R x - c F'x|| / ||c F'x||, diffusion
RESIDUAL_SN = 1e-8     # the same, SN (angular space)


def _handle():
    h = C.c_void_p(None)
    err = C.c_int(0)
    pg.lib().pampa_get_problem(C.byref(h), C.byref(err))
    assert err.value == 0, pg.last_error()
    return h


def _solve_handle(h, n_phi, **opts):
    o = pg.default_options(**opts)
    s = pg.pgpu_stats()
    st = pg.lib().pgpu_problem_solve(h, C.byref(o), C.byref(s))
    assert st == pg.PGPU_OK, pg.last_error()
    phi = np.zeros(n_phi)
    assert pg.lib().pgpu_problem_get_scalar_flux(h, phi.ctypes.data_as(C.POINTER(C.c_double))) == pg.PGPU_OK
    return s.keff, phi


def test_seven_group_256x256x128_eigenpair(tmp_path):
    path = wl.diffusion_3d_7g(str(tmp_path))
    mats, layout = wl.diffusion_3d_7g_data()
    V = 2.0 ** 3
    with pg.Pampa(path, "-silent") as p:
        p.solve()
        k64 = p.keff
        phi64 = p.field("scalar-flux")
        c, rel = eigen_residual(p.apply_operator(phi64), fission_source(mats, layout, phi64))
        print(f"7-group FP64: k {k64:.12f} residual {rel:.3e} |ck/V-1| {abs(c * k64 / V - 1):.3e}")
        assert abs(c * k64 / V - 1.0) <= K_REL
        assert rel <= RESIDUAL_DIFF
        km, phim = _solve_handle(_handle(), phi64.size, precision=pg.PGPU_MIXED)
        c, rel = eigen_residual(p.apply_operator(phim), fission_source(mats, layout, phim))
        print(f"7-group mixed: k {km:.12f} |dk| {abs(km - k64):.3e} flux L2 {rel_l2(phim, phi64):.3e} "
              f"residual {rel:.3e} |ck/V-1| {abs(c * km / V - 1):.3e}")
        assert abs(km - k64) <= 1e-5
        assert rel_l2(phim, phi64) <= 1e-4
        assert abs(c * km / V - 1.0) <= K_REL
        assert rel <= RESIDUAL_DIFF


def test_hexagonal_lattice_200x200x40_s8_eigenpair(tmp_path):
    pitch, dz, G = 2.0, 2.0, 4
    path = wl.sn_hex(str(tmp_path), pitch=pitch, dz=dz)
    mats, layout = wl.sn_hex_data()
    V = math.sqrt(3.0) / 2.0 * pitch * pitch * dz
    _, w, _ = po.quadrature(8)
    with pg.Pampa(path, "-silent", "-pgpu_precision", "mixed", "-pgpu_shift", "0.02") as p:
        p.solve()
        k = p.keff
        psi = p.field("angular-flux")
        phi = sn_scalar_flux(psi, w, G)
        assert rel_l2(p.field("scalar-flux"), phi.reshape(-1)) <= 1e-12
        Rpsi = p.apply_operator(psi)
        del psi
        c, rel = eigen_residual(Rpsi, fission_source(mats, layout, phi), w.size)
        print(f"hexagonal S8 mixed: k {k:.12f} residual {rel:.3e} |ck/V-1| {abs(c * k / V - 1):.3e}")
        assert abs(c * k / V - 1.0) <= K_REL
        assert rel <= RESIDUAL_SN
