"""The allocation-free normalisation entry point against the allocating solver path.

pgpu_normalize_power_noalloc serves callers that cannot call cudaMalloc (their device
memory is owned by another allocator, or they must not grow the device footprint after
start-up): they pass device buffers they already hold and the entry point uses a fixed
scratch array compiled into the library.  This file is collected last so that a run
stopping at the first failure has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

import pampa_gb300 as pg

pytestmark = pytest.mark.gpu

REL_TOL = 1e-12  # same arithmetic as the solver's own normalisation, in another order


def _fn():
    f = pg.lib().pgpu_normalize_power_noalloc
    f.restype = C.c_int
    f.argtypes = [C.c_int, C.c_int] + [C.c_void_p] * 5 + [C.c_double, C.c_double] + [C.c_void_p] * 6
    return f


def _rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b)))


def test_noalloc_normalisation_matches_solver_output(tmp_path):
    import torch
    from pampa_gb300 import workloads as wl
    from oracle import pampa_oracle as po

    path = wl.diffusion_2d(str(tmp_path))
    with pg.Pampa(path, "-silent") as p:          # existing path: solve + normalise on the GPU
        p.solve()
        k = p.keff
        phi_ref = p.field("scalar-flux")
        q_ref = p.field("power")
        P_ref = p.field("production-rate")

    prob = po.read_problem(path)                   # reader only: material ids and tables
    st, nsf, ksf, chi, ss, D = po._material_tables(prob)
    n, G = prob.mesh.n, prob.G
    dev = torch.device("cuda", 0)
    mat = torch.tensor(prob.mesh.materials.astype(np.int32), device=dev)
    vol = torch.tensor(prob.mesh.volumes, dtype=torch.float64, device=dev)
    ksf_d = torch.tensor(ksf.reshape(-1), dtype=torch.float64, device=dev)
    nsf_d = torch.tensor(nsf.reshape(-1), dtype=torch.float64, device=dev)
    phi_out = torch.empty(n * G, dtype=torch.float64, device=dev)
    q = torch.empty(n, dtype=torch.float64, device=dev)
    P = torch.empty(n, dtype=torch.float64, device=dev)
    total = torch.zeros(1, dtype=torch.float64, device=dev)
    neg = torch.full((1,), -1, dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    fn = _fn()
    for scale in (3.7, 0.25):                      # two calls in a row share the scratch
        phi_raw = torch.tensor(phi_ref * scale, dtype=torch.float64, device=dev)
        status = fn(n, G, mat.data_ptr(), vol.data_ptr(), ksf_d.data_ptr(), nsf_d.data_ptr(), phi_raw.data_ptr(),
                    1.0, k, phi_out.data_ptr(), q.data_ptr(), P.data_ptr(), total.data_ptr(), neg.data_ptr(), stream)
        assert status == pg.PGPU_OK, pg.last_error()
        torch.cuda.synchronize()
        assert _rel(phi_out.cpu().numpy(), phi_ref) <= REL_TOL
        assert _rel(q.cpu().numpy(), q_ref) <= REL_TOL
        assert _rel(P.cpu().numpy(), P_ref) <= REL_TOL
        assert total.item() == pytest.approx(1.0, rel=REL_TOL)
        assert neg.item() == 0
        # and against the oracle's restatement of the reference's normalisation
        # (NeutronicSolver::normalizeScalarFlux, calculatePowerAndProductionRate)
        phi_o = po.normalize_scalar_flux(prob, phi_ref * scale)
        q_o, P_o, tot_o = po.power_and_production(prob, phi_o, k)
        assert _rel(phi_out.cpu().numpy(), phi_o) <= REL_TOL
        assert _rel(q.cpu().numpy(), q_o) <= REL_TOL
        assert _rel(P.cpu().numpy(), P_o) <= REL_TOL
        assert total.item() == pytest.approx(tot_o, rel=REL_TOL)


def test_noalloc_flux_without_power_is_marked(tmp_path):
    """An all-zero flux has no power to normalise by: the outputs are zeroed and the
    negatives count carries the -1 marker, and the next call on a good flux is clean."""
    import torch
    from pampa_gb300 import workloads as wl
    from oracle import pampa_oracle as po

    prob = po.read_problem(wl.diffusion_2d(str(tmp_path), n=6))
    st, nsf, ksf, chi, ss, D = po._material_tables(prob)
    n, G = prob.mesh.n, prob.G
    dev = torch.device("cuda", 0)
    mat = torch.tensor(prob.mesh.materials.astype(np.int32), device=dev)
    vol = torch.tensor(prob.mesh.volumes, dtype=torch.float64, device=dev)
    ksf_d = torch.tensor(ksf.reshape(-1), dtype=torch.float64, device=dev)
    nsf_d = torch.tensor(nsf.reshape(-1), dtype=torch.float64, device=dev)
    phi_out = torch.full((n * G,), 7.0, dtype=torch.float64, device=dev)
    q = torch.full((n,), 7.0, dtype=torch.float64, device=dev)
    P = torch.full((n,), 7.0, dtype=torch.float64, device=dev)
    total = torch.full((1,), 7.0, dtype=torch.float64, device=dev)
    neg = torch.zeros(1, dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    fn = _fn()
    args = lambda phi: (n, G, mat.data_ptr(), vol.data_ptr(), ksf_d.data_ptr(), nsf_d.data_ptr(),  # noqa: E731
                        phi.data_ptr(), 1.0, 1.0, phi_out.data_ptr(), q.data_ptr(), P.data_ptr(),
                        total.data_ptr(), neg.data_ptr(), stream)
    zero = torch.zeros(n * G, dtype=torch.float64, device=dev)
    assert fn(*args(zero)) == pg.PGPU_OK, pg.last_error()
    torch.cuda.synchronize()
    assert neg.item() == -1
    assert total.item() == 0.0
    assert not phi_out.any() and not q.any() and not P.any()
    ones = torch.ones(n * G, dtype=torch.float64, device=dev)
    assert fn(*args(ones)) == pg.PGPU_OK, pg.last_error()
    torch.cuda.synchronize()
    assert neg.item() == 0
    assert total.item() == pytest.approx(1.0, rel=REL_TOL)


def test_noalloc_rejects_problems_beyond_its_scratch():
    fn = _fn()
    status = fn(1 << 21, 2, 1, 1, 1, 1, 1, 1.0, 1.0, 1, 1, 1, 1, 1, None)  # rejected before any launch
    assert status == pg.PGPU_ERR_INVALID
    assert "scratch capacity" in pg.last_error()
