"""Full-size workloads (fp 4+4, n = 1,963,461; fp 5+5, n = 18,600,516) checked
through size-independent properties, since the oracle cannot run them in
seconds: basis sizes, the block-tiled product against the row-wise product,
symmetry (x . H y = y . H x, dots accumulated in FP64) and linearity of the
stored and on-the-fly products, the on-the-fly product against the stored
one, the mixed solve's residuals under the FP64 product, and the mixed
solve's 10 eigenpairs against the same solver run entirely in FP64.
Tolerances: 2e-6 of max|y| between the two FP32 stored kernels (same values,
different summation order), 1e-5 for FP32 products against each other or in
linear combinations, 1e-6 relative for the FP32 symmetry defect, 1e-4 MeV per
eigenvalue and 1e-6 per <J-J+> between the mixed and the FP64 solves."""
import numpy as np
import pytest

import cosmo_gb300 as cg
from cosmo_gb300.synthetic import SyntheticSystem, make_system

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _system(tmp, space, nv, zv, seed):
    xml = make_system(str(tmp), SyntheticSystem(space, nv, zv, 0, "+", 0.5, seed))[1]
    p = cg.Problem(xml)
    return p, cg.ManyBodyStates(p)


def _prod(h, x, prec=cg.CG_PREC_FP32):
    y = torch.empty_like(x)
    torch.cuda.synchronize()
    h.spmm_device(x.data_ptr(), x.shape[1], y.data_ptr(), y.shape[1], x.shape[1], prec)
    torch.cuda.synchronize()
    return y


def _sym_defect(h, n, gen):
    x = torch.randn(n, 8, generator=gen, dtype=torch.float32).cuda()
    y = torch.randn(n, 8, generator=gen, dtype=torch.float32).cuda()
    hx, hy = _prod(h, x), _prod(h, y)
    a = (x.double() * hy.double()).sum(0)
    b = (y.double() * hx.double()).sum(0)
    scale = (x.double().norm(dim=0) * hy.double().norm(dim=0))
    return float(((a - b).abs() / scale).max())


def test_fp44_tiled_rows_symmetry_linearity(gpu_available, tmp_path):
    p, b = _system(tmp_path, "fp", 4, 4, 7)
    assert b.n == 1963461
    h = cg.Hamiltonian(p, b, cg.CG_PREC_FP32)
    fi = h.format_info()
    assert fi["tiled_available"] and fi["entries"] >= h.info.nnz_full
    gen = torch.Generator().manual_seed(44)
    x = torch.randn(b.n, 8, generator=gen, dtype=torch.float32).cuda()
    h.set_format(cg.CG_FORMAT_TILED)
    yt = _prod(h, x)
    h.set_format(cg.CG_FORMAT_ROWS)
    yr = _prod(h, x)
    h.set_format(cg.CG_FORMAT_TILED)
    scale = float(yr.abs().max())
    assert float((yt - yr).abs().max()) <= 2e-6 * scale
    # symmetry and linearity of the tiled product at full size
    assert _sym_defect(h, b.n, gen) <= 1e-6
    z = torch.randn(b.n, 8, generator=gen, dtype=torch.float32).cuda()
    lhs = _prod(h, 2 * x + 3 * z)
    rhs = 2 * yt + 3 * _prod(h, z)
    assert float((lhs - rhs).abs().max()) <= 1e-5 * float(rhs.abs().max())
    # the on-the-fly product of the same operator
    hv = cg.Hamiltonian(p, b, cg.CG_PREC_FP32, virtual=True)
    yv = _prod(hv, x)
    assert float((yv - yt).abs().max()) <= 1e-5 * scale


def test_fp55_on_the_fly_symmetry_linearity(gpu_available, tmp_path):
    p, b = _system(tmp_path, "fp", 5, 5, 8)
    assert b.n == 18600516
    hv = cg.Hamiltonian(p, b, cg.CG_PREC_FP32, virtual=True)
    gen = torch.Generator().manual_seed(55)
    assert _sym_defect(hv, b.n, gen) <= 1e-6
    x = torch.randn(b.n, 8, generator=gen, dtype=torch.float32).cuda()
    z = torch.randn(b.n, 8, generator=gen, dtype=torch.float32).cuda()
    lhs = _prod(hv, 2 * x - 0.5 * z)
    rhs = 2 * _prod(hv, x) - 0.5 * _prod(hv, z)
    assert float((lhs - rhs).abs().max()) <= 1e-5 * float(rhs.abs().max())


def test_fp44_mixed_solve_true_residuals(gpu_available, tmp_path):
    """The mixed solve at full size (the benchmark's parameters): the returned
    vectors' residuals under the FP64 on-the-fly product equal the reported
    ones and are <= 1e-5."""
    p, b = _system(tmp_path, "fp", 4, 4, 7)
    h = cg.Hamiltonian(p, b, cg.CG_PREC_FP32)
    r = cg.davidson_diagonalization(h, 10, want_vectors=True, precision=cg.CG_PREC_FP32, tol_resid=1e-5,
                                    block=8, lim=96, keep=32, algorithm=1, precond=1, switch_resid=3e-5,
                                    refine_lim=32, refine_keep=16)
    assert r.stats.converged == 10, (r.resid, r.stats.ierr)
    del h
    hv = cg.Hamiltonian(p, b, cg.CG_PREC_FP64, virtual=True)
    V = r.vecs.T
    res = np.linalg.norm(hv.times_matrix(V, cg.CG_PREC_FP64) - V * r.eig, axis=0)
    assert np.all(res <= 1e-5), res
    np.testing.assert_allclose(res, r.resid, rtol=1e-3, atol=1e-8)


MIXED = dict(precision=cg.CG_PREC_FP32, tol_resid=1e-5, block=8, lim=96, keep=32, algorithm=1, precond=1,
             switch_resid=3e-5, refine_lim=32, refine_keep=16)
FP64_SAME = dict(precision=cg.CG_PREC_FP64, tol_resid=1e-5, block=8, lim=96, keep=32, algorithm=1, precond=1)


def _compare_states(b, rm, r64):
    """Mixed vs FP64 solve, state by state in energy order: eigenvalues within
    1e-4 MeV and <J-J+> within 1e-6 (a missed or swapped state fails)."""
    assert rm.stats.converged == 10 and r64.stats.converged == 10, (rm.resid, r64.resid)
    np.testing.assert_allclose(rm.eig, r64.eig, rtol=0, atol=1e-4)
    jm, _ = cg.jt_expectations(b, rm.vecs)
    j6, _ = cg.jt_expectations(b, r64.vecs)
    np.testing.assert_allclose(jm, j6, rtol=0, atol=1e-6)


def test_fp44_mixed_matches_fp64_solve(gpu_available, tmp_path):
    """The headline workload: the 10 lowest eigenpairs of the mixed solve (FP32
    stored H and vectors) against the same solver run entirely in FP64 (FP64
    stored H) to the same tolerance."""
    p, b = _system(tmp_path, "fp", 4, 4, 7)
    h = cg.Hamiltonian(p, b, cg.CG_PREC_FP32)
    rm = cg.davidson_diagonalization(h, 10, want_vectors=True, **MIXED)
    del h
    h64 = cg.Hamiltonian(p, b, cg.CG_PREC_FP64)
    r64 = cg.davidson_diagonalization(h64, 10, want_vectors=True, **FP64_SAME)
    _compare_states(b, rm, r64)


def test_fp55_mixed_matches_fp64_on_the_fly_solve(gpu_available, tmp_path):
    """fp 5+5 (n = 18,600,516, H never stored): the mixed solve on the FP32
    on-the-fly product against the same solver on the FP64 on-the-fly product
    (about two minutes of FP64 products)."""
    p, b = _system(tmp_path, "fp", 5, 5, 8)
    hv = cg.Hamiltonian(p, b, cg.CG_PREC_FP32, virtual=True)
    rm = cg.davidson_diagonalization(hv, 10, want_vectors=True, **MIXED)
    r64 = cg.davidson_diagonalization(hv, 10, want_vectors=True, **FP64_SAME)
    _compare_states(b, rm, r64)


def test_fp44_fp32_product_accumulation_error(gpu_available, tmp_path):
    """The FP32 products sum in FP32 within a row, across all its tiles (no FP64
    accumulation between tiles): against the FP64-accurate double-float
    product of the same operator the error stays within 5e-6 of max|y| and
    2e-6 in the RMS, for the block-tiled and the row-wise kernel."""
    p, b = _system(tmp_path, "fp", 4, 4, 7)
    h = cg.Hamiltonian(p, b, cg.CG_PREC_FP32)
    gen = torch.Generator().manual_seed(7)
    x = torch.randn(b.n, 8, generator=gen, dtype=torch.float32).cuda()
    ref = torch.empty(b.n, 8, dtype=torch.float64, device="cuda")
    x64 = x.double()
    torch.cuda.synchronize()
    h.spmm_device(x64.data_ptr(), 8, ref.data_ptr(), 8, 8, cg.CG_PREC_REFINE)
    torch.cuda.synchronize()
    scale = float(ref.abs().max())
    for fmt in (cg.CG_FORMAT_TILED, cg.CG_FORMAT_ROWS):
        h.set_format(fmt)
        d = (_prod(h, x).double() - ref)
        assert float(d.abs().max()) <= 5e-6 * scale, fmt
        assert float(d.norm() / ref.norm()) <= 2e-6, fmt
