"""Allocation-free refinement product (cg_spmm_refine_static), called through
the C ABI, against the allocating entry points on the same inputs: the host
product cg_spmm (same double-float kernels, staging area allocated per call)
and the device product cg_spmm_device, both with CG_PREC_REFINE.  Tolerance:
1e-11 of max |y| (FP64-accurate products, as in the SpMM parity tests).

This file is collected last so that the static staging area is exercised after
every other GPU test; it also passes alone in a fresh process."""
import ctypes as C

import numpy as np
import pytest

import cosmo_gb300 as cg
from conftest import problem_for

pytestmark = pytest.mark.gpu

TOL = 1e-11


def _fp32_hamiltonian(p):
    b = cg.ManyBodyStates(p)
    return cg.Hamiltonian(p, b, cg.CG_PREC_FP32)


def _static(h, xd, ldx, yd, ldy, m) -> int:
    return cg.lib().cg_spmm_refine_static(h._h, C.c_void_p(xd.data_ptr()), ldx, C.c_void_p(yd.data_ptr()), ldy, m)


def test_static_refine_matches_allocating_entry_points(gpu_available, tmp_path):
    import torch
    rows = C.c_uint64()
    assert cg.lib().cg_spmm_refine_static_max_rows(C.byref(rows)) == cg.CG_OK
    h = _fp32_hamiltonian(problem_for("sd66m0s5", str(tmp_path)))  # n = 93,710
    n = h.n
    assert n <= rows.value
    rng = np.random.default_rng(2026)
    dev = torch.device("cuda", 0)
    # two calls in a row with different inputs and widths (one and two
    # 8-column staging blocks); the second must not see the first's staging
    for m, ld in ((8, 8), (11, 12)):
        x = rng.standard_normal((n, m))
        xr = np.zeros((n, ld))
        xr[:, :m] = x
        xd = torch.from_numpy(xr).to(dev)
        yd = torch.full((n, ld), float("nan"), dtype=torch.float64, device=dev)
        torch.cuda.synchronize()
        st = _static(h, xd, ld, yd, ld, m)
        assert st == cg.CG_OK, cg.lib().cg_last_error()
        torch.cuda.synchronize()
        y = yd.cpu().numpy()[:, :m]
        # allocating host entry point: the same double-float kernels
        y_host = h.times_matrix(x, cg.CG_PREC_REFINE)
        scale = np.abs(y_host).max()
        np.testing.assert_allclose(y, y_host, rtol=0, atol=TOL * scale)
        # allocating device entry point
        yd2 = torch.zeros((n, ld), dtype=torch.float64, device=dev)
        h.spmm_device(xd.data_ptr(), ld, yd2.data_ptr(), ld, m, cg.CG_PREC_REFINE)
        torch.cuda.synchronize()
        np.testing.assert_allclose(y, yd2.cpu().numpy()[:, :m], rtol=0, atol=TOL * scale)
        # columns beyond m are left alone
        assert np.isnan(yd.cpu().numpy()[:, m:]).all()


def test_static_refine_rejects_bad_calls(gpu_available, tmp_path):
    import torch
    from cosmo_gb300.synthetic import SyntheticSystem, make_system
    dev = torch.device("cuda", 0)
    rows = C.c_uint64()
    assert cg.lib().cg_spmm_refine_static_max_rows(C.byref(rows)) == cg.CG_OK
    # fp-shell 3p+4n, 2M = 1, negative parity: 483,887 rows, beyond the static staging area
    xml = make_system(str(tmp_path), SyntheticSystem("fp", 4, 3, 1, "-", 0.5, 3))[1]
    big = _fp32_hamiltonian(cg.Problem(xml))
    assert big.n > rows.value
    xd = torch.zeros((big.n, 1), dtype=torch.float64, device=dev)
    yd = torch.zeros((big.n, 1), dtype=torch.float64, device=dev)
    assert _static(big, xd, 1, yd, 1, 1) == cg.CG_ERR_ARG
    assert b"static staging area" in cg.lib().cg_last_error()
    del big
    # vector count and matrix precision
    small = _fp32_hamiltonian(problem_for("sd22m0s1", str(tmp_path)))
    xs = torch.zeros((small.n, 17), dtype=torch.float64, device=dev)
    ys = torch.zeros((small.n, 17), dtype=torch.float64, device=dev)
    assert _static(small, xs, 17, ys, 17, 17) == cg.CG_ERR_ARG
    assert _static(small, xs, 17, ys, 17, 0) == cg.CG_ERR_ARG
    p = problem_for("sd22m0s1", str(tmp_path))
    h64 = cg.Hamiltonian(p, cg.ManyBodyStates(p), cg.CG_PREC_FP64)
    assert _static(h64, xs, 17, ys, 17, 4) == cg.CG_ERR_ARG
    # a rejected call leaves the product usable
    x = np.random.default_rng(1).standard_normal((small.n, 4))
    xd4 = torch.from_numpy(x).to(dev)
    yd4 = torch.zeros((small.n, 4), dtype=torch.float64, device=dev)
    assert _static(small, xd4, 4, yd4, 4, 4) == cg.CG_OK
    torch.cuda.synchronize()
    y_host = small.times_matrix(x, cg.CG_PREC_REFINE)
    np.testing.assert_allclose(yd4.cpu().numpy(), y_host, rtol=0, atol=TOL * np.abs(y_host).max())
