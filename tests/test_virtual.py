"""On-the-fly (virtual) Hamiltonian product against the stored matrix and the
oracle, through the C ABI.  Tolerances: diagonal 1e-12 absolute (FP64 sums in
another order); FP64 products 1e-11 of max |y|; FP32 products 1e-5 of max |y|;
eigenvalues 1e-4 MeV with residual <= 1e-5."""
import numpy as np
import pytest

import cosmo_gb300 as cg
from conftest import golden, problem_for
from oracle import oracle as O

pytestmark = pytest.mark.gpu

SMALL = ["sd22m0s1", "sd32m1s2", "fp21m3s6"]
MEDIUM = ["fp22m0s3", "sd44m0s4", "mg24usdb", "sd66m0s5"]


def _pair(name, tmp, prec=cg.CG_PREC_FP64):
    p = problem_for(name, tmp)
    b = cg.ManyBodyStates(p)
    return p, b, cg.Hamiltonian(p, b, prec), cg.Hamiltonian(p, b, prec, virtual=True)


@pytest.mark.parametrize("name", SMALL)
def test_virtual_matches_oracle(gpu_available, name, tmp_path):
    """FP64 on-the-fly product vs the oracle's pull-form CSB product of the
    reference's rows (golden fixtures)."""
    g = golden(name)
    p = problem_for(name, str(tmp_path))
    b = cg.ManyBodyStates(p)
    hv = cg.Hamiltonian(p, b, cg.CG_PREC_FP64, virtual=True)
    x = g["spmm_x"].T.copy()
    yref = g["spmm_y"].T
    y = hv.times_matrix(x)
    np.testing.assert_allclose(y, yref, rtol=0, atol=1e-11 * np.abs(yref).max())
    rp, c, v = g["rowptr"], g["cols"], g["vals"]
    d = np.zeros(hv.n)
    rows = np.repeat(np.arange(hv.n), np.diff(rp).astype(np.int64))
    on = c == rows
    d[rows[on]] = v[on]
    np.testing.assert_allclose(hv.diagonal(), d, rtol=0, atol=1e-12)


@pytest.mark.parametrize("name", SMALL + MEDIUM)
@pytest.mark.parametrize("m", [1, 4, 8, 11])
def test_virtual_matches_stored(gpu_available, name, m, tmp_path):
    _, _, hs, hv = _pair(name, str(tmp_path))
    assert hv.virtual and hv.info.nnz_upper == 0 and hv.info.nnz_full >= hs.info.nnz_full
    np.testing.assert_allclose(hv.diagonal(), hs.diagonal(), rtol=0, atol=1e-12)
    x = np.random.default_rng(m).standard_normal((hs.n, m))
    ys = hs.times_matrix(x)
    yv = hv.times_matrix(x)
    scale = np.abs(ys).max()
    np.testing.assert_allclose(yv, ys, rtol=0, atol=1e-11 * scale)
    y32 = hv.times_matrix(x, cg.CG_PREC_FP32)
    np.testing.assert_allclose(y32, ys, rtol=0, atol=1e-5 * scale)
    yr = hv.times_matrix(x, cg.CG_PREC_REFINE)
    np.testing.assert_allclose(yr, ys, rtol=0, atol=1e-11 * scale)


def test_virtual_rejects_row_export(gpu_available, tmp_path):
    p = problem_for("sd22m0s1", str(tmp_path))
    b = cg.ManyBodyStates(p)
    hv = cg.Hamiltonian(p, b, cg.CG_PREC_FP32, virtual=True)
    with pytest.raises(cg.CosmoError):
        hv.upper_rows()
    with pytest.raises(cg.CosmoError):
        hv.write_hh(str(tmp_path / "x.HH"))
    with pytest.raises(cg.CosmoError):
        hv.autotune(8)


def _exact(name, tmp, k):
    import scipy.sparse.linalg as sla
    p = problem_for(name, tmp)
    inf = p.info
    z = O.basis(p.sps(), inf.nv + inf.zv, inf.twom, inf.nv - inf.zv, inf.parity)
    k1, v1 = p.one_body()
    k2, v2 = p.two_body()
    rp, c, v = O.build_upper(inf.n_sps, k1, v1, k2, v2, z)
    return np.sort(sla.eigsh(O.full_from_upper(rp, c, v), k=k, which="SA", tol=1e-13)[0])


@pytest.mark.parametrize("name", ["sd44m0s4", "mg24usdb", "sd66m0s5"])
def test_virtual_davidson(gpu_available, name, tmp_path):
    """Mixed (FP32 on-the-fly products, FP64 projection and refinement) and
    plain FP64 Davidson on the on-the-fly product agree with an exact solve."""
    nst = 10
    exact = _exact(name, str(tmp_path), 2 * nst)[:nst]
    spectrum = _exact(name, str(tmp_path), 2 * nst)
    p = problem_for(name, str(tmp_path))
    b = cg.ManyBodyStates(p)
    hv = cg.Hamiltonian(p, b, cg.CG_PREC_FP32, virtual=True)
    r = cg.davidson_diagonalization(hv, nst, want_vectors=True, precision=cg.CG_PREC_FP32, tol_resid=1e-5,
                                    block=8, lim=48)
    assert r.stats.converged == nst, (r.resid, r.stats.ierr)
    assert np.all(r.resid <= 1e-5)
    np.testing.assert_allclose(r.eig, exact, rtol=0, atol=1e-4)
    # plain FP64 Davidson (the reference algorithm: block = nstates, limit
    # nstates + 20) on the FP64 on-the-fly product; like the reference it may
    # leave a state unconverged, so every converged state is checked
    r64 = cg.davidson_diagonalization(hv, nst, precision=cg.CG_PREC_FP64)
    ok = r64.resid <= 1e-5
    assert ok.sum() >= nst // 2
    assert np.all(np.min(np.abs(r64.eig[ok][:, None] - spectrum[None, :]), axis=1) < 1e-4)
    np.testing.assert_allclose(r64.eig[:4], exact[:4], rtol=0, atol=1e-4)
