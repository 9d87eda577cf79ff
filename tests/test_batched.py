"""Batched solve of many sd-shell problems (lockstep block Davidson under CUDA
graphs, exact batched Jacobi for dimensions <= 64) against exact solves of
each problem built by the oracle.  Bar: the lowest min(5, n) eigenvalues of
every problem within 1e-4 MeV, residual <= 1e-5."""
import numpy as np
import pytest

import cosmo_gb300 as cg
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _problems(tmp, idx=None):
    from cosmo_gb300.synthetic import batched_sd_systems, make_system
    systems = batched_sd_systems()
    if idx is not None:
        systems = [systems[i] for i in idx]
    return [cg.Problem(make_system(tmp, s)[1]) for s in systems]


def _exact(p, k):
    import scipy.linalg as la
    import scipy.sparse.linalg as sla
    inf = p.info
    z = O.basis(p.sps(), inf.nv + inf.zv, inf.twom, inf.nv - inf.zv, inf.parity)
    n = len(z)
    if n == 0:
        return np.zeros(0)
    k1, v1 = p.one_body()
    k2, v2 = p.two_body()
    rp, c, v = O.build_upper(inf.n_sps, k1, v1, k2, v2, z)
    H = O.full_from_upper(rp, c, v)
    if n <= 2000:
        return la.eigvalsh(H.toarray())[:k]
    return np.sort(sla.eigsh(H, k=k, which="SA", tol=1e-12)[0])


def _check(problems, eig, res, nconv, nst):
    for i, p in enumerate(problems):
        ex = _exact(p, nst)
        m = len(ex)
        assert nconv[i] == m, (i, nconv[i], m, res[i])
        np.testing.assert_allclose(eig[i, :m], ex, rtol=0, atol=1e-4, err_msg=f"problem {i}")
        assert np.all(res[i, :m] <= 1e-5)
        assert np.all(np.isnan(eig[i, m:]))


def _subset_indices(tmp):
    """One problem of each of these dimensions of the 64-problem batch."""
    probs = _problems(tmp)
    b = cg.Batch(probs)
    d = b.dims()
    want = [0, 3, 11, 14, 28, 72, 128, 640, 1290, 4206, 7562, 20564]
    idx = []
    for w in want:
        hit = [i for i in range(len(d)) if int(d[i]) == w and i not in idx]
        if hit:
            idx.append(hit[0])
    return idx


def test_batch_subset_matches_exact(gpu_available, tmp_path):
    idx = _subset_indices(str(tmp_path))
    assert len(idx) >= 10
    probs = _problems(str(tmp_path), idx)
    b = cg.Batch(probs)
    eig, res, nconv, st = b.solve(5)
    _check(probs, eig, res, nconv, 5)
    assert st.graph_launches == st.iterations_fp32 + st.iterations_fp64
    assert st.graph_kernels > 10
    # the same solve without graphs gives the same numbers
    eig2, res2, nconv2, st2 = b.solve(5, use_graph=0)
    assert st2.graph_launches == 0
    np.testing.assert_array_equal(eig2, eig)
    np.testing.assert_array_equal(nconv2, nconv)


def test_batch_all_64(gpu_available, tmp_path):
    probs = _problems(str(tmp_path))
    b = cg.Batch(probs)
    d = b.dims()
    assert len(d) == 64 and int(d.max()) == 67251 and int(d.min()) == 0
    eig, res, nconv, st = b.solve(5)
    _check(probs, eig, res, nconv, 5)
