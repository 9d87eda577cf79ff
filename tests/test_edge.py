"""Edge cases of the path: an empty (M, parity) sector, one-state and
three-state bases, and as many wanted states as the dimension.  The basis
sizes are checked against the oracle's enumeration on the CPU; on the GPU
the basis, the stored matrix and the solvers must handle them: an empty
basis builds an empty matrix and the Davidson call refuses it
(CG_ERR_ARG, nstates above the dimension); on the tiny bases every solver
returns the exact spectrum (dense eigensolve of the oracle's matrix)."""
import numpy as np
import pytest

from oracle import oracle as O

# (space, neutrons, protons, 2M, parity): sd with one neutron and 2M = 7 is
# empty (j <= 5/2); 2M = 5 has the single d5/2 m = 5/2 state; 2M = 1 three
CASES = {"empty": ("sd", 1, 0, 7, "+"), "one": ("sd", 1, 0, 5, "+"), "three": ("sd", 1, 0, 1, "+"),
         "fp_one_each": ("fp", 1, 1, 0, "+")}


def _xml(tmp, key):
    from cosmo_gb300.synthetic import SyntheticSystem, make_system
    sp, nv, zv, twom, par = CASES[key]
    return make_system(tmp, SyntheticSystem(sp, nv, zv, twom, par, 0.5, 3, name="edge_" + key))[1]


def _oracle(tmp, key):
    import cosmo_gb300 as cg
    p = cg.Problem(_xml(tmp, key))
    inf = p.info
    z = O.basis(p.sps(), inf.nv + inf.zv, inf.twom, inf.nv - inf.zv, inf.parity)
    if len(z) == 0:
        return p, z, np.zeros((0, 0))
    k1, v1 = p.one_body()
    k2, v2 = p.two_body()
    rp, c, v = O.build_upper(inf.n_sps, k1, v1, k2, v2, z)
    H = O.full_from_upper(rp, c, v)
    return p, z, H.toarray() if hasattr(H, "toarray") else np.asarray(H)


@pytest.mark.parametrize("key,n", [("empty", 0), ("one", 1), ("three", 3)])
def test_edge_basis_sizes(tmp_path, key, n):
    _, z, _ = _oracle(str(tmp_path), key)
    assert len(z) == n


@pytest.mark.gpu
def test_edge_empty_sector(gpu_available, tmp_path):
    import cosmo_gb300 as cg
    p, z, _ = _oracle(str(tmp_path), "empty")
    b = cg.ManyBodyStates(p)
    assert b.n == 0
    for prec in (cg.CG_PREC_FP64, cg.CG_PREC_FP32):
        h = cg.Hamiltonian(p, b, prec)
        assert h.n == 0 and h.info.nnz_full == 0
        with pytest.raises(cg.CosmoError) as e:
            cg.davidson_diagonalization(h, 1, precision=prec)
        assert e.value.status == cg.CG_ERR_ARG


@pytest.mark.gpu
@pytest.mark.parametrize("key", ["one", "three", "fp_one_each"])
def test_edge_tiny_spectra(gpu_available, tmp_path, key):
    import cosmo_gb300 as cg
    p, z, H = _oracle(str(tmp_path), key)
    exact = np.linalg.eigvalsh(H)
    b = cg.ManyBodyStates(p)
    assert np.array_equal(b.states(), z)
    n = len(z)
    k = min(n, 4)
    for prec in (cg.CG_PREC_FP64, cg.CG_PREC_FP32):
        h = cg.Hamiltonian(p, b, prec)
        for kw in (dict(algorithm=0), dict(algorithm=1)):
            r = cg.davidson_diagonalization(h, k, precision=prec, tol_resid=1e-7, **kw)
            np.testing.assert_allclose(r.eig, exact[:k], rtol=0, atol=1e-8 * max(1.0, np.abs(exact).max()))
        # as many states as the engine takes (all of a tiny basis), the basis
        # limit at the whole space: the reference's own default, lim =
        # nstates + 20, lets its convergence test (eigenvalue changes) stop
        # on a subspace that misses states when nstates is a large share of
        # n (the oracle's dvdrvr2 returns the same wrong set on fp 1+1), so
        # that default is not what this checks
        r = cg.davidson_diagonalization(h, n if n <= 16 else 16, precision=prec, tol_resid=1e-7, lim=64)
        np.testing.assert_allclose(r.eig, exact[:len(r.eig)], rtol=0, atol=1e-8 * max(1.0, np.abs(exact).max()))


@pytest.mark.gpu
@pytest.mark.parametrize("key", ["one", "three", "fp_one_each"])
def test_exact_diagonalization(gpu_available, tmp_path, key):
    """cg_dense_eigensolve (the reference DXHV's path for small dimensions):
    every eigenvalue of the stored matrix, FP64 and FP32 (hi + lo) storage,
    against the dense spectrum of the oracle's matrix; eigenvectors
    orthonormal with H v = E v."""
    import cosmo_gb300 as cg
    p, z, H = _oracle(str(tmp_path), key)
    exact = np.linalg.eigvalsh(H)
    b = cg.ManyBodyStates(p)
    for prec in (cg.CG_PREC_FP64, cg.CG_PREC_FP32):
        h = cg.Hamiltonian(p, b, prec)
        eig, vecs = h.dense_eigensolve()
        np.testing.assert_allclose(eig, exact, rtol=0, atol=1e-10 * max(1.0, np.abs(exact).max()))
        assert np.abs(vecs @ vecs.T - np.eye(len(z))).max() < 1e-12
        assert np.abs(H @ vecs.T - vecs.T * eig[None, :]).max() < 1e-10 * max(1.0, np.abs(exact).max())
