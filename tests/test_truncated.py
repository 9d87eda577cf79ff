"""Truncated bases on the GPU (oscillator-quanta windows, <hwrejection>,
orbital-occupation rejections), pinned to the reference's XsysmbsOMP output
(the .mbs sha256 of tests/golden/manifest.json, made by running the reference
on these XML files) and to the oracle: the basis byte for byte, the
Hamiltonian projected on the basis (the reference's PPMatrix2CSBBlk skips a
ket its locate does not find) with bit-exact connectivity and values within
1e-12, eigenvalues within 1e-6 MeV of an exact solve, integral J for the
eigenvectors (hw and occupation truncations commute with J), and the batched
solver.  The on-the-fly product (nothing stored) of a truncated basis equals
the stored matrix's product: diagonal within 1e-12, FP64 and double-float
products within 1e-11 of max |y|, FP32 within 1e-5, and its Davidson solves
agree with the stored matrix's within 1e-5 MeV."""
import os
import sys

import numpy as np
import pytest

import cosmo_gb300 as cg
from conftest import conn_hash, golden, manifest, mbs_sha
from oracle import oracle as O

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
import truncated as T  # noqa: E402

pytestmark = pytest.mark.gpu
CASES = sorted(T.CASES)


def _oracle(p, name):
    inf = p.info
    hw, rej = T.truncation(name)
    z = O.basis_truncated(p.sps(), inf.nv, inf.zv, inf.twom, inf.parity, hw=hw, rejections=rej)
    k1, v1 = p.one_body()
    k2, v2 = p.two_body()
    return z, O.build_upper(inf.n_sps, k1, v1, k2, v2, z)


@pytest.mark.parametrize("name", CASES)
def test_truncated_basis_matches_reference(gpu_available, name, tmp_path):
    m = manifest()[name]
    p = cg.Problem(T.write_case(str(tmp_path), name))
    b = cg.ManyBodyStates(p)
    z = b.states()
    assert z.shape == (m["n"], m["N"])
    assert mbs_sha(z) == m["mbs_sha256"]
    g = golden(name)
    if "mbs" in g:
        assert np.array_equal(z, g["mbs"])
    # locate: every basis state finds itself
    idx = b.locate(z)
    assert np.array_equal(idx, np.arange(b.n))


def test_truncated_hwmax_child_element(gpu_available, tmp_path):
    """hwmax as a child element (<hwmax>2</hwmax>, read by the reference's
    getXMLData too) gives the same basis as the attribute."""
    xml = T.write_case(str(tmp_path), "psd22m0_hw2")
    txt = open(xml).read().replace(' hwmax="2"', "", 1).replace("<matrix JJ", "<hwmax>2</hwmax><matrix JJ", 1)
    child = tmp_path / "child.xml"
    child.write_text(txt)
    z = cg.ManyBodyStates(cg.Problem(str(child))).states()
    assert mbs_sha(z) == manifest()["psd22m0_hw2"]["mbs_sha256"]


@pytest.mark.parametrize("name", CASES)
def test_truncated_hamiltonian_and_spectrum(gpu_available, name, tmp_path):
    p = cg.Problem(T.write_case(str(tmp_path), name))
    b = cg.ManyBodyStates(p)
    z, (orp, oc, ov) = _oracle(p, name)
    h = cg.Hamiltonian(p, b, cg.CG_PREC_FP64)
    rp, c, v = h.upper_rows()
    assert conn_hash(rp, c) == conn_hash(orp, oc)
    assert np.abs(v - ov).max() <= 1e-12
    exact = np.linalg.eigvalsh(O.full_from_upper(orp, oc, ov).toarray())
    nst = min(5, b.n - 1)
    for prec in (cg.CG_PREC_FP64, cg.CG_PREC_FP32):
        hh = h if prec == cg.CG_PREC_FP64 else cg.Hamiltonian(p, b, prec)
        r = cg.davidson_diagonalization(hh, nst, want_vectors=True, precision=prec, tol_resid=1e-6,
                                        block=nst, lim=min(4 * nst, b.n), algorithm=1)
        assert r.stats.converged == nst, (r.resid, r.stats.ierr)
        np.testing.assert_allclose(r.eig, exact[:nst], rtol=0, atol=1e-6)
    jj, _ = cg.jt_expectations(b, r.vecs)
    twom = p.info.twom
    for q in jj:  # 2J from <J-J+> is an integer of the parity of 2M
        x = np.sqrt(4 * q + twom * (twom + 2) + 1) - 1
        assert abs(x - round(x)) < 1e-6 and (round(x) - twom) % 2 == 0, jj


def test_truncated_batch(gpu_available, tmp_path):
    probs = [cg.Problem(T.write_case(str(tmp_path), n)) for n in ("psd22m0_hw2", "psd21m1_rej")]
    eig, res, nconv, _ = cg.Batch(probs).solve(3)
    for i, (p, n) in enumerate(zip(probs, ("psd22m0_hw2", "psd21m1_rej"))):
        _, (orp, oc, ov) = _oracle(p, n)
        ex = np.linalg.eigvalsh(O.full_from_upper(orp, oc, ov).toarray())[:3]
        np.testing.assert_allclose(eig[i], ex, rtol=0, atol=1e-4)


@pytest.mark.parametrize("name", CASES + sorted(T.LARGE))
def test_truncated_on_the_fly_matches_stored(gpu_available, name, tmp_path):
    p = cg.Problem(T.write_case(str(tmp_path), name))
    b = cg.ManyBodyStates(p)
    hs = cg.Hamiltonian(p, b, cg.CG_PREC_FP64)
    hv = cg.Hamiltonian(p, b, cg.CG_PREC_FP64, virtual=True)
    assert hv.virtual and hv.n == b.n
    np.testing.assert_allclose(hv.diagonal(), hs.diagonal(), rtol=0, atol=1e-12)
    for m in (1, 5, 8):
        x = np.random.default_rng(m).standard_normal((b.n, m))
        ys = hs.times_matrix(x)
        scale = np.abs(ys).max()
        np.testing.assert_allclose(hv.times_matrix(x), ys, rtol=0, atol=1e-11 * scale)
        np.testing.assert_allclose(hv.times_matrix(x, cg.CG_PREC_FP32), ys, rtol=0, atol=1e-5 * scale)
        np.testing.assert_allclose(hv.times_matrix(x, cg.CG_PREC_REFINE), ys, rtol=0, atol=1e-11 * scale)


@pytest.mark.parametrize("name", sorted(T.LARGE))
def test_truncated_on_the_fly_davidson(gpu_available, name, tmp_path):
    """Mixed Davidson on the FP32 on-the-fly product against the FP64
    residual-driven solve of the stored matrix."""
    p = cg.Problem(T.write_case(str(tmp_path), name))
    b = cg.ManyBodyStates(p)
    nst = 8
    hs = cg.Hamiltonian(p, b, cg.CG_PREC_FP64)
    r64 = cg.davidson_diagonalization(hs, nst, precision=cg.CG_PREC_FP64, tol_resid=1e-7, block=8, lim=48,
                                      algorithm=1)
    assert r64.stats.converged == nst
    hv = cg.Hamiltonian(p, b, cg.CG_PREC_FP32, virtual=True)
    r = cg.davidson_diagonalization(hv, nst, want_vectors=True, precision=cg.CG_PREC_FP32, tol_resid=1e-5,
                                    block=8, lim=48)
    assert r.stats.converged == nst, (r.resid, r.stats.ierr)
    np.testing.assert_allclose(r.eig, r64.eig, rtol=0, atol=1e-5)
