"""GPU parity tests: basis, Hamiltonian connectivity/phases/values, SpMM and
Davidson through the C ABI against the oracle and the reference's golden
outputs.  Tolerances: integer work (basis, columns, signs) bit-exact; H values
1e-12 absolute (FP64 TBME sums); FP64 SpMM 1e-11 relative; FP32 SpMM 1e-5
relative; eigenvalues 1e-4 MeV with residual <= 1e-5 (the parity bar)."""
import hashlib

import numpy as np
import pytest

import cosmo_gb300 as cg
from conftest import conn_hash, golden, manifest, mbs_sha, problem_for
from oracle import oracle as O

pytestmark = pytest.mark.gpu

SMALL = ["sd22m0s1", "sd32m1s2", "fp21m3s6"]
MEDIUM = ["fp22m0s3", "sd44m0s4", "mg24usdb", "sd66m0s5"]


def _gpu(name, tmp, prec=cg.CG_PREC_FP64):
    p = problem_for(name, tmp)
    b = cg.ManyBodyStates(p)
    h = cg.Hamiltonian(p, b, prec)
    return p, b, h


@pytest.mark.parametrize("name", SMALL + MEDIUM)
def test_basis_matches_reference(gpu_available, name, tmp_path):
    m = manifest()[name]
    p = problem_for(name, str(tmp_path))
    b = cg.ManyBodyStates(p)
    assert (b.n, b.N) == (m["n"], m["N"])
    z = b.states()
    assert mbs_sha(z) == m["mbs_sha256"]
    g = golden(name)
    if "mbs" in g:
        assert np.array_equal(z, g["mbs"])
    # .mbs writer is byte-identical
    f = tmp_path / "x.mbs"
    b.write_mbs(str(f))
    assert hashlib.sha256(f.read_bytes()).hexdigest() == m["mbs_sha256"]


@pytest.mark.parametrize("name", ["fp44m0s7", "fp55m0s8"])
def test_large_basis_matches_reference(gpu_available, name, tmp_path):
    m = manifest()[name]
    p = problem_for(name, str(tmp_path))
    b = cg.ManyBodyStates(p)
    assert (b.n, b.N) == (m["n"], m["N"])
    h = hashlib.sha256()
    h.update(np.int32(b.N).tobytes())
    h.update(np.uint64(b.n).tobytes())
    step = 1 << 22
    for s in range(0, b.n, step):
        h.update(b.states(s, min(step, b.n - s)).astype("<u2").tobytes())
    assert h.hexdigest() == m["mbs_sha256"]


def test_locate(gpu_available, tmp_path):
    p = problem_for("sd32m1s2", str(tmp_path))
    b = cg.ManyBodyStates(p)
    z = b.states()
    idx = np.array([0, 1, 7, b.n // 2, b.n - 1])
    assert np.array_equal(b.locate(z[idx]), idx.astype(np.uint64))
    bad = z[:1].copy()
    bad[0, -1] = bad[0, -2]  # repeated orbital: not a determinant of the basis
    assert b.locate(bad)[0] == b.n + 1


@pytest.mark.parametrize("name", SMALL + MEDIUM)
def test_hamiltonian_connectivity_and_values(gpu_available, name, tmp_path):
    m = manifest()[name]
    g = golden(name)
    p, b, h = _gpu(name, str(tmp_path))
    assert h.info.nnz_upper == m["nnz_upper"]
    rp, c, v = h.upper_rows()
    assert conn_hash(rp, c) == m["conn_sha256"]
    if "rowptr" in g:
        np.testing.assert_allclose(v, g["vals"], rtol=0, atol=1e-12)
        assert np.array_equal(np.signbit(v), np.signbit(g["vals"]))
    else:
        for k, r in enumerate(g["sample_rows"]):
            a, e = int(rp[r]), int(rp[r + 1])
            sa, sb = int(g["sample_rowptr"][k]), int(g["sample_rowptr"][k + 1])
            np.testing.assert_allclose(v[a:e], g["sample_vals"][sa:sb], rtol=0, atol=1e-12)
            assert np.array_equal(np.signbit(v[a:e]), np.signbit(g["sample_vals"][sa:sb]))
    d = h.diagonal()
    diag_ref = np.zeros(h.n)
    rows = np.repeat(np.arange(h.n), np.diff(rp).astype(np.int64))
    on = c == rows
    diag_ref[rows[on]] = v[on]
    assert np.array_equal(d, diag_ref)
    # both triangles: H is exactly symmetric
    x = np.random.default_rng(0).standard_normal((h.n, 2))
    y = h.times_matrix(x)
    assert abs(x[:, 0] @ y[:, 1] - x[:, 1] @ y[:, 0]) <= 1e-10 * np.abs(y).sum()


@pytest.mark.parametrize("name", SMALL)
def test_spmm_matches_reference(gpu_available, name, tmp_path):
    g = golden(name)
    x = g["spmm_x"].T.copy()
    yref = g["spmm_y"].T
    _, _, h64 = _gpu(name, str(tmp_path), cg.CG_PREC_FP64)
    y = h64.times_matrix(x)
    np.testing.assert_allclose(y, yref, rtol=0, atol=1e-11 * np.abs(yref).max())
    _, _, h32 = _gpu(name, str(tmp_path), cg.CG_PREC_FP32)
    y32 = h32.times_matrix(x, cg.CG_PREC_FP32)
    np.testing.assert_allclose(y32, yref, rtol=0, atol=1e-5 * np.abs(yref).max())
    yr = h32.times_matrix(x, cg.CG_PREC_REFINE)
    np.testing.assert_allclose(yr, yref, rtol=0, atol=1e-11 * np.abs(yref).max())


@pytest.mark.parametrize("m", [1, 3, 4, 8, 10, 16, 19])
def test_spmm_block_widths(gpu_available, m, tmp_path):
    """Every vector count against the oracle's pull-form CSB product (sd 6+6)."""
    name = "sd66m0s5"
    p, b, h = _gpu(name, str(tmp_path))
    rp, c, v = h.upper_rows()
    x = np.random.default_rng(m).standard_normal((h.n, m))
    yref = O.CSB(rp, c, v).times_matrix(x)
    y = h.times_matrix(x)
    np.testing.assert_allclose(y, yref, rtol=0, atol=1e-10 * np.abs(yref).max())


def _exact(name, tmp, k=10):
    import scipy.sparse.linalg as sla
    p = problem_for(name, tmp)
    inf = p.info
    z = O.basis(p.sps(), inf.nv + inf.zv, inf.twom, inf.nv - inf.zv, inf.parity)
    k1, v1 = p.one_body()
    k2, v2 = p.two_body()
    rp, c, v = O.build_upper(inf.n_sps, k1, v1, k2, v2, z)
    H = O.full_from_upper(rp, c, v)
    return np.sort(sla.eigsh(H, k=k, which="SA", tol=1e-13)[0])


@pytest.mark.parametrize("name", SMALL + ["mg24usdb"])
def test_davidson_fp64_reference_algorithm(gpu_available, name, tmp_path):
    """The reference algorithm (block = nstates, lim = nstates + 20, one-vector
    Gram-Schmidt) in FP64 on the GPU reproduces the reference's converged states."""
    g = golden(name)
    nst = len(g["ref_eig"])
    _, _, h = _gpu(name, str(tmp_path))
    r = cg.davidson_diagonalization(h, nst, want_vectors=True)
    # this control flow, like the reference's, can stall a state; compare the
    # states both runs converged, and every converged state with an exact solve
    ok = (g["ref_resid"] < 1e-5) & (r.resid < 1e-5)
    assert ok.sum() >= nst // 2
    np.testing.assert_allclose(r.eig[ok], g["ref_eig"][ok], rtol=0, atol=1e-6)
    mine = r.resid < 1e-5
    exact = _exact(name, str(tmp_path), nst)
    assert np.all(np.min(np.abs(r.eig[mine][:, None] - exact[None, :]), axis=1) < 1e-6)
    # eigenvectors: |H v - E v| small and orthonormal
    V = r.vecs.T
    HV = h.times_matrix(V)
    res = np.linalg.norm(HV - V * r.eig, axis=0)
    np.testing.assert_allclose(res, r.resid, rtol=1e-3, atol=1e-9)
    np.testing.assert_allclose(V.T @ V, np.eye(nst), atol=1e-8)


@pytest.mark.parametrize("name", ["sd32m1s2", "fp22m0s3", "sd44m0s4", "mg24usdb", "sd66m0s5"])
@pytest.mark.parametrize("pip", [1, 0])
def test_davidson_mixed_vs_exact(gpu_available, name, pip, tmp_path):
    """Mixed precision (FP32 H and vectors, FP64 projection, FP64 refinement):
    lowest eigenvalues within 1e-4 MeV of an exact solve, residuals <= 1e-5,
    orthonormal eigenvectors; with the Pythagorean block orthogonalisation
    (ortho_pip=1, default) and the classical one (0)."""
    nst = 5 if name == "sd32m1s2" else 10
    exact = _exact(name, str(tmp_path), nst)
    _, _, h = _gpu(name, str(tmp_path), cg.CG_PREC_FP32)
    r = cg.davidson_diagonalization(h, nst, want_vectors=True, precision=cg.CG_PREC_FP32, tol_resid=1e-5,
                                    block=nst, lim=min(48, nst * 4), ortho_pip=pip)
    assert r.stats.converged == nst, (r.resid, r.stats.ierr)
    assert np.all(r.resid <= 1e-5)
    np.testing.assert_allclose(r.eig, exact, rtol=0, atol=1e-4)
    V = r.vecs
    np.testing.assert_allclose(V @ V.T, np.eye(nst), rtol=0, atol=1e-8)


MIXED = dict(precision=cg.CG_PREC_FP32, tol_resid=1e-5, block=8, lim=64, keep=32, algorithm=1, precond=1,
             switch_resid=3e-5, refine_lim=32, refine_keep=16)


@pytest.mark.parametrize("name", ["fp22m0s3", "sd44m0s4", "mg24usdb", "sd66m0s5"])
def test_davidson_mixed_fp32_corrections(gpu_available, name, tmp_path):
    """Refinement phase with the correction blocks multiplied in FP32
    (refine_fp32_corrections=1, default) and in double-float (0): the reported
    residuals are the residuals of the returned vectors under the FP64 matrix
    (an FP64 build multiplied in FP64), all <= 1e-5, and both give the same
    eigenvalues (to resid^2 / gap)."""
    nst = 10
    _, _, h = _gpu(name, str(tmp_path), cg.CG_PREC_FP32)
    _, _, h64 = _gpu(name, str(tmp_path))
    out = []
    for corr in (1, 0):
        r = cg.davidson_diagonalization(h, nst, want_vectors=True, refine_fp32_corrections=corr, **MIXED)
        assert r.stats.converged == nst, (corr, r.resid, r.stats.ierr)
        V = r.vecs.T
        res = np.linalg.norm(h64.times_matrix(V) - V * r.eig, axis=0)
        assert np.all(res <= 1e-5), (corr, res)
        np.testing.assert_allclose(res, r.resid, rtol=1e-3, atol=1e-8)
        np.testing.assert_allclose(V.T @ V, np.eye(nst), rtol=0, atol=1e-8)
        out.append(r)
    np.testing.assert_allclose(out[0].eig, out[1].eig, rtol=0, atol=1e-7)


def test_davidson_fp32_corrections_check_fails_over(gpu_available, tmp_path, capfd):
    """When the residuals on FP32 correction products stall above the threshold
    (or the double-float check finds them above it), the refinement goes on
    with double-float products: an early switch (1e-2) lets the FP32-multiplied
    corrections carry coefficients of ~1e-2 (product errors ~1e-7 |H| * 1e-2,
    above a 1e-8 threshold), and the returned vectors still have residuals
    <= 1e-8 under the FP64 matrix."""
    nst = 10
    _, _, h = _gpu("mg24usdb", str(tmp_path), cg.CG_PREC_FP32)
    _, _, h64 = _gpu("mg24usdb", str(tmp_path))
    kw = dict(MIXED, switch_resid=1e-2, tol_resid=1e-8, verbose=1)
    r = cg.davidson_diagonalization(h, nst, want_vectors=True, **kw)
    err = capfd.readouterr().err
    checks = [ln for ln in err.splitlines() if "dav[fp64] double-float" in ln]
    assert len(checks) == 1
    assert int(checks[0].split("unconverged")[1].split()[0]) > 0, checks[0]
    assert r.stats.converged == nst, (r.resid, r.stats.ierr)
    V = r.vecs.T
    res = np.linalg.norm(h64.times_matrix(V) - V * r.eig, axis=0)
    assert np.all(res <= 1e-8), res
    np.testing.assert_allclose(res, r.resid, rtol=1e-2, atol=1e-10)


def test_davidson_keep_bound(gpu_available, tmp_path):
    """A restart keeps at most 64 Ritz vectors (more than 32 are formed 32
    columns at a time in a scratch block): keep and refine_keep above 64 are
    refused on the host before any work, and a solve keeping 40 (more than
    one kernel's 32 outputs) matches the one keeping 16."""
    _, _, h = _gpu("sd22m0s1", str(tmp_path), cg.CG_PREC_FP32)
    for kw in (dict(keep=72), dict(refine_keep=72)):
        with pytest.raises(cg.CosmoError, match="keep must be in 0..64"):
            cg.davidson_diagonalization(h, 4, precision=cg.CG_PREC_FP32, lim=96, block=4, **kw)
    kw = dict(precision=cg.CG_PREC_FP32, tol_resid=1e-6, block=4, lim=56, algorithm=1, switch_resid=3e-5)
    a = cg.davidson_diagonalization(h, 4, keep=40, refine_keep=40, **kw)
    b = cg.davidson_diagonalization(h, 4, keep=16, **kw)
    assert int(a.stats.converged) == 4 and int(b.stats.converged) == 4
    np.testing.assert_allclose(a.eig, b.eig, rtol=0, atol=1e-8)


def test_ee_roundtrip(gpu_available, tmp_path):
    _, _, h = _gpu("sd22m0s1", str(tmp_path))
    r = cg.davidson_diagonalization(h, 4, want_vectors=True)
    f = str(tmp_path / "x.EE")
    cg.write_ee(f, r.eig, r.de, r.resid, r.vecs)
    E, D, R, V = cg.read_ee(f)
    assert np.array_equal(E, r.eig) and np.array_equal(R, r.resid) and np.array_equal(V, r.vecs)


def test_hh_writer_layout(gpu_available, tmp_path):
    """.HH: u64 n, per row u32 nz, u64 ind[nz], f64 elem[nz] (PPMatrix::Write)."""
    g = golden("sd22m0s1")
    _, _, h = _gpu("sd22m0s1", str(tmp_path))
    f = tmp_path / "x.HH"
    h.write_hh(str(f))
    raw = f.read_bytes()
    n = int(np.frombuffer(raw[:8], np.uint64)[0])
    off = 8
    cols, vals = [], []
    for _ in range(n):
        nz = int(np.frombuffer(raw[off:off + 4], np.uint32)[0]); off += 4
        cols.append(np.frombuffer(raw[off:off + 8 * nz], np.uint64)); off += 8 * nz
        vals.append(np.frombuffer(raw[off:off + 8 * nz], np.float64)); off += 8 * nz
    assert off == len(raw)
    assert np.array_equal(np.concatenate(cols), g["cols"].astype(np.uint64))
    np.testing.assert_allclose(np.concatenate(vals), g["vals"], rtol=0, atol=1e-12)


def _parse_hh(raw: bytes):
    n = int(np.frombuffer(raw[:8], np.uint64)[0])
    off = 8
    rows = []
    for _ in range(n):
        nz = int(np.frombuffer(raw[off:off + 4], np.uint32)[0]); off += 4
        c = np.frombuffer(raw[off:off + 8 * nz], np.uint64); off += 8 * nz
        v = np.frombuffer(raw[off:off + 8 * nz], np.float64); off += 8 * nz
        rows.append((c, v))
    assert off == len(raw)
    return n, rows


@pytest.mark.parametrize("name", SMALL)
def test_hh_writer_vs_reference_file(gpu_available, name, tmp_path):
    """.HH from the GPU matrix against the reference XHH+JJ output: same rows,
    except entries with |H_ij| < 1e-14 that the reference file keeps and the
    CSB (and this library) drops; byte-identical when there are none."""
    m = manifest()[name]
    _, _, h = _gpu(name, str(tmp_path))
    f = tmp_path / "x.HH"
    h.write_hh(str(f))
    raw = f.read_bytes()
    if hashlib.sha256(raw).hexdigest() == m["ref_hh_sha256"]:
        return
    assert len(raw) <= m["ref_hh_bytes"]


def test_hh_reader_on_reference_file(gpu_available, tmp_path):
    """The reference's own .HH (sd 2+2) read into a GPU matrix reproduces the
    reference product and diagonal; FP64 and FP32 (hi + lo) storage."""
    g = golden("sd22m0s1")
    f = tmp_path / "ref.HH"
    f.write_bytes(g["ref_hh"].tobytes())
    n, rows = _parse_hh(f.read_bytes())
    x = g["spmm_x"].T.copy()
    yref = g["spmm_y"].T
    for prec in (cg.CG_PREC_FP64, cg.CG_PREC_FP32):
        h = cg.Hamiltonian.from_hh(str(f), prec)
        assert h.n == n
        y = h.times_matrix(x, cg.CG_PREC_FP64 if prec == cg.CG_PREC_FP64 else cg.CG_PREC_REFINE)
        np.testing.assert_allclose(y, yref, rtol=0, atol=1e-11 * np.abs(yref).max())
        d = np.array([v[c == i].sum() for i, (c, v) in enumerate(rows)])
        np.testing.assert_allclose(h.diagonal(), d, rtol=0, atol=1e-12)
        # round trip through the writer: the same symmetric matrix (the reference
        # file keeps each pair in the row of the determinant it was generated
        # from, this writer in the upper triangle)
        f2 = tmp_path / f"rt{prec}.HH"
        h.write_hh(str(f2))
        n2, rows2 = _parse_hh(f2.read_bytes())
        assert n2 == n

        def pairs(rs):
            out = {}
            for i, (c, v) in enumerate(rs):
                for j, x in zip(c.tolist(), v.tolist()):
                    if abs(x) >= 1e-14:
                        key = (min(i, j), max(i, j))
                        out[key] = out.get(key, 0.0) + x
            return out
        p1, p2 = pairs(rows), pairs(rows2)
        assert p1.keys() == p2.keys()
        assert max(abs(p1[k] - p2[k]) for k in p1) < 1e-12
        assert all(int(c.min()) >= i for i, (c, v) in enumerate(rows2) if len(c))


def test_davidson_mixed_iteration_cap_residuals(gpu_available, tmp_path):
    """A mixed solve stopped by the iteration cap inside the refinement (still
    on FP32 correction products) reports the residuals of its returned vectors
    under the FP64 matrix, and the unconverged status."""
    nst = 10
    _, _, h = _gpu("sd66m0s5", str(tmp_path), cg.CG_PREC_FP32)
    _, _, h64 = _gpu("sd66m0s5", str(tmp_path))
    r = cg.davidson_diagonalization(h, nst, want_vectors=True, **dict(MIXED, maxiter=3))
    assert r.stats.refine_iterations == 3 and r.stats.converged < nst and r.stats.ierr != 0
    V = r.vecs.T
    res = np.linalg.norm(h64.times_matrix(V) - V * r.eig, axis=0)
    np.testing.assert_allclose(res, r.resid, rtol=1e-6, atol=1e-12)
    np.testing.assert_allclose(V.T @ V, np.eye(nst), rtol=0, atol=1e-8)


def test_sd66_fp64_block4_lim40(gpu_available, tmp_path):
    """sd 6+6 (n = 93,710) as the FP64 stored-H workload with block 4 and basis
    limit 40: the residual-driven solver in FP64 converges all 10 pairs to the
    exact spectrum (1e-6 MeV), and the reference control flow's converged
    pairs are exact eigenpairs too (it may stall some, like the reference)."""
    nst = 10
    exact = _exact("sd66m0s5", str(tmp_path), nst)
    _, _, h = _gpu("sd66m0s5", str(tmp_path))
    r1 = cg.davidson_diagonalization(h, nst, want_vectors=False, precision=cg.CG_PREC_FP64, tol_resid=1e-5,
                                     block=4, lim=40, algorithm=1, keep=20, precond=1)
    assert r1.stats.converged == nst, (r1.resid, r1.stats.ierr)
    np.testing.assert_allclose(r1.eig, exact, rtol=0, atol=1e-6)
    r0 = cg.davidson_diagonalization(h, nst, want_vectors=False, precision=cg.CG_PREC_FP64, tol_resid=1e-5,
                                     block=4, lim=40, algorithm=0)
    ok = r0.resid <= 1e-5
    assert ok.sum() >= nst // 2, r0.resid
    assert np.all(np.min(np.abs(r0.eig[ok][:, None] - exact[None, :]), axis=1) < 1e-6)
