"""CPU tests: the oracle against the reference's golden outputs, the host-side
interaction restatement against the reference's operator terms, and the
synthetic input generator."""
import os

import numpy as np
import pytest

from conftest import conn_hash, golden, manifest, mbs_sha, problem_for, synthetic_xml
from oracle import oracle as O

SMALL = ["sd22m0s1", "sd32m1s2", "fp21m3s6"]
MEDIUM = ["fp22m0s3", "sd44m0s4", "mg24usdb"]


def _terms(name, tmp):
    p = problem_for(name, tmp)
    k1, v1 = p.one_body()
    k2, v2 = p.two_body()
    return p, k1, v1, k2, v2


def test_synthetic_channel_counts():
    from cosmo_gb300.synthetic import FP_ORBITS, SD_ORBITS, channel_lines
    assert len(channel_lines(SD_ORBITS)) == 63
    assert len(channel_lines(FP_ORBITS)) == 195


@pytest.mark.parametrize("name", SMALL)
def test_host_operator_terms_match_reference(name, tmp_path):
    """xReadSPInt restatement (ESP, VSPX incl. lambda J-J+) vs the reference dump."""
    g = golden(name)
    p, k1, v1, k2, v2 = _terms(name, str(tmp_path))
    assert np.array_equal(p.sps(), g["sps"])
    assert np.array_equal(k1, g["esp_keys"])
    assert np.array_equal(v1, g["esp_vals"])
    assert np.array_equal(k2, g["vspx_keys"])
    np.testing.assert_allclose(v2, g["vspx_vals"], rtol=0, atol=1e-13)


def test_host_operator_usdb_matches_reference(tmp_path):
    """usdb with its mass scaling (needs the reference interaction file; skipped elsewhere)."""
    root = O.reference_root()
    usdb = os.path.join(root, "interactions", "sd", "usdb.int") if root else ""
    if not os.path.exists(usdb):
        pytest.skip("reference checkout not given (COSMO_REFERENCE)")
    import cosmo_gb300 as cg
    from cosmo_gb300.synthetic import SyntheticSystem, write_xml
    orbits = [("0d3", 0, 2, 3), ("0d5", 0, 2, 5), ("1s1", 1, 0, 1)]
    xml = str(tmp_path / "mg24.xml")
    write_xml(xml, SyntheticSystem("sd", 4, 4, 0, "+", 0.0, 0, name="mg24usdb"), usdb, orbits, hname="usdb")
    txt = open(xml).read().replace('<matrix JJ="0.0"/>', "")
    open(xml, "w").write(txt)
    p = cg.Problem(xml)
    g = golden("mg24usdb")
    k2, v2 = p.two_body()
    assert np.array_equal(k2, g["vspx_keys"])
    np.testing.assert_allclose(v2, g["vspx_vals"], rtol=0, atol=1e-13)
    k1, v1 = p.one_body()
    assert np.array_equal(k1, g["esp_keys"]) and np.array_equal(v1, g["esp_vals"])


@pytest.mark.parametrize("name", SMALL)
def test_oracle_interaction_matches_reference(name, tmp_path):
    """The oracle's own XML/Oxbash/AddPPVsp/J-J+ restatement (no product
    library) against the reference's operator terms: keys identical, values
    within 1e-13."""
    from oracle import interaction as OI
    g = golden(name)
    sysd, k1, v1, k2, v2 = OI.operator_terms(synthetic_xml(name, str(tmp_path)))
    assert np.array_equal(sysd.sps, g["sps"])
    assert np.array_equal(k1, g["esp_keys"]) and np.array_equal(k2, g["vspx_keys"])
    np.testing.assert_allclose(v1, g["esp_vals"], rtol=0, atol=1e-13)
    np.testing.assert_allclose(v2, g["vspx_vals"], rtol=0, atol=1e-13)


def test_oracle_interaction_usdb_matches_reference(tmp_path):
    """usdb with its mass scaling through the oracle's restatement (needs the
    reference interaction file; skipped without the reference checkout)."""
    from oracle import interaction as OI
    from cosmo_gb300.synthetic import SyntheticSystem, write_xml
    root = O.reference_root()
    usdb = os.path.join(root, "interactions", "sd", "usdb.int") if root else ""
    if not os.path.exists(usdb):
        pytest.skip("reference checkout not given (COSMO_REFERENCE)")
    orbits = [("0d3", 0, 2, 3), ("0d5", 0, 2, 5), ("1s1", 1, 0, 1)]
    xml = str(tmp_path / "mg24.xml")
    write_xml(xml, SyntheticSystem("sd", 4, 4, 0, "+", 0.0, 0, name="mg24usdb"), usdb, orbits, hname="usdb")
    txt = open(xml).read().replace('<matrix JJ="0.0"/>', "")
    open(xml, "w").write(txt)
    g = golden("mg24usdb")
    sysd, k1, v1, k2, v2 = OI.operator_terms(xml)
    assert np.array_equal(k1, g["esp_keys"]) and np.array_equal(k2, g["vspx_keys"])
    np.testing.assert_allclose(v1, g["esp_vals"], rtol=0, atol=1e-13)
    np.testing.assert_allclose(v2, g["vspx_vals"], rtol=0, atol=1e-13)


@pytest.mark.parametrize("name", ["sd32m1s2", "fp21m3s6", "fp22m0s3"])
def test_oracle_only_pipeline_matches_reference(name, tmp_path):
    """The CPU baseline's pipeline, with nothing from the product library:
    oracle interaction -> oracle basis -> oracle rows reproduce the reference's
    basis and connectivity hashes."""
    from oracle import interaction as OI
    m = manifest()[name]
    sysd, k1, v1, k2, v2 = OI.operator_terms(synthetic_xml(name, str(tmp_path)))
    z = O.basis(sysd.sps, sysd.nv + sysd.zv, sysd.twom, sysd.nv - sysd.zv, sysd.parity)
    assert mbs_sha(z) == m["mbs_sha256"]
    rp, c, v = O.build_upper(len(sysd.sps), k1, v1, k2, v2, z)
    assert int(rp[-1]) == m["nnz_upper"] and conn_hash(rp, c) == m["conn_sha256"]


@pytest.mark.parametrize("name", SMALL + MEDIUM + ["sd66m0s5", "fp44m0s7"])
def test_oracle_basis_matches_reference(name, tmp_path):
    m = manifest()[name]
    p = problem_for(name, str(tmp_path))
    inf = p.info
    z = O.basis(p.sps(), inf.nv + inf.zv, inf.twom, inf.nv - inf.zv, inf.parity)
    assert z.shape == (m["n"], m["N"])
    assert mbs_sha(z) == m["mbs_sha256"]
    g = golden(name) if name != "fp44m0s7" else {}
    if "mbs" in g:
        assert np.array_equal(z, g["mbs"])


@pytest.mark.parametrize("name", SMALL + MEDIUM)
def test_oracle_rows_match_reference(name, tmp_path):
    """Upper-triangle rows with the reference's own operator terms: bit-exact."""
    m = manifest()[name]
    g = golden(name)
    p = problem_for(name, str(tmp_path))
    inf = p.info
    z = O.basis(p.sps(), inf.nv + inf.zv, inf.twom, inf.nv - inf.zv, inf.parity)
    if "esp_keys" in g:
        k1, v1, k2, v2 = g["esp_keys"], g["esp_vals"], g["vspx_keys"], g["vspx_vals"]
    else:
        k1, v1 = p.one_body()
        k2, v2 = p.two_body()
    rp, c, v = O.build_upper(inf.n_sps, k1, v1, k2, v2, z)
    assert int(rp[-1]) == m["nnz_upper"]
    assert conn_hash(rp, c) == m["conn_sha256"]
    if "rowptr" in g:
        assert np.array_equal(v, g["vals"])
    else:
        for k, r in enumerate(g["sample_rows"]):
            a, b = int(rp[r]), int(rp[r + 1])
            sa, sb = int(g["sample_rowptr"][k]), int(g["sample_rowptr"][k + 1])
            assert np.array_equal(c[a:b], g["sample_cols"][sa:sb])
            np.testing.assert_allclose(v[a:b], g["sample_vals"][sa:sb], rtol=0, atol=1e-12)


@pytest.mark.parametrize("name", SMALL)
def test_oracle_spmm_matches_reference(name):
    g = golden(name)
    csb = O.CSB(g["rowptr"], g["cols"], g["vals"])
    y = csb.times_matrix(g["spmm_x"].T).T
    assert np.array_equal(y, g["spmm_y"])


@pytest.mark.parametrize("name", SMALL + ["mg24usdb"])
def test_oracle_davidson_matches_reference(name, tmp_path):
    """Eigenvalues of the restated Davidson vs the reference run, on the states
    the reference converged (the reference sometimes stalls a state)."""
    g = golden(name)
    if "rowptr" in g:
        rp, c, v = g["rowptr"], g["cols"], g["vals"]
    else:
        p = problem_for(name, str(tmp_path))
        inf = p.info
        z = O.basis(p.sps(), inf.nv + inf.zv, inf.twom, inf.nv - inf.zv, inf.parity)
        rp, c, v = O.build_upper(inf.n_sps, g["esp_keys"], g["esp_vals"], g["vspx_keys"], g["vspx_vals"], z)
    nst = len(g["ref_eig"])
    r = O.CSB(rp, c, v).davidson(max(nst, 10) if nst >= 10 else nst)
    ok = g["ref_resid"] < 1e-5
    assert ok.sum() >= nst // 2
    np.testing.assert_allclose(r["eig"][:nst][ok], g["ref_eig"][ok], rtol=0, atol=1e-6)


def test_oracle_mg24_known_answers(tmp_path):
    """EXAMPLE-24Mg-usdb.md:29-38 energies (4 decimals) on the converged states."""
    m = manifest()["mg24usdb"]
    g = golden("mg24usdb")
    ex = np.array(m["example_E"])
    ok = g["ref_resid"] < 1e-5
    np.testing.assert_allclose(g["ref_eig"][ok], ex[ok], atol=6e-5)


def test_header_symbols_exported():
    """The C-ABI library exports every function include/cosmo_gb300.h declares."""
    import re
    import ctypes
    import cosmo_gb300 as cg
    hdr = open(os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include",
                            "cosmo_gb300.h")).read()
    names = sorted(set(re.findall(r"\b(cg_[a-z0-9_]+)\s*\(", hdr)))
    assert len(names) >= 25
    L = ctypes.CDLL(cg.LIB_PATH)
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    assert set(names) <= set(cg._SIGS), set(names) - set(cg._SIGS)


def test_error_status_codes(tmp_path):
    import cosmo_gb300 as cg
    with pytest.raises(cg.CosmoError) as e:
        cg.Problem(str(tmp_path / "missing.xml"))
    assert e.value.status == -2
    bad = tmp_path / "bad.xml"
    bad.write_text("<cosmo><valencespace><orbital index='1' j='5/2'/></valencespace>")
    with pytest.raises(cg.CosmoError) as e:
        cg.Problem(str(bad))
    assert e.value.status == -3
    if cg.device_count() == 0:
        p = problem_for("sd22m0s1", str(tmp_path))
        with pytest.raises(cg.CosmoError) as e:
            cg.ManyBodyStates(p)
        assert e.value.status == -9


def test_problem_from_terms_rejects_backward_keys():
    import cosmo_gb300 as cg
    g = golden("sd22m0s1")
    k2 = g["vspx_keys"].copy()
    k2[0] = k2[0][[2, 3, 0, 1]] if tuple(k2[0][:2]) != tuple(k2[0][2:]) else k2[0]
    bad = np.array([[5, 6, 1, 2]], dtype=np.int32)
    with pytest.raises(cg.CosmoError) as e:
        cg.Problem.from_terms(g["sps"], 12, 2, 2, 0, 0, g["esp_keys"], g["esp_vals"], bad, np.array([1.0]))
    assert e.value.status == -1


def _header_struct(hdr, name):
    """(member name, byte size) in declaration order of `typedef struct {...} name;`."""
    import re
    body = re.search(r"typedef struct \{([^{}]*)\}\s*" + name + r";", hdr).group(1)
    body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
    sizes = {"int32_t": 4, "uint32_t": 4, "int64_t": 8, "uint64_t": 8, "double": 8, "float": 4}
    out = []
    for decl in body.split(";"):
        decl = decl.strip()
        if not decl:
            continue
        m = re.match(r"(?:const\s+)?([A-Za-z_0-9]+)\s*(.*)$", " ".join(decl.split()))
        assert m, decl
        for var in m.group(2).split(","):
            var = var.strip()
            out.append((var.lstrip("*").strip(), 8 if var.startswith("*") else sizes[m.group(1)]))
    return out


def test_python_structs_mirror_header():
    """Every ctypes structure of the Python mirror has the members, order and
    sizes of its C struct in include/cosmo_gb300.h (a mismatch would let the
    library write past the Python object), and cg_davidson_defaults fills the
    documented defaults."""
    import ctypes
    import cosmo_gb300 as cg
    hdr = open(os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include",
                            "cosmo_gb300.h")).read()
    pairs = {"cg_problem_info": cg.ProblemInfo, "cg_problem_desc": cg.ProblemDesc,
             "cg_hamiltonian_info": cg.HamiltonianInfo, "cg_spmm_format_info": cg.SpmmFormatInfo,
             "cg_davidson_params": cg.DavidsonParams, "cg_davidson_stats": cg.DavidsonStats,
             "cg_batch_params": cg.BatchParams, "cg_batch_stats": cg.BatchStats}
    for cname, py in pairs.items():
        want = _header_struct(hdr, cname)
        got = [(f[0], ctypes.sizeof(f[1])) for f in py._fields_]
        assert got == want, (cname, got, want)
    p = cg.davidson_params(10)
    assert (p.block, p.lim, p.ortho_pip, p.refine_block, p.refine_fp32_corrections) == (10, 30, 1, 0, 1)
    assert (p.keep, p.refine_keep, p.algorithm, p.precond) == (0, 0, -1, 1)


@pytest.mark.parametrize("name", ["psd22m0_hw2", "psd32m1_hwr13", "psd22m0_hw2_rej", "psd21m1_rej", "sdp22m0_hw2"])
def test_oracle_truncated_basis_matches_reference(name, tmp_path):
    """Truncated bases (oscillator-quanta limits and orbital-occupation
    rejections of the reference's XsysmbsOMP, on p+sd spaces): the oracle's
    filter of the untruncated basis equals the reference's .mbs, byte for
    byte (fixtures from tests/golden/make_golden.py)."""
    import hashlib
    import sys
    import cosmo_gb300 as cg
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
    import truncated as T
    m = manifest()[name]
    p = cg.Problem(T.write_case(str(tmp_path), name))
    inf = p.info
    hw, rej = T.truncation(name)
    assert [hw, rej] == [tuple(m["truncation"]["hw"]) if m["truncation"]["hw"] else None,
                         [(a, b, list(c)) for a, b, c in m["truncation"]["rejections"]]]
    z = O.basis_truncated(p.sps(), inf.nv, inf.zv, inf.twom, inf.parity, hw, rej)
    assert z.shape == (m["n"], m["N"])
    assert np.array_equal(z, golden(name)["mbs"])
    raw = np.int32(m["N"]).tobytes() + np.uint64(m["n"]).tobytes() + z.astype("<u2").tobytes()
    assert hashlib.sha256(raw).hexdigest() == m["mbs_sha256"]
    # every truncation drops determinants of the untruncated basis, none is added
    full = O.basis(p.sps(), inf.nv + inf.zv, inf.twom, inf.nv - inf.zv, inf.parity)
    assert 0 < len(z) < len(full)


def test_truncated_system_loads_and_parses(tmp_path):
    """Systems with basis truncations (hwmax as an attribute or as a child
    element, <hwrejection>, <rejection>) load; a malformed <hwrejection>
    without HWMAX is a parse error.  The truncated bases themselves are built
    and checked on the GPU (tests/test_truncated.py)."""
    import sys
    import cosmo_gb300 as cg
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
    import truncated as T
    for name in T.CASES:
        p = cg.Problem(T.write_case(str(tmp_path), name))
        assert len(p.sps()) == 36
    xml = T.write_case(str(tmp_path), "psd32m1_hwr13")
    bad = tmp_path / "bad.xml"
    bad.write_text(open(xml).read().replace(' HWMAX="3"', "", 1))
    with pytest.raises(cg.CosmoError) as e:
        cg.Problem(str(bad))
    assert e.value.status == -3 and "HWMAX" in str(e.value)
