"""Wide valence spaces (a species with more than 32 m-states): the spsdpf
space of the reference's 33Al example, 20 neutrons and 13 protons in 40
m-states each, in its 0 hw (119 states) and 1 hw (23,842 states) windows,
pinned to the reference run on the same XML (tests/golden/wide.py,
make_golden.py): the oracle's pruned enumeration and the GPU basis equal the
reference's .mbs byte for byte; the operator terms equal the reference's dump;
the Hamiltonian rows equal the reference's PPMatrix2CSBBlk rows (bit-exact
connectivity, values within 1e-12); eigenvalues within 1e-6 MeV of the
reference's Davidson (and of the dense spectrum of its rows); <J-J+> and
<T-T+> of the reference's vectors within 1e-9.  The wide representation
forced on bitstring-sized systems gives the same basis, rows, <J-J+>, <T-T+>
and occupations as the bitstring path."""
import os
import sys

import numpy as np
import pytest

from conftest import GOLDEN, conn_hash, golden, manifest, mbs_sha, problem_for
from oracle import oracle as O

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
import truncated as T  # noqa: E402
import wide as W  # noqa: E402

CASES = sorted(W.CASES)


@pytest.mark.parametrize("name", CASES)
def test_oracle_pruned_basis_matches_reference(name, tmp_path):
    import cosmo_gb300 as cg
    p = cg.Problem(W.write_case(str(tmp_path), name))
    inf = p.info
    assert inf.n_sps == 80
    z = O.basis_pruned(p.sps(), inf.nv, inf.zv, inf.twom, inf.parity, hw=W.CASES[name]["hw"])
    m = manifest()[name]
    assert z.shape == (m["n"], m["N"])
    assert mbs_sha(z) == m["mbs_sha256"]


@pytest.mark.parametrize("name", sorted(T.CASES))
def test_oracle_pruned_equals_filtered(name, tmp_path):
    """The pruned enumeration against the filter of the untruncated basis."""
    import cosmo_gb300 as cg
    p = cg.Problem(T.write_case(str(tmp_path), name))
    inf = p.info
    hw, rej = T.truncation(name)
    a = O.basis_truncated(p.sps(), inf.nv, inf.zv, inf.twom, inf.parity, hw=hw, rejections=rej)
    b = O.basis_pruned(p.sps(), inf.nv, inf.zv, inf.twom, inf.parity, hw=hw, rejections=rej)
    assert np.array_equal(a, b)


@pytest.mark.parametrize("name", ["spsdpf_0hw", "spsdpf_21"])
def test_oracle_rows_wide_match_reference(name, tmp_path):
    """The oracle's tuple-based row builder (no width limit on the s.p.
    index) on the pruned basis: the reference's rows, connectivity bit-exact,
    values within 1e-12."""
    import cosmo_gb300 as cg
    m, g = manifest()[name], golden(name)
    p = cg.Problem(W.write_case(str(tmp_path), name))
    inf = p.info
    z = O.basis_pruned(p.sps(), inf.nv, inf.zv, inf.twom, inf.parity, hw=W.CASES[name]["hw"])
    k1, v1 = p.one_body()
    k2, v2 = p.two_body()
    rp, c, v = O.build_upper(inf.n_sps, k1, v1, k2, v2, z)
    assert conn_hash(rp, c) == m["conn_sha256"]
    np.testing.assert_allclose(v, g["vals"], rtol=0, atol=1e-12)


def test_wide_operator_terms_match_reference(tmp_path):
    import cosmo_gb300 as cg
    g = golden("spsdpf_0hw")
    p = cg.Problem(W.write_case(str(tmp_path), "spsdpf_0hw"))
    assert np.array_equal(p.sps(), g["sps"])
    k1, v1 = p.one_body()
    k2, v2 = p.two_body()
    assert np.array_equal(k1, g["esp_keys"]) and np.array_equal(v1, g["esp_vals"])
    assert np.array_equal(k2, g["vspx_keys"])
    np.testing.assert_allclose(v2, g["vspx_vals"], rtol=0, atol=1e-13)


def test_wide_problem_from_terms(tmp_path):
    """A problem built from an explicit 80-state table and operator terms
    (cg_problem_create) holds them unchanged; more than 64 states in a
    species is refused."""
    import cosmo_gb300 as cg
    g = golden("spsdpf_0hw")
    p = cg.Problem(W.write_case(str(tmp_path), "spsdpf_0hw"))
    k1, v1 = p.one_body()
    k2, v2 = p.two_body()
    q = cg.Problem.from_terms(p.sps(), 40, 20, 13, 1, 0, k1, v1, k2, v2)
    assert q.info.n_sps == 80 and np.array_equal(q.sps(), g["sps"])
    r1, w1 = q.one_body()
    r2, w2 = q.two_body()
    assert np.array_equal(r1, k1) and np.array_equal(w1, v1)
    assert np.array_equal(r2, k2) and np.array_equal(w2, v2)
    big = np.concatenate([p.sps()[:40]] * 2)  # 80 neutron states
    with pytest.raises(cg.CosmoError):
        cg.Problem.from_terms(big, 80, 2, 0, 0, 0, k1[:0], v1[:0], k2[:0], v2[:0])


@pytest.mark.gpu
@pytest.mark.parametrize("name", CASES)
def test_wide_basis_matches_reference(gpu_available, name, tmp_path):
    import cosmo_gb300 as cg
    m = manifest()[name]
    b = cg.ManyBodyStates(cg.Problem(W.write_case(str(tmp_path), name)))
    assert b.wide and (b.n, b.N) == (m["n"], m["N"])
    z = b.states()
    assert mbs_sha(z) == m["mbs_sha256"]
    assert np.array_equal(b.locate(z), np.arange(b.n))
    # misses: a wrongly ordered tuple and, in a truncated window, a determinant
    # two oscillator quanta up (two sd protons moved into the fp shell, M and
    # parity kept)
    d = [int(x) for x in z[0]]
    swapped = list(d)
    swapped[0], swapped[1] = swapped[1], swapped[0]
    probes = [swapped]
    if W.CASES[name]["hw"] is not None:
        sps = cg.Problem(W.write_case(str(tmp_path), name)).sps()
        q = 2 * sps[:, 1] + sps[:, 2]
        occ = set(d)
        sd = [i for i in d if i >= 40 and q[i] == 2]
        fp = [i for i in range(40, 80) if q[i] == 3 and i not in occ]
        probes.append(next(sorted(set(d) - {a, b2} | {c, e}) for a in sd for b2 in sd if a < b2 for c in fp
                           for e in fp if c < e and sps[a, 4] + sps[b2, 4] == sps[c, 4] + sps[e, 4]))
    out = b.locate(np.array(probes, dtype=np.uint16))
    assert list(out) == [b.n + 1] * len(probes)


@pytest.mark.gpu
@pytest.mark.parametrize("name", CASES)
def test_wide_hamiltonian_rows_match_reference(gpu_available, name, tmp_path):
    import cosmo_gb300 as cg
    m, g = manifest()[name], golden(name)
    p = cg.Problem(W.write_case(str(tmp_path), name))
    b = cg.ManyBodyStates(p)
    h = cg.Hamiltonian(p, b, cg.CG_PREC_FP64)
    rp, c, v = h.upper_rows()
    assert int(rp[-1]) == m["nnz_upper"]
    assert conn_hash(rp, c) == m["conn_sha256"]
    if "vals" in g:
        np.testing.assert_allclose(v, g["vals"], rtol=0, atol=1e-12)
    else:
        for k, r in enumerate(g["sample_rows"]):
            a, e = int(g["sample_rowptr"][k]), int(g["sample_rowptr"][k + 1])
            np.testing.assert_allclose(v[int(rp[r]):int(rp[r + 1])], g["sample_vals"][a:e], rtol=0, atol=1e-12)


@pytest.mark.gpu
def test_wide_spectrum_0hw(gpu_available, tmp_path):
    """All 119 states: the exact path against the dense spectrum of the
    reference's rows, both Davidson engines against the reference's."""
    import cosmo_gb300 as cg
    g = golden("spsdpf_0hw")
    H = O.full_from_upper(g["rowptr"], g["cols"], g["vals"]).toarray()
    exact = np.linalg.eigvalsh(H)
    p = cg.Problem(W.write_case(str(tmp_path), "spsdpf_0hw"))
    b = cg.ManyBodyStates(p)
    for prec in (cg.CG_PREC_FP64, cg.CG_PREC_FP32):
        h = cg.Hamiltonian(p, b, prec)
        eig, _ = h.dense_eigensolve()
        np.testing.assert_allclose(eig, exact, rtol=0, atol=1e-9)
        r = cg.davidson_diagonalization(h, 10, precision=prec, tol_resid=1e-6, block=10, lim=40, algorithm=1)
        assert r.stats.converged == 10
        np.testing.assert_allclose(r.eig, g["ref_eig"][:10], rtol=0, atol=1e-6)


@pytest.mark.gpu
def test_wide_davidson_1hw(gpu_available, tmp_path):
    import cosmo_gb300 as cg
    g = golden("spsdpf_1hw")
    p = cg.Problem(W.write_case(str(tmp_path), "spsdpf_1hw"))
    b = cg.ManyBodyStates(p)
    h = cg.Hamiltonian(p, b, cg.CG_PREC_FP32)
    r = cg.davidson_diagonalization(h, 5, want_vectors=True, precision=cg.CG_PREC_FP32, tol_resid=1e-6, block=5,
                                    lim=48)
    assert r.stats.converged == 5
    np.testing.assert_allclose(r.eig, g["ref_eig"][:5], rtol=0, atol=1e-6)
    jj, tt = cg.jt_expectations(b, r.vecs)
    for q in jj:  # 2J of the M = 1/2 states: odd integers
        x = np.sqrt(4 * q + 1 * 3 + 1) - 1
        assert abs(x - round(x)) < 1e-5 and round(x) % 2 == 1, jj


@pytest.mark.gpu
def test_wide_jt_of_reference_vectors(gpu_available, tmp_path):
    import cosmo_gb300 as cg
    m, g = manifest()["spsdpf_0hw"], golden("spsdpf_0hw")
    p = cg.Problem(W.write_case(str(tmp_path), "spsdpf_0hw"))
    b = cg.ManyBodyStates(p)
    vecs = g["ref_vecs"]
    jj, tt = cg.jt_expectations(b, vecs)
    np.testing.assert_allclose(jj, m["ref_jj"], rtol=0, atol=1e-9)
    np.testing.assert_allclose(tt, m["ref_tt"], rtol=0, atol=1e-9)
    occ = cg.occupations(b, vecs)
    assert occ.shape == (len(vecs), 80)
    np.testing.assert_allclose(occ.sum(1), 33.0, rtol=0, atol=1e-9)
    np.testing.assert_allclose(occ[:, :40].sum(1), 20.0, rtol=0, atol=1e-9)


@pytest.mark.gpu
@pytest.mark.parametrize("name", CASES)
def test_wide_on_the_fly_matches_stored(gpu_available, name, tmp_path):
    """The on-the-fly product of a wide basis (64-bit species masks, the
    class-to-list maps of the truncated tables) equals the stored matrix's:
    diagonal within 1e-12, FP64 and double-float within 1e-11 of max |y|,
    FP32 within 1e-5."""
    import cosmo_gb300 as cg
    p = cg.Problem(W.write_case(str(tmp_path), name))
    b = cg.ManyBodyStates(p)
    hs = cg.Hamiltonian(p, b, cg.CG_PREC_FP64)
    hv = cg.Hamiltonian(p, b, cg.CG_PREC_FP64, virtual=True)
    assert hv.virtual
    np.testing.assert_allclose(hv.diagonal(), hs.diagonal(), rtol=0, atol=1e-12)
    for m in (1, 5, 8):
        x = np.random.default_rng(m).standard_normal((b.n, m))
        ys = hs.times_matrix(x)
        scale = np.abs(ys).max()
        np.testing.assert_allclose(hv.times_matrix(x), ys, rtol=0, atol=1e-11 * scale)
        np.testing.assert_allclose(hv.times_matrix(x, cg.CG_PREC_FP32), ys, rtol=0, atol=1e-5 * scale)
        np.testing.assert_allclose(hv.times_matrix(x, cg.CG_PREC_REFINE), ys, rtol=0, atol=1e-11 * scale)


@pytest.mark.gpu
def test_wide_on_the_fly_davidson_and_forced(gpu_available, tmp_path):
    """Mixed Davidson on the wide on-the-fly product reaches the reference's
    1 hw eigenvalues; forced on bitstring-sized systems the wide on-the-fly
    product equals the bitstring one's."""
    import cosmo_gb300 as cg
    g = golden("spsdpf_1hw")
    p = cg.Problem(W.write_case(str(tmp_path), "spsdpf_1hw"))
    b = cg.ManyBodyStates(p)
    hv = cg.Hamiltonian(p, b, cg.CG_PREC_FP32, virtual=True)
    r = cg.davidson_diagonalization(hv, 5, precision=cg.CG_PREC_FP32, tol_resid=1e-6, block=5, lim=40)
    assert r.stats.converged == 5
    np.testing.assert_allclose(r.eig, g["ref_eig"][:5], rtol=0, atol=1e-6)
    for name, pp in _narrow_cases(str(tmp_path)):
        bn, bw = cg.ManyBodyStates(pp), cg.ManyBodyStates(pp, wide=True)
        hn = cg.Hamiltonian(pp, bn, cg.CG_PREC_FP64, virtual=True)
        hw = cg.Hamiltonian(pp, bw, cg.CG_PREC_FP64, virtual=True)
        x = np.random.default_rng(3).standard_normal((bn.n, 8))
        yn = hn.times_matrix(x)
        np.testing.assert_allclose(hw.times_matrix(x), yn, rtol=0, atol=1e-11 * np.abs(yn).max(), err_msg=name)


def _narrow_cases(tmp):
    out = [(n, problem_for(n, tmp)) for n in ("sd22m0s1", "fp21m3s6", "sd32m1s2")]
    import cosmo_gb300 as cg
    out += [(n, cg.Problem(T.write_case(tmp, n))) for n in ("psd22m0_hw2_rej", "psd32m1_hwr13")]
    return out


@pytest.mark.gpu
def test_wide_forced_equals_bitstring(gpu_available, tmp_path):
    import cosmo_gb300 as cg
    for name, p in _narrow_cases(str(tmp_path)):
        bn = cg.ManyBodyStates(p)
        bw = cg.ManyBodyStates(p, wide=True)
        assert bw.wide and not bn.wide and bw.n == bn.n, name
        z = bn.states()
        assert np.array_equal(bw.states(), z), name
        assert np.array_equal(bw.locate(z), np.arange(bn.n)), name
        hn = cg.Hamiltonian(p, bn, cg.CG_PREC_FP64)
        hw = cg.Hamiltonian(p, bw, cg.CG_PREC_FP64)
        rn, cn, vn = hn.upper_rows()
        rw, cw, vw = hw.upper_rows()
        assert np.array_equal(rn, rw) and np.array_equal(cn, cw), name
        np.testing.assert_allclose(vw, vn, rtol=0, atol=1e-13)
        np.testing.assert_allclose(hw.diagonal(), hn.diagonal(), rtol=0, atol=1e-13)
        k = min(4, bn.n)
        r = cg.davidson_diagonalization(hn, k, want_vectors=True, precision=cg.CG_PREC_FP64, tol_resid=1e-8,
                                        block=k, lim=min(bn.n, 4 * k), algorithm=1)
        jn, tn = cg.jt_expectations(bn, r.vecs)
        jw, tw = cg.jt_expectations(bw, r.vecs)
        np.testing.assert_allclose(jw, jn, rtol=0, atol=1e-9)
        np.testing.assert_allclose(tw, tn, rtol=0, atol=1e-9)
        np.testing.assert_allclose(cg.occupations(bw, r.vecs), cg.occupations(bn, r.vecs), rtol=0, atol=1e-12)


def _random_terms(sps, rng, same_species=True):
    """Random one-body terms (i, f, v) that keep species, m and parity."""
    ns = len(sps)
    nn = int((sps[:, 6] > 0).sum())
    out = []
    for i in range(ns):
        for f in range(ns):
            if (i < nn) != (f < nn) or sps[i, 4] != sps[f, 4] or sps[i, 7] != sps[f, 7]:
                continue
            out.append((i, f, float(rng.standard_normal())))
    return out


@pytest.mark.gpu
def test_wide_forced_amplitudes_equal_bitstring(gpu_available, tmp_path):
    """Transition (XSHLEMB) and removal (XSHLSF) amplitudes on wide bases equal
    the bitstring kernels' on the same systems and vectors."""
    import cosmo_gb300 as cg
    from cosmo_gb300.synthetic import SyntheticSystem, make_system
    rng = np.random.default_rng(5)
    pp = problem_for("sd22m0s1", str(tmp_path))
    pd = cg.Problem(make_system(str(tmp_path), SyntheticSystem("sd", 2, 1, 1, "+", 0.5, 1, name="sd21m1s1"))[1])
    bpn, bpw = cg.ManyBodyStates(pp), cg.ManyBodyStates(pp, wide=True)
    bdn, bdw = cg.ManyBodyStates(pd), cg.ManyBodyStates(pd, wide=True)
    vp = rng.standard_normal((3, bpn.n))
    vd = rng.standard_normal((4, bdn.n))
    np.testing.assert_allclose(cg.sf_amplitudes(bpw, vp, bdw, vd), cg.sf_amplitudes(bpn, vp, bdn, vd),
                               rtol=0, atol=1e-12)
    terms = _random_terms(pp.sps(), rng)
    vq = rng.standard_normal((5, bpn.n))
    np.testing.assert_allclose(cg.onebody_amplitudes(bpw, vp, bpw, vq, terms),
                               cg.onebody_amplitudes(bpn, vp, bpn, vq, terms), rtol=0, atol=1e-12)
    with pytest.raises(cg.CosmoError):
        cg.onebody_amplitudes(bpw, vp, bpn, vq, terms)


@pytest.mark.gpu
def test_wide_onebody_amplitudes_spsdpf(gpu_available, tmp_path):
    """Transition amplitudes between the reference's 0 hw spsdpf vectors on
    the GPU against the oracle's pull over the reference's .mbs tuples."""
    import cosmo_gb300 as cg
    from oracle import transitions as TR
    g = golden("spsdpf_0hw")
    p = cg.Problem(W.write_case(str(tmp_path), "spsdpf_0hw"))
    b = cg.ManyBodyStates(p)
    vecs = g["ref_vecs"]
    terms = _random_terms(p.sps(), np.random.default_rng(7))
    amp = cg.onebody_amplitudes(b, vecs, b, vecs[:8], terms)
    ref = TR.onebody_amplitudes(g["mbs"], vecs, g["mbs"], vecs[:8], terms)
    np.testing.assert_allclose(amp, ref, rtol=0, atol=1e-11 * max(1.0, np.abs(ref).max()))


@pytest.mark.gpu
def test_wide_cli_example_flow(gpu_available, tmp_path):
    """The command-line flow of the reference's 33Al example (basis tool,
    DEXHVJTcsb, Xlevels, XSHLAO) on the two spsdpf windows: cg_xsysmbs writes
    the reference's .mbs; cg_dexhvjt diagonalizes the 119-state window exactly
    (every state in the .EE, the <state> records of the reference's XSHLJT)
    and the 23,842-state one by Davidson; cg_xlevels lists both systems'
    states; cg_xshlao writes occupations."""
    import hashlib
    import re
    import subprocess
    import cosmo_gb300 as cg
    bindir = os.path.join(os.path.dirname(cg.__file__), "bin")
    work = str(tmp_path)

    def run(*args):
        r = subprocess.run([os.path.join(bindir, args[0])] + list(args[1:]), cwd=work, capture_output=True,
                           text=True, stdin=subprocess.DEVNULL)
        assert r.returncode == 0, r.stderr
        return r
    m0, m1 = manifest()["spsdpf_0hw"], manifest()["spsdpf_1hw"]
    xml0 = W.write_case(work, "spsdpf_0hw")
    xml1 = W.write_case(work, "spsdpf_1hw")
    for xml, m, tag in ((xml0, m0, "a"), (xml1, m1, "b")):
        run("cg_xsysmbs", xml, "-o", tag + ".mbs")
        assert hashlib.sha256(open(os.path.join(work, tag + ".mbs"), "rb").read()).hexdigest() == m["mbs_sha256"]
    r = run("cg_dexhvjt", xml0, "-n", "10", "-o", "out0.xml")
    assert "exact diagonalization" in r.stderr
    E, D, R, V = cg.read_ee(os.path.join(work, "spsdpf_0hw.HH.EE"))
    g = golden("spsdpf_0hw")
    exact = np.linalg.eigvalsh(O.full_from_upper(g["rowptr"], g["cols"], g["vals"]).toarray())
    assert len(E) == 119
    np.testing.assert_allclose(E, exact, rtol=0, atol=1e-9)
    txt = open(os.path.join(work, "out0.xml")).read()
    states = [dict(re.findall(r'(\w+)="([^"]*)"', x)) for x in re.findall(r"<state ([^>]*)>", txt)]
    ref_states = m0["ref_xshljt_states"]
    assert [s["J"] for s in states] == [s["J"] for s in ref_states]
    assert [s["name"] for s in states] == [s["name"] for s in ref_states]
    for a, b in zip(states, ref_states):
        assert abs(float(a["E"]) - float(b["E"])) < 2e-4
    run("cg_dexhvjt", xml1, "-n", "5", "-o", "out1.xml")
    E1, _, R1, _ = cg.read_ee(os.path.join(work, "spsdpf_1hw.HH.EE"))
    assert np.all(R1 <= 1e-5)
    np.testing.assert_allclose(E1, m1["ref_eig"][:5], rtol=0, atol=1e-4)
    lv = run("cg_xlevels", "out0.xml", "out1.xml", "-o", "levels.xml")
    assert len(lv.stdout.splitlines()) >= len(states) + 1
    run("cg_xshlao", "out0.xml", "-o", "ao.xml")
    assert len(re.findall(r"<occupation ", open(os.path.join(work, "ao.xml")).read())) > 0


@pytest.mark.gpu
def test_wide_xshlemb_matches_reference(gpu_available, tmp_path):
    """Step 5 of the 33Al example on the spsdpf 0 hw window: E2 transitions
    (-w -u, en 0.5, ep 1.5) among the reference's own lowest states (its .EE
    and XSHLJT <state> nodes); B, Weisskopf and Bu within 1e-6 + 1e-5
    relative of the 6 digits the reference XSHLEMB writes."""
    import re
    import cosmo_gb300 as cg
    m = manifest()["em_wide"]
    work = str(tmp_path)
    xml = W.write_case(work, "spsdpf_0hw")
    txt = open(xml).read().replace("<system ", '<system A="33" ', 1)
    jj = re.search(r'<matrix JJ="([^"]*)"/>', txt)
    txt = txt.replace(jj.group(0), f'<matrix name="spsdpf_0hw" format="pp" JJ="{jj.group(1)}"/>')
    txt = txt.replace("</system>", "".join(m["states"]) + "</system>", 1)
    pin = os.path.join(work, "em_wide.xml")
    open(pin, "w").write(txt.replace("</cosmo>", m["operator"] + "\n</cosmo>", 1))
    np.load(os.path.join(GOLDEN, "em_wide.npz"))["EE"].tofile(os.path.join(work, "spsdpf_0hw.EE"))
    out = os.path.join(work, "out.xml")
    cg.xshlemb(pin, out, weisskopf=True, units=True)

    def attrs(t):
        return dict(re.findall(r'(\w+)="([^"]*)"', t))
    mine = re.findall(r"<state [^>]*>.*?</state>", open(out).read(), re.S)
    ref = m["out_states"]
    assert len(mine) == len(ref) and sum(x.count("<transition") for x in ref) > 0
    for a, b in zip(mine, ref):
        ta = [attrs(t) for t in re.findall(r"<transition [^>]*/>", a)]
        tb = [attrs(t) for t in re.findall(r"<transition [^>]*/>", b)]
        assert [t["final"] for t in ta] == [t["final"] for t in tb]
        for x, y in zip(ta, tb):
            for key in ("B", "weisskopf", "Bu"):
                assert abs(float(x[key]) - float(y[key])) <= 1e-6 + 1e-5 * abs(float(y[key])), (key, x, y)


@pytest.mark.gpu
def test_wide_untruncated_spectrum_and_product(gpu_available, tmp_path):
    """Untruncated wide basis (2 neutrons and 1 proton in the spsdpf space):
    the stored product against the reference's SpMM output, the 5 lowest
    states against the reference's Davidson, <J-J+> and <T-T+> of the
    reference's vectors."""
    import cosmo_gb300 as cg
    m, g = manifest()["spsdpf_21"], golden("spsdpf_21")
    p = cg.Problem(W.write_case(str(tmp_path), "spsdpf_21"))
    b = cg.ManyBodyStates(p)
    assert b.wide and b.n == m["n"]
    h = cg.Hamiltonian(p, b, cg.CG_PREC_FP64)
    y = h.times_matrix(g["spmm_x"].T.copy())
    np.testing.assert_allclose(y, g["spmm_y"].T, rtol=0, atol=1e-11 * np.abs(g["spmm_y"]).max())
    r = cg.davidson_diagonalization(h, 5, precision=cg.CG_PREC_FP64, tol_resid=1e-7, block=5, lim=40, algorithm=1)
    assert r.stats.converged == 5
    np.testing.assert_allclose(r.eig, g["ref_eig"], rtol=0, atol=1e-6)
    jj, tt = cg.jt_expectations(b, g["ref_vecs"])
    np.testing.assert_allclose(jj, m["ref_jj"], rtol=0, atol=1e-9)
    np.testing.assert_allclose(tt, m["ref_tt"], rtol=0, atol=1e-9)


@pytest.mark.gpu
def test_wide_batched(gpu_available, tmp_path):
    """Wide and bitstring systems solved together in lockstep (the batched
    solver takes the wide bases' rows like any other)."""
    import cosmo_gb300 as cg
    probs = [cg.Problem(W.write_case(str(tmp_path), "spsdpf_0hw")),
             cg.Problem(W.write_case(str(tmp_path), "spsdpf_21")), problem_for("sd22m0s1", str(tmp_path))]
    eig, res, nconv, _ = cg.Batch(probs).solve(3)
    np.testing.assert_allclose(eig[0], golden("spsdpf_0hw")["ref_eig"][:3], rtol=0, atol=1e-4)
    np.testing.assert_allclose(eig[1], golden("spsdpf_21")["ref_eig"][:3], rtol=0, atol=1e-4)
    np.testing.assert_allclose(eig[2], golden("sd22m0s1")["ref_eig"][:3], rtol=0, atol=1e-4)


def test_example_33al_known_answers(tmp_path):
    """The reference's 33Al example with its fsu9 interaction (needs the
    reference checkout, COSMO_REFERENCE; skipped elsewhere): the basis tool's
    counts (119 and 23,842, the oracle's pruned enumeration) and the levels
    the example prints (5/2+ at -303.079 MeV; 1/2-, 7/2-, 5/2-, 3/2- at
    -301.132, -299.928, -299.874, -299.817) from the library's operator terms
    and the oracle's rows of both windows (about a minute of CPU for the
    23,842 rows)."""
    root = O.reference_root()
    int_dir = os.path.join(root, "interactions", "spsdpf") if root else ""
    if not os.path.exists(os.path.join(int_dir, "fsu9", "spsdfp-fsu9.int")):
        pytest.skip("reference checkout not given (COSMO_REFERENCE)")
    import cosmo_gb300 as cg
    for parity, (lo, hi, n) in W.EXAMPLE_33AL.items():
        p = cg.Problem(W.write_33al(str(tmp_path), int_dir, parity))
        inf = p.info
        z = O.basis_pruned(p.sps(), inf.nv, inf.zv, inf.twom, inf.parity, hw=(lo, hi))
        assert len(z) == n
        k1, v1 = p.one_body()
        k2, v2 = p.two_body()
        rp, c, v = O.build_upper(inf.n_sps, k1, v1, k2, v2, z)
        H = O.full_from_upper(rp, c, v)
        if parity == "+":
            e = np.linalg.eigvalsh(H.toarray())
            assert abs(e[0] - W.EXAMPLE_33AL_LEVELS[0][1]) < 5e-4
        else:
            import scipy.sparse.linalg as sla
            e = np.sort(sla.eigsh(H, k=4, which="SA", tol=1e-10)[0])
            np.testing.assert_allclose(e, [x for _, x in W.EXAMPLE_33AL_LEVELS[1:]], rtol=0, atol=5e-4)
