"""Spin / isospin analysis (XSHLJT) on the GPU against the reference.

<J-J+> and <T-T+> of the reference's own eigenvectors are pinned to the
values the reference's PPMatrix::Sqr computes (oracle/_ref/ref_jt, golden
fixtures); 2J assignments to the reference's SM::JJSpin; the <state> nodes
written into the system XML to the ones the reference XSHLJT writes (except
T, which the reference derives from an unset Tz for these XML files; here
2Tz = Nv - Zv).  Tolerance: 1e-9 absolute on <J-J+> and <T-T+> (FP64 sums of
up to 1e5 terms of O(1))."""
import os

import numpy as np
import pytest

import cosmo_gb300 as cg
from conftest import golden, manifest, problem_for

FULL = ["sd22m0s1", "sd32m1s2", "fp21m3s6"]


def test_jj_spin_host():
    """SM::JJSpin: 2J = sqrt(4x + 2M(2M+2) + 1) - 1 when J + M is integral within 0.1."""
    assert cg.jj_spin(0.0, 0) == 0
    assert cg.jj_spin(2.0, 0) == 2
    assert cg.jj_spin(6.0, 0) == 4
    assert cg.jj_spin(0.0, 1) == 1          # J = 1/2, M = 1/2
    assert cg.jj_spin(3.0, 1) == 3          # J = 3/2, M = 1/2: 15/4 - 3/4
    assert cg.jj_spin(1.0, 0) == -1         # J(J+1) = 1 has no (half-)integer J
    assert cg.jj_spin(2.0 + 0.05, 0) == 2   # inside the 0.1 window


@pytest.mark.gpu
@pytest.mark.parametrize("name", FULL)
def test_jt_matches_reference(gpu_available, name, tmp_path):
    m = manifest()[name]
    g = golden(name)
    p = problem_for(name, str(tmp_path))
    b = cg.ManyBodyStates(p)
    jj, tt = cg.jt_expectations(b, g["ref_vecs"])
    np.testing.assert_allclose(jj, m["ref_jj"], rtol=0, atol=1e-9)
    np.testing.assert_allclose(tt, m["ref_tt"], rtol=0, atol=1e-9)
    twom = p.info.twom
    assert [cg.jj_spin(x, twom) for x in jj] == m["ref_twoJ"]


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["mg24usdb", "sd66m0s5"])
def test_jt_of_gpu_solve(gpu_available, name, tmp_path):
    """Mixed-precision eigenvectors: <J-J+> within 1e-6 of J(J+1) (integral J
    at M = 0), and the reference's spin sequence where it is pinned."""
    p = problem_for(name, str(tmp_path))
    b = cg.ManyBodyStates(p)
    h = cg.Hamiltonian(p, b, cg.CG_PREC_FP32)
    r = cg.davidson_diagonalization(h, 10, want_vectors=True, precision=cg.CG_PREC_FP32, tol_resid=1e-5)
    jj, tt = cg.jt_expectations(b, r.vecs)
    twoJ = np.array([cg.jj_spin(x, 0) for x in jj])
    assert np.all(twoJ >= 0) and np.all(twoJ % 2 == 0)
    J = twoJ / 2
    np.testing.assert_allclose(jj, J * (J + 1), rtol=0, atol=1e-6)
    m = manifest()[name]
    if "ref_twoJ" in m:
        assert list(twoJ) == m["ref_twoJ"]


@pytest.mark.gpu
@pytest.mark.parametrize("name", FULL)
def test_xshljt_states_match_reference(gpu_available, name, tmp_path):
    """XSHLJT end to end: .EE with the reference's eigenpairs -> <state> nodes."""
    from cosmo_gb300.synthetic import SyntheticSystem, make_system
    m = manifest()[name]
    g = golden(name)
    s = m["system"]
    sysd = SyntheticSystem(s["space"], s["nv"], s["zv"], s["twom"], s["parity"], s["jj"], s["seed"], name=name)
    xml = make_system(str(tmp_path), sysd)[1]
    ee = os.path.join(str(tmp_path), name + ".EE")
    cg.write_ee(ee, g["ref_eig"], g["ref_de"], g["ref_resid"], g["ref_vecs"])
    out = os.path.join(str(tmp_path), "out.xml")
    k = cg.xshljt(xml, ee, len(g["ref_eig"]), out, system=name)
    assert k == len(g["ref_eig"])
    txt = open(out).read()
    import re
    states = [dict(re.findall(r'(\w+)="([^"]*)"', x)) for x in re.findall(r"<state ([^>]*)>", txt)]
    ref = m["ref_xshljt_states"]
    assert len(states) == len(ref)
    for a, r in zip(states, ref):
        for key in ("J", "P", "E", "name", "Ex"):
            assert a[key] == r[key], (key, a, r)
        assert float(a["dE"]) == pytest.approx(float(r["dE"]), abs=1e-12)
    # attribute order of the reference writer
    first = re.search(r"<state ([^>]*)>", txt).group(1)
    assert [kv.split("=")[0] for kv in first.split()] == ["J", "P", "T", "E", "dE", "name", "Ex"]
    # the rest of the file is untouched
    before = open(xml).read()
    assert txt.startswith(before[:before.index("<system")])
    # a second pass merges into the existing states (same J, T, E): no new nodes
    k2 = cg.xshljt(out, ee, len(g["ref_eig"]), out, system=name)
    assert k2 == k
    assert len(re.findall(r"<state ", open(out).read())) == len(ref)
