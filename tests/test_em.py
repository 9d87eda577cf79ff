"""Electromagnetic and beta transitions (the reference's XSHLEMB,
xmlshell/XSHLEMB.cpp): the oracle's one-body operators, overlaps and B values
against the <transition>/<moment> nodes the reference XSHLEMB wrote for a
parent sd 2n+2p system (E2, E2 with radial functions positive at infinity,
M1 with the default moments; E2 and M1 to the 2M = 2 states, kappa = 1), for
GT- and F a daughter sd 1n+3p system, and GT+ from that system back
(tests/golden/make_golden.py, em_case), from the reference's own
eigenvectors (.EE files) and <state> nodes; the library's operator terms
against the oracle's; on the GPU the amplitudes against the oracle's and the
tool end to end.  The reference writes 6 significant digits: values are
compared within 1e-6 + 1e-5 relative (moments and B of 0 -> 0 transitions
that are pure rounding noise, ~1e-28, only absolutely)."""
import os
import re

import numpy as np
import pytest

from conftest import GOLDEN, manifest
from oracle import interaction as OI
from oracle import oracle as O
from oracle import transitions as TR

CASE = "em_sd22"


def _attrs(tag_text):
    return dict(re.findall(r'(\w+)="([^"]*)"', tag_text))


def _ee(raw):
    b = raw.tobytes()
    cnt = int(np.frombuffer(b[:4], np.uint32)[0])
    off, vecs, E = 4, [], []
    for _ in range(cnt):
        E.append(float(np.frombuffer(b[off:off + 8], np.float64)[0]))
        n = int(np.frombuffer(b[off + 24:off + 32], np.uint64)[0])
        vecs.append(np.frombuffer(b[off + 32:off + 32 + 8 * n], np.float64).copy())
        off += 32 + 8 * n
    return np.array(vecs), np.array(E)


def _states(name, raw):
    vecs, E = _ee(raw)
    out = []
    for node in manifest()[CASE][name]["states"]:
        st = _attrs(node.split("<wavefunction")[0])
        wf = _attrs(node.split("<wavefunction")[1])
        k = int(wf["id"])
        out.append(dict(name=st["name"], E_text=st["E"], twoJ=OI.spin2(st["J"]), twoT=OI.spin2(st["T"]),
                        twoJz=OI.spin2(wf["Jz"]), twoTz=OI.spin2(wf["Tz"]), E=E[k], vec=vecs[k]))
    return out


def _systems(tmp):
    import sys
    sys.path.insert(0, GOLDEN)
    import make_golden as MG
    g = np.load(os.path.join(GOLDEN, CASE + ".npz"))
    out = {}
    for name, sysd in MG.EM_SYSTEMS:
        A = MG.EM_CORE[sysd.space] + sysd.nv + sysd.zv
        xml = MG.sf_xml(tmp, name, sysd)
        txt = open(xml).read().replace("<system ", f'<system A="{A}" ', 1)
        open(xml, "w").write(txt)
        sp = OI.System(xml)
        z = O.basis(sp.sps, sp.nv + sp.zv, sp.twom, sp.nv - sp.zv, sp.parity)
        out[name] = dict(xml=xml, sys=sp, z=z, states=_states(name, g[name + "_EE"]), ee=g[name + "_EE"], A=A)
    return out


def _op(run):
    a = _attrs(manifest()[CASE]["runs"][run]["operator"])
    op = dict(name=a["name"], K=int(a["J"]), origin_positive="-p" not in manifest()[CASE]["runs"][run]["flags"],
              en=float(a.get("en", 0)), ep=float(a.get("ep", 0)), mu_n=float(a.get("mu_n", TR.MU_N)),
              mu_p=float(a.get("mu_p", TR.MU_P)), gl_n=float(a.get("gl_n", 0)), gl_p=float(a.get("gl_p", 1)))
    return op


def _ref_records(run):
    """Per parent state: [(final, attrs)] of its transitions and [attrs] of its moments."""
    trans, moms = [], []
    for st in manifest()[CASE]["runs"][run]["states"]:
        trans.append([(_attrs(t)["final"], _attrs(t)) for t in re.findall(r"<transition [^>]*/>", st)])
        moms.append([_attrs(m) for m in re.findall(r"<moment [^>]*/>", st)])
    return trans, moms


def _close(x, y):
    return abs(x - y) <= 1e-6 + 1e-5 * abs(y)


def _check_records(run, trans, moms, A):
    rtrans, rmoms = _ref_records(run)
    assert len(trans) == len(rtrans)
    for mine, ref in zip(trans, rtrans):
        assert [r["final"] for r in mine] == [f for f, _ in ref]
        for r, (_, a) in zip(mine, ref):
            for key in ("B", "weisskopf", "Bu", "logft"):
                if key in a:
                    assert key in r and _close(r[key], float(a[key])), (run, key, r, a)
                else:
                    assert key not in r, (run, key)
    for mine, ref in zip(moms, rmoms):
        assert len(mine) == len(ref)
        for r, a in zip(mine, ref):
            assert _close(r["m"], float(a["m"])), (run, r, a)
            if "oscl" in a:
                assert _close(np.sqrt(TR.oscillator_b2(A)), float(a["oscl"]))


def _flags(run):
    return tuple(manifest()[CASE]["runs"][run]["flags"])


RUNS = ("E2", "E2p", "M1", "GT-", "F", "M1k", "E2k", "GT+", "E2fp", "M1fp", "E4fp", "GT-fp")


def _parent(s, run):
    return s[manifest()[CASE]["runs"][run].get("parent", "sd22m0s1")]


@pytest.mark.parametrize("run", RUNS)
def test_oracle_transitions_match_reference(tmp_path, run):
    s = _systems(str(tmp_path))
    parent = _parent(s, run)
    d = manifest()[CASE]["runs"][run]["daughter"]
    daughter = s[d] if d else parent
    op = _op(run)
    kappa = (daughter["sys"].twom - parent["sys"].twom) // 2
    terms = TR.transition_terms(parent["sys"].sps, op, kappa)
    P, D = parent["states"], daughter["states"]
    amp = TR.onebody_amplitudes(parent["z"], np.array([p["vec"] for p in P]), daughter["z"],
                                np.array([q["vec"] for q in D]), terms)
    trans, moms = TR.transitions(op, P, D, amp, A=parent["A"], flags=_flags(run))
    _check_records(run, trans, moms, parent["A"])


@pytest.mark.parametrize("run", RUNS)
def test_library_terms_match_oracle(tmp_path, run):
    """The library's host operator construction against the oracle's, term by term."""
    import cosmo_gb300 as cg
    s = _systems(str(tmp_path))
    parent = _parent(s, run)
    xml = os.path.join(str(tmp_path), "op.xml")
    op_node = manifest()[CASE]["runs"][run]["operator"]
    open(xml, "w").write(open(parent["xml"]).read().replace("</cosmo>", op_node + "\n</cosmo>", 1))
    op = _op(run)
    for kappa in (0, 1, -2):
        if op["name"] == "F" and kappa:
            continue
        mine = sorted(cg.transition_terms(xml, kappa=kappa, phase_infinity=not op["origin_positive"]))
        ref = sorted(TR.transition_terms(parent["sys"].sps, op, kappa))
        assert [(i, f) for i, f, _ in mine] == [(i, f) for i, f, _ in ref]
        assert max((abs(a[2] - b[2]) for a, b in zip(mine, ref)), default=0.0) <= 1e-13


def test_oracle_radial_and_6j_known_values():
    # <0s|r^2|0s> = 3/2, <0p|r^2|0p> = 5/2, <1s|r^2|0s> = -sqrt(3/2) (positive at the origin)
    assert abs(TR.ho_radial(2, 0, 0, 0, 0) - 1.5) < 1e-15
    assert abs(TR.ho_radial(2, 0, 1, 0, 1) - 2.5) < 1e-15
    assert abs(TR.ho_radial(2, 1, 0, 0, 0) + np.sqrt(1.5)) < 1e-15
    assert abs(TR.ho_radial(2, 1, 0, 0, 0, origin_positive=False) - np.sqrt(1.5)) < 1e-15
    # {1/2 1/2 1; 1/2 1/2 0} = 1/2 ... {1 1 1; 1 1 1} = 1/6
    assert abs(TR.six_j(1, 1, 2, 1, 1, 0) - 0.5) < 1e-15
    assert abs(TR.six_j(2, 2, 2, 2, 2, 2) - 1.0 / 6.0) < 1e-15


@pytest.mark.gpu
@pytest.mark.parametrize("run", RUNS)
def test_gpu_transition_amplitudes_and_tool(gpu_available, tmp_path, run):
    import cosmo_gb300 as cg
    s = _systems(str(tmp_path))
    parent = _parent(s, run)
    d = manifest()[CASE]["runs"][run]["daughter"]
    daughter = s[d] if d else parent
    op = _op(run)
    kappa = (daughter["sys"].twom - parent["sys"].twom) // 2
    terms = TR.transition_terms(parent["sys"].sps, op, kappa)
    pb = cg.ManyBodyStates(cg.Problem(parent["xml"]))
    db = cg.ManyBodyStates(cg.Problem(daughter["xml"]))
    assert np.array_equal(pb.states(), parent["z"]) and np.array_equal(db.states(), daughter["z"])
    vp = np.array([p["vec"] for p in parent["states"]])
    vd = np.array([q["vec"] for q in daughter["states"]])
    amp = cg.onebody_amplitudes(pb, vp, db, vd, terms)
    ref = TR.onebody_amplitudes(parent["z"], vp, daughter["z"], vd, terms)
    assert np.abs(amp - ref).max() <= 1e-12
    # the tool end to end: both XMLs with the reference's <state> nodes, the .EE files beside them
    for x in {id(parent): parent, id(daughter): daughter}.values():
        name = x["sys"].name
        txt = open(x["xml"]).read().replace("</system>", "".join(manifest()[CASE][name]["states"]) + "</system>", 1)
        open(x["xml"], "w").write(txt)
        x["ee"].tofile(os.path.join(str(tmp_path), name + ".EE"))
    pin = os.path.join(str(tmp_path), "p_" + run + ".xml")
    open(pin, "w").write(open(parent["xml"]).read().replace(
        "</cosmo>", manifest()[CASE]["runs"][run]["operator"] + "\n</cosmo>", 1))
    out = os.path.join(str(tmp_path), "out_" + run + ".xml")
    fl = _flags(run)
    cg.xshlemb(pin, out, daughter_xml=daughter["xml"] if d else None, weisskopf="-w" in fl, units="-u" in fl,
               logft="-ft" in fl, phase_infinity="-p" in fl)
    txt = open(out).read()
    # the command-line drop-in writes the same file
    import subprocess
    exe = os.path.join(os.path.dirname(cg.__file__), "bin", "cg_xshlemb")
    out2 = os.path.join(str(tmp_path), "cli_" + run + ".xml")
    args = [exe, pin, "-o", out2] + list(fl) + (["-f", daughter["xml"]] if d else [])
    r = subprocess.run(args, cwd=str(tmp_path), capture_output=True, text=True, stdin=subprocess.DEVNULL)
    assert r.returncode == 0, r.stderr
    assert open(out2).read() == txt
    op_out = re.search(r"<operator [^>]*/>", txt).group(0)
    assert _attrs(op_out) == _attrs(manifest()[CASE]["runs"][run]["operator_out"])
    states = re.findall(r"<state [^>]*>.*?</state>", txt, re.S)
    trans = [[dict({k: (float(v) if k not in ("final", "name", "E", "units") else v)
                    for k, v in _attrs(t).items()}) for t in re.findall(r"<transition [^>]*/>", st)]
             for st in states]
    moms = [[{"m": float(_attrs(m)["m"])} for m in re.findall(r"<moment [^>]*/>", st)] for st in states]
    _check_records(run, trans, moms, parent["A"])
    if run == "E2":
        # XSHLJT run again on the result keeps the states' other children
        ntr = txt.count("<transition"), txt.count("<moment")
        cg.xshljt(out, os.path.join(str(tmp_path), "sd22m0s1.EE"), nstates=5)
        again = open(out).read()
        assert (again.count("<transition"), again.count("<moment")) == ntr
        for st0, st1 in zip(states, re.findall(r"<state [^>]*>.*?</state>", again, re.S)):
            assert re.findall(r"<(?:transition|moment) [^>]*/>", st0) == re.findall(r"<(?:transition|moment) [^>]*/>", st1)


def _ao_reference(name):
    return [[_attrs(o) for o in re.findall(r"<occupation [^>]*/>", st)]
            for st in manifest()[CASE]["xshlao"][name]]


def _ao_records(sysp, occ, orbitals):
    out = []
    for k in range(len(occ)):
        rec = []
        for oname, level in orbitals:
            sel = sysp.sps[:, 0] == level
            rec.append({"name": oname, "N": float(occ[k][sel & (sysp.sps[:, 6] == 1)].sum()),
                        "Z": float(occ[k][sel & (sysp.sps[:, 6] == -1)].sum())})
        out.append(rec)
    return out


def _orbitals(xml):
    import xml.etree.ElementTree as ET
    return [(o.get("name"), int(o.get("index")) - 1) for o in ET.parse(xml).getroot().find("valencespace")]


def _check_ao(name, recs):
    ref = _ao_reference(name)
    assert len(recs) == len(ref)
    for mine, theirs in zip(recs, ref):
        assert [r["name"] for r in mine] == [a["name"] for a in theirs]
        for r, a in zip(mine, theirs):
            assert _close(r["N"], float(a["N"])) and _close(r["Z"], float(a["Z"])), (name, r, a)


@pytest.mark.parametrize("name", ["sd22m0s1", "sd13m0s1", "sd22m2s1"])
def test_oracle_occupations_match_reference(tmp_path, name):
    """XSHLAO: the oracle's occupation numbers of the reference's vectors
    against the <occupation> nodes the reference XSHLAO wrote."""
    s = _systems(str(tmp_path))[name]
    occ = TR.occupations(s["z"], np.array([x["vec"] for x in s["states"]]), len(s["sys"].sps))
    _check_ao(name, _ao_records(s["sys"], occ, _orbitals(s["xml"])))


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["sd22m0s1", "sd13m0s1"])
def test_gpu_occupations_and_xshlao(gpu_available, tmp_path, name):
    import subprocess
    import cosmo_gb300 as cg
    s = _systems(str(tmp_path))[name]
    b = cg.ManyBodyStates(cg.Problem(s["xml"]))
    vecs = np.array([x["vec"] for x in s["states"]])
    occ = cg.occupations(b, vecs)
    assert np.abs(occ - TR.occupations(s["z"], vecs, len(s["sys"].sps))).max() <= 1e-12
    # the tool and its command line on the XML with the reference's <state> nodes
    txt = open(s["xml"]).read().replace("</system>", "".join(manifest()[CASE][name]["states"]) + "</system>", 1)
    open(s["xml"], "w").write(txt)
    s["ee"].tofile(os.path.join(str(tmp_path), name + ".EE"))
    out = os.path.join(str(tmp_path), "ao.xml")
    cg.xshlao(s["xml"], out)
    states = re.findall(r"<state [^>]*>.*?</state>", open(out).read(), re.S)
    recs = [[{k: (float(v) if k in ("N", "Z") else v) for k, v in _attrs(o).items()}
             for o in re.findall(r"<occupation [^>]*/>", st)] for st in states]
    _check_ao(name, recs)
    exe = os.path.join(os.path.dirname(cg.__file__), "bin", "cg_xshlao")
    r = subprocess.run([exe, s["xml"], "-o", os.path.join(str(tmp_path), "ao2.xml")], cwd=str(tmp_path),
                       capture_output=True, text=True, stdin=subprocess.DEVNULL)
    assert r.returncode == 0, r.stderr
    assert open(os.path.join(str(tmp_path), "ao2.xml")).read() == open(out).read()


def test_xlevels_matches_reference(tmp_path, capfd):
    """Xlevels (host only): the listing of two systems' states, one with an
    experimental <data Ex>, line for line the reference tool's stdout; the
    command line and the C ABI give the same; the organized XML holds every
    state with its new name and Ex."""
    import subprocess
    import cosmo_gb300 as cg
    s = _systems(str(tmp_path))
    lv = manifest()[CASE]["xlevels"]
    files = []
    for k, name in enumerate(("sd22m0s1", "sd22m2s1")):
        nodes = list(manifest()[CASE][name]["states"])
        if k == 0:
            i = lv["data_state"]
            nodes[i] = nodes[i].replace("</state>", '<data Ex="%s"/>\n</state>' % lv["data_ex"])
        txt = open(s[name]["xml"]).read().replace("</system>", "".join(nodes) + "</system>", 1)
        path = os.path.join(str(tmp_path), "lv_" + name + ".xml")
        open(path, "w").write(txt)
        files.append(path)
    exe = os.path.join(os.path.dirname(cg.__file__), "bin", "cg_xlevels")
    out = os.path.join(str(tmp_path), "levels.xml")
    r = subprocess.run([exe] + files + ["-o", out], capture_output=True, text=True, stdin=subprocess.DEVNULL)
    assert r.returncode == 0, r.stderr
    assert r.stdout.splitlines() == lv["lines"]
    cg.xlevels(files)
    assert capfd.readouterr().out.splitlines() == lv["lines"]
    organized = re.findall(r"<state [^>]*>", open(out).read())
    assert len(organized) == sum(len(manifest()[CASE][n]["states"]) for n in ("sd22m0s1", "sd22m2s1"))
    names = [_attrs(x)["name"] for x in organized]
    assert names == [ln.split()[0] for ln in lv["lines"][:len(names)]]
