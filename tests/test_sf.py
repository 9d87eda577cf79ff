"""Spectroscopic factors (the reference's XSHLSF, xmlshell/XSHLSF.cpp): the
oracle's one-particle removal amplitudes and the GPU ones against the tables
the reference XSHLSF wrote for a parent sd 2n+2p and a daughter sd 2n+1p
system (tests/golden/make_golden.py, sf_case), using the reference's own
eigenvectors (.EE files) and <state> nodes.  The tables print 6 significant
digits: amplitudes and factors are compared within 1e-6 + 1e-5 relative; the
GPU amplitudes against the oracle's within 1e-12."""
import os
import re
import tempfile

import numpy as np
import pytest

from conftest import GOLDEN, manifest
from oracle import interaction as OI
from oracle import oracle as O

PAIR = "sf_sd22_sd21"
NAMES = ("sd22m0s1", "sd21m1s1")


def _spin2(t):
    return OI.spin2(t)


def _states(name):
    out = []
    for node in manifest()[PAIR][name]["states"]:
        st = dict(re.findall(r'(\w+)="([^"]*)"', node.split("<wavefunction")[0]))
        wf = dict(re.findall(r'(\w+)="([^"]*)"', node.split("<wavefunction")[1]))
        out.append(dict(name=st["name"], ex=st["Ex"], twoJ=_spin2(st["J"]), parity=1 if st["P"] == "-" else 0,
                        twoJz=_spin2(wf["Jz"]), twoTz=_spin2(wf["Tz"]), id=int(wf["id"])))
    return out


def _ee_vectors(raw):
    b = raw.tobytes()
    cnt = int(np.frombuffer(b[:4], np.uint32)[0])
    off, vecs = 4, []
    for _ in range(cnt):
        n = int(np.frombuffer(b[off + 24:off + 32], np.uint64)[0])
        vecs.append(np.frombuffer(b[off + 32:off + 32 + 8 * n], np.float64).copy())
        off += 32 + 8 * n
    return np.array(vecs)


def _setup(tmp):
    """Both systems' XML (with Tz), oracle bases and the state vectors in state order."""
    import sys
    sys.path.insert(0, GOLDEN)
    import make_golden as MG
    g = np.load(os.path.join(GOLDEN, PAIR + ".npz"))
    out = {}
    for name, sysd in MG.SF_PAIR:
        xml = MG.sf_xml(tmp, name, sysd)
        sysp = OI.System(xml)
        z = O.basis(sysp.sps, sysp.nv + sysp.zv, sysp.twom, sysp.nv - sysp.zv, sysp.parity)
        st = _states(name)
        vecs = _ee_vectors(g[name + "_EE"])
        out[name] = dict(xml=xml, sys=sysp, z=z, states=st, vecs=np.array([vecs[s["id"]] for s in st]),
                         ee=g[name + "_EE"])
    return out


def _table(sysp, P, D, amp):
    """Rows (parent, daughter, l, 2j, A, SF) as XSHLSF -of forms them, and the
    per-l sums."""
    full, perl = [], {}
    for ip, p in enumerate(P):
        for iq, q in enumerate(D):
            jz, tz, par = p["twoJz"] - q["twoJz"], p["twoTz"] - q["twoTz"], p["parity"] ^ q["parity"]
            for s, sp in enumerate(sysp.sps):
                if sp[4] != jz or sp[6] != tz or (sp[7] ^ par):
                    continue
                cg = OI.clebsch_gordan(q["twoJ"], q["twoJz"], int(sp[3]), jz, p["twoJ"], p["twoJz"])
                if abs(cg) < 1e-10:
                    continue
                a = amp[iq, ip, s] / cg
                full.append((p["name"], q["name"], int(sp[2]), int(sp[3]), a, a * a))
                key = (p["name"], q["name"], int(sp[2]))
                perl[key] = perl.get(key, 0.0) + a * a
    return full, perl


def _ref_tables():
    m = manifest()[PAIR]
    full = []
    for ln in m["table_full"]:
        f = ln.split("\t")
        full.append((f[0], f[2], int(f[4]), _spin2(f[5]), float(f[6]), float(f[7])))
    perl = {}
    for ln in m["table"]:
        f = ln.split("\t")
        perl[(f[0], f[2], int(f[4]))] = float(f[5])
    return full, perl


def _close(x, y):
    return abs(x - y) <= 1e-6 + 1e-5 * abs(y)


def _check_against_reference(full, perl):
    rfull, rperl = _ref_tables()
    assert len(full) == len(rfull)
    for mine, ref in zip(full, rfull):
        assert mine[:4] == ref[:4], (mine, ref)
        assert _close(mine[4], ref[4]) and _close(mine[5], ref[5]), (mine, ref)
    for key in set(perl) | set(rperl):
        assert _close(perl.get(key, 0.0), rperl.get(key, 0.0)), key


def test_oracle_sf_matches_reference(tmp_path):
    s = _setup(str(tmp_path))
    P, D = s[NAMES[0]], s[NAMES[1]]
    amp = O.annihilation_amplitudes(P["z"], P["vecs"], D["z"], D["vecs"], len(P["sys"].sps))
    _check_against_reference(*_table(P["sys"], P["states"], D["states"], amp))


@pytest.mark.gpu
def test_gpu_sf_amplitudes_and_tool(gpu_available, tmp_path):
    import cosmo_gb300 as cg
    s = _setup(str(tmp_path))
    P, D = s[NAMES[0]], s[NAMES[1]]
    pb = cg.ManyBodyStates(cg.Problem(P["xml"]))
    db = cg.ManyBodyStates(cg.Problem(D["xml"]))
    assert np.array_equal(pb.states(), P["z"]) and np.array_equal(db.states(), D["z"])
    amp = cg.sf_amplitudes(pb, P["vecs"], db, D["vecs"])
    ref = O.annihilation_amplitudes(P["z"], P["vecs"], D["z"], D["vecs"], len(P["sys"].sps))
    assert np.abs(amp - ref).max() <= 1e-12
    _check_against_reference(*_table(P["sys"], P["states"], D["states"], amp))
    # the tool end to end: XML with the reference's <state> nodes, the .EE files beside them
    for name in NAMES:
        x = s[name]
        txt = open(x["xml"]).read().replace("</system>", "".join(manifest()[PAIR][name]["states"]) + "</system>", 1)
        open(x["xml"], "w").write(txt)
        x["ee"].tofile(os.path.join(str(tmp_path), name + ".EE"))
    for full, key in ((False, "table"), (True, "table_full")):
        out = os.path.join(str(tmp_path), key + ".txt")
        cg.xshlsf(P["xml"], out, daughter_xml=D["xml"], full=full)
        lines = [ln for ln in open(out).read().splitlines() if ln and not ln.startswith("#")]
        ref = manifest()[PAIR][key]
        mine = {tuple(ln.split("\t")[:5 if not full else 6]): float(ln.split("\t")[-1]) for ln in lines}
        theirs = {tuple(ln.split("\t")[:5 if not full else 6]): float(ln.split("\t")[-1]) for ln in ref}
        for k in set(mine) | set(theirs):
            assert _close(mine.get(k, 0.0), theirs.get(k, 0.0)), (k, mine.get(k), theirs.get(k))
