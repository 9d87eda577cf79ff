"""Generate the golden fixtures in tests/golden/ from the reference itself.

Runs the reference CoSMo code compiled from the reference sources by
oracle/Makefile (oracle/_ref/ref_dump = the DEXHVJTcsb CSB path without the
Eigen fallback, oracle/_ref/XsysmbsOMP = the basis tool) on seeded synthetic
inputs (cosmo_gb300.synthetic) and on the 24Mg/usdb example, and stores what
the GPU build must reproduce:

* s.p. table, ESP and VSPX operator terms (full, small)
* the .mbs basis: full tuples for small cases, sha256 of the file otherwise
* the upper-triangle Hamiltonian rows: full for small cases; otherwise the
  sha256 of (rowptr u64 | cols u32) plus every 97th row with values
* y = H x from the reference SpMM for small cases
* eigenvalues, eigenvalue changes and residual norms of the reference Davidson
* the reference's .HH file (XHH+JJ): sha256 for small cases, bytes for one
* <J-J+> and <T-T+> of the reference's eigenvectors (oracle/_ref/ref_jt, the
  XSHLJT computation) with those vectors for small cases, and the <state>
  nodes the reference XSHLJT writes

usage (needs the reference tree; the fixtures are committed):
    python tests/golden/make_golden.py --ref /path/to/reference [--only NAME[,NAME...]]
(--ref defaults to the COSMO_REFERENCE environment variable)
"""
from __future__ import annotations

import argparse
import hashlib
import json
import os
import shutil
import re
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from cosmo_gb300.synthetic import SD_ORBITS, SyntheticSystem, make_system, write_xml  # noqa: E402

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
import truncated as TRUNC  # noqa: E402
import wide as WIDE  # noqa: E402

# name: (system, full dumps, Davidson nstates, Davidson iterations)
CASES = {
    "sd22m0s1": (SyntheticSystem("sd", 2, 2, 0, "+", 0.5, 1), True, 10, 0),
    "sd32m1s2": (SyntheticSystem("sd", 3, 2, 1, "+", 0.5, 2), True, 5, 0),
    "fp22m0s3": (SyntheticSystem("fp", 2, 2, 0, "+", 0.5, 3), False, 10, 0),
    "fp21m3s6": (SyntheticSystem("fp", 2, 1, 3, "-", 0.5, 6), True, 5, 0),
    "sd44m0s4": (SyntheticSystem("sd", 4, 4, 0, "+", 0.5, 4), False, 10, 0),
    "sd66m0s5": (SyntheticSystem("sd", 6, 6, 0, "+", 0.5, 5), False, 10, 0),
}
# basis-only cases (XsysmbsOMP)
BASIS_CASES = {
    "fp44m0s7": SyntheticSystem("fp", 4, 4, 0, "+", 0.5, 7),
    "fp55m0s8": SyntheticSystem("fp", 5, 5, 0, "+", 0.5, 8),
}
# 24Mg with usdb (EXAMPLE-24Mg-usdb.md); usdb orbit order 1=d3/2 2=d5/2 3=s1/2
USDB_ORBITS = [("0d3", 0, 2, 3), ("0d5", 0, 2, 5), ("1s1", 1, 0, 1)]


def sha(path_or_bytes) -> str:
    h = hashlib.sha256()
    if isinstance(path_or_bytes, (bytes, bytearray)):
        h.update(path_or_bytes)
    else:
        with open(path_or_bytes, "rb") as f:
            for blk in iter(lambda: f.read(1 << 24), b""):
                h.update(blk)
    return h.hexdigest()


def conn_hash(rowptr: np.ndarray, cols: np.ndarray) -> str:
    """sha256 over rowptr (u64 LE) then cols (u32 LE) of the upper rows."""
    return sha(np.ascontiguousarray(rowptr, dtype="<u8").tobytes() + np.ascontiguousarray(cols, dtype="<u4").tobytes())


def read_rows(path: str, n: int):
    raw = open(path, "rb").read()
    nnz = int(np.frombuffer(raw[:8], np.uint64)[0])
    r = np.frombuffer(raw[8:8 + 4 * nnz], np.uint32)
    c = np.frombuffer(raw[8 + 4 * nnz:8 + 8 * nnz], np.uint32)
    v = np.frombuffer(raw[8 + 8 * nnz:], np.float64)
    rp = np.zeros(n + 1, dtype=np.uint64)
    np.add.at(rp, r.astype(np.int64) + 1, 1)
    return np.cumsum(rp).astype(np.uint64), c.copy(), v.copy()


def read_ee(path: str):
    with open(path, "rb") as f:
        cnt = int(np.frombuffer(f.read(4), np.uint32)[0])
        E, D, R = [], [], []
        for _ in range(cnt):
            e, d, r = np.frombuffer(f.read(24), np.float64)
            n = int(np.frombuffer(f.read(8), np.uint64)[0])
            f.seek(8 * n, 1)
            E.append(e); D.append(d); R.append(r)
    return np.array(E), np.array(D), np.array(R)


def run_ref(ref_bin: str, xml: str, prefix: str, cwd: str, nstates: int, iters: int) -> None:
    cmd = [os.path.join(ROOT, "oracle", "_ref", ref_bin), xml]
    if ref_bin == "ref_dump":
        cmd.append(prefix)
    if nstates:
        cmd += [str(nstates), str(iters)]
    with open(os.path.join(cwd, prefix + ".log"), "w") as log:
        subprocess.run(cmd, cwd=cwd, stdin=subprocess.DEVNULL, stdout=log, stderr=subprocess.STDOUT, check=True)


def dump_case(name: str, work: str, xml: str, full: bool, nstates: int, iters: int, manifest: dict,
              keep_terms: bool = False) -> None:
    run_ref("ref_dump", xml, name, work, nstates, iters)
    sysname = name
    mbs = os.path.join(work, sysname + ".mbs")
    raw = open(mbs, "rb").read(12)
    N = int(np.frombuffer(raw[:4], np.int32)[0])
    n = int(np.frombuffer(raw[4:12], np.uint64)[0])
    sps = np.loadtxt(os.path.join(work, name + ".sps.txt"), dtype=np.int64, ndmin=2)
    esp = np.loadtxt(os.path.join(work, name + ".esp.txt"), ndmin=2)
    vspx = np.loadtxt(os.path.join(work, name + ".vspx.txt"), ndmin=2)
    rp, cols, vals = read_rows(os.path.join(work, name + ".rows.bin"), n)
    entry = dict(n=n, N=N, mbs_sha256=sha(mbs), nnz_upper=int(rp[-1]), conn_sha256=conn_hash(rp, cols))
    arrays = dict(sps=sps[:, 1:].astype(np.int32),
                  esp_keys=esp[:, :2].astype(np.int32), esp_vals=esp[:, 2],
                  vspx_keys=vspx[:, :4].astype(np.int32), vspx_vals=vspx[:, 4])
    if full:
        z = np.frombuffer(open(mbs, "rb").read()[12:], np.uint16).reshape(n, N)
        arrays.update(mbs=z, rowptr=rp, cols=cols, vals=vals)
        sp = open(os.path.join(work, name + ".spmm.bin"), "rb").read()
        nn = int(np.frombuffer(sp[:8], np.uint64)[0]); m = int(np.frombuffer(sp[8:12], np.uint32)[0])
        arrays["spmm_x"] = np.frombuffer(sp[12:12 + 8 * m * nn], np.float64).reshape(m, nn)
        arrays["spmm_y"] = np.frombuffer(sp[12 + 8 * m * nn:], np.float64).reshape(m, nn)
    else:
        sample = np.arange(0, n, 97, dtype=np.int64)
        srp = [0]
        sc, sv = [], []
        for r in sample:
            a, b = int(rp[r]), int(rp[r + 1])
            sc.append(cols[a:b]); sv.append(vals[a:b]); srp.append(srp[-1] + b - a)
        arrays.update(sample_rows=sample, sample_rowptr=np.array(srp, dtype=np.uint64),
                      sample_cols=np.concatenate(sc), sample_vals=np.concatenate(sv))
    if not keep_terms and not full:
        # the operator terms of synthetic cases are regenerated from the .int by the tests
        for k in ("esp_keys", "esp_vals", "vspx_keys", "vspx_vals"):
            arrays.pop(k)
    if nstates:
        E, D, R = read_ee(os.path.join(work, name + ".EE"))
        arrays.update(ref_eig=E, ref_de=D, ref_resid=R)
        entry.update(ref_eig=[float(x) for x in E], ref_resid=[float(x) for x in R])
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **arrays)
    manifest[name] = entry
    print(name, json.dumps({k: v for k, v in entry.items() if k not in ("ref_eig", "ref_resid")}))


def jt_case(name: str, work: str, xml: str, nstates: int, manifest: dict, keep_vecs: bool) -> None:
    """<J-J+>, <T-T+> of the reference's own eigenvectors (oracle/_ref/ref_jt, the
    computation of XSHLJT, include/xsm/XSHLJT.cxx:94-126) and the <state> nodes
    the reference XSHLJT writes into the system XML."""
    txt = open(xml).read()
    jj = re.search(r'<matrix JJ="([^"]*)"/>', txt)
    lam = jj.group(1) if jj else "0"
    node = f'<matrix name="{name}" format="pp" JJ="{lam}"/>'
    txt = txt.replace(jj.group(0), node) if jj else txt.replace("</system>", node + "</system>")
    xj = os.path.join(work, name + ".jt.xml")
    open(xj, "w").write(txt)
    ee = os.path.join(work, name + ".EE")
    with open(os.path.join(work, name + ".jt.log"), "w") as log:
        subprocess.run([os.path.join(ROOT, "oracle", "_ref", "ref_jt"), xj, ee, str(nstates), name], cwd=work,
                       stdin=subprocess.DEVNULL, stdout=log, stderr=subprocess.STDOUT, check=True)
        subprocess.run([os.path.join(ROOT, "oracle", "_ref", "XSHLJT"), xj, "-n", str(nstates)], cwd=work,
                       stdin=subprocess.DEVNULL, stdout=log, stderr=subprocess.STDOUT, check=True)
    t = np.loadtxt(os.path.join(work, name + ".jt.txt"), ndmin=2)
    out = open(xj).read()
    states = [dict(re.findall(r'(\w+)="([^"]*)"', m)) for m in re.findall(r"<state ([^>]*)>", out)]
    manifest[name]["ref_jj"] = [float(v) for v in t[:, 3]]
    manifest[name]["ref_tt"] = [float(v) for v in t[:, 4]]
    manifest[name]["ref_twoJ"] = [int(v) for v in t[:, 5]]
    manifest[name]["ref_xshljt_states"] = states
    if keep_vecs:
        n = manifest[name]["n"]
        v = np.fromfile(os.path.join(work, name + ".vecs.bin"), np.float64).reshape(-1, n)
        arrays = dict(np.load(os.path.join(HERE, name + ".npz")))
        arrays["ref_vecs"] = v
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **arrays)
    print(name, "jt", manifest[name]["ref_twoJ"])


# spectroscopic factors (XSHLSF): parent sd 2n+2p, daughter sd 2n+1p, same
# seed (same TBMEs); the systems carry Tz so that the reference's XSHLJT
# records it in the <wavefunction> nodes XSHLSF reads
SF_PAIR = (("sd22m0s1", SyntheticSystem("sd", 2, 2, 0, "+", 0.5, 1)),
           ("sd21m1s1", SyntheticSystem("sd", 2, 1, 1, "+", 0.5, 1)))
SF_STATES = 5


def spin_text(t2: int) -> str:
    return str(t2 // 2) if t2 % 2 == 0 else f"{t2}/2"


def sf_xml(work: str, name: str, sysd) -> str:
    """The synthetic system XML with a Tz attribute on the system node."""
    sysd.name = name
    _, xml = make_system(work, sysd)
    txt = open(xml).read().replace("<system ", f'<system Tz="{spin_text(sysd.nv - sysd.zv)}" ', 1)
    open(xml, "w").write(txt)
    return xml


def sf_case(work: str, manifest: dict) -> None:
    """The reference's XSHLSF tables (per l, and per s.p. state with -of) for
    the SF_PAIR systems, after the reference's Davidson (ref_dump) and XSHLJT
    recorded their states; stores the <state> nodes, the .EE files and the
    tables."""
    arrays = {}
    entry = {}
    xjs = []
    for name, sysd in SF_PAIR:
        xml = sf_xml(work, name, sysd)
        run_ref("ref_dump", xml, name, work, SF_STATES, 0)
        txt = open(xml).read()
        jj = re.search(r'<matrix JJ="([^"]*)"/>', txt)
        txt = txt.replace(jj.group(0), f'<matrix name="{name}" format="pp" JJ="{jj.group(1)}"/>')
        xj = os.path.join(work, name + ".sf.xml")
        open(xj, "w").write(txt)
        with open(os.path.join(work, name + ".sf.log"), "w") as log:
            subprocess.run([os.path.join(ROOT, "oracle", "_ref", "XSHLJT"), xj, "-n", str(SF_STATES)], cwd=work,
                           stdin=subprocess.DEVNULL, stdout=log, stderr=subprocess.STDOUT, check=True)
        out = open(xj).read()
        entry[name] = {"states": re.findall(r"<state [^>]*>\s*<wavefunction[^>]*/>\s*</state>", out)}
        arrays[name + "_EE"] = np.fromfile(os.path.join(work, name + ".EE"), np.uint8)
        xjs.append(xj)
    for key, flags in (("table", []), ("table_full", ["-of"])):
        outp = os.path.join(work, key + ".txt")
        subprocess.run([os.path.join(ROOT, "oracle", "_ref", "XSHLSF"), xjs[0], "-f", xjs[1], "-o", outp] + flags,
                       cwd=work, stdin=subprocess.DEVNULL, stdout=subprocess.DEVNULL, stderr=subprocess.STDOUT,
                       check=True)
        entry[key] = [ln for ln in open(outp).read().splitlines() if ln and not ln.startswith("#")]
    manifest["sf_sd22_sd21"] = entry
    np.savez_compressed(os.path.join(HERE, "sf_sd22_sd21.npz"), **arrays)
    print("sf", len(entry["table"]), "lines per l,", len(entry["table_full"]), "per s.p. state")


# electromagnetic and beta transitions (XSHLEMB): parent sd 2n+2p, and for the
# beta operators a daughter sd 1n+3p; both with the mass number A (Weisskopf
# units) and Tz, their states from the reference's Davidson and XSHLJT, their
# .mbs from the reference's XsysmbsOMP
EM_SYSTEMS = (("sd22m0s1", SyntheticSystem("sd", 2, 2, 0, "+", 0.5, 1)),
              ("sd13m0s1", SyntheticSystem("sd", 1, 3, 0, "+", 0.5, 1)),
              ("sd22m2s1", SyntheticSystem("sd", 2, 2, 2, "+", 0.5, 1)),
              # fp: oscillator radial integrals of 0f and 1p orbits
              ("fp11m0s9", SyntheticSystem("fp", 1, 1, 0, "+", 0.5, 9)),
              ("fp20m0s9", SyntheticSystem("fp", 2, 0, 0, "+", 0.5, 9)))
EM_CORE = {"sd": 16, "fp": 40}  # mass number of the core (Weisskopf and standard units)
EM_STATES = 5
# run name: (operator node, daughter system or None for the parent itself, flags[, parent system])
EM_RUNS = {
    "E2": ('<operator name="E2" J="2" en="0.5" ep="1.5"/>', None, ["-w", "-u"]),
    "E2p": ('<operator name="E2" J="2" en="0.5" ep="1.5"/>', None, ["-p"]),
    "M1": ('<operator name="M1" J="1"/>', None, ["-w", "-u"]),
    "GT-": ('<operator name="GT-" J="1"/>', "sd13m0s1", ["-ft"]),
    "F": ('<operator name="F" J="0"/>', "sd13m0s1", []),
    # projection kappa = 1 (daughter 2M = 2), explicit moments
    "M1k": ('<operator name="M1" J="1" mu_n="-1.5" mu_p="2.5" gl_n="0.1" gl_p="0.9"/>', "sd22m2s1", ["-u"]),
    "E2k": ('<operator name="E2" J="2" en="0.6" ep="1.4"/>', "sd22m2s1", ["-w"]),
    # beta plus from the sd 1n+3p states to the sd 2n+2p ones
    "GT+": ('<operator name="GT+" J="1"/>', "sd22m0s1", ["-ft"], "sd13m0s1"),
    # fp shell: E2, M1, E4 (r^4 radial integrals) within fp 1n+1p, GT- from fp 2n+0p
    "E2fp": ('<operator name="E2" J="2" en="0.5" ep="1.5"/>', None, ["-w", "-u"], "fp11m0s9"),
    "M1fp": ('<operator name="M1" J="1"/>', None, ["-w"], "fp11m0s9"),
    "E4fp": ('<operator name="E4" J="4" en="0.5" ep="1.5"/>', None, ["-u"], "fp11m0s9"),
    "GT-fp": ('<operator name="GT-" J="1"/>', "fp11m0s9", ["-ft"], "fp20m0s9"),
}


def em_xml(work: str, name: str, sysd) -> str:
    """A system with its reference basis (.mbs, XsysmbsOMP), eigenvectors
    (.EE, ref_dump) and <state> nodes (XSHLJT); returns the XML path."""
    xml = sf_xml(work, name, sysd)
    txt = open(xml).read().replace("<system ", f'<system A="{EM_CORE[sysd.space] + sysd.nv + sysd.zv}" ', 1)
    open(xml, "w").write(txt)
    run_ref("ref_dump", xml, name, work, EM_STATES, 0)
    txt = open(xml).read()
    jj = re.search(r'<matrix JJ="([^"]*)"/>', txt)
    txt = txt.replace(jj.group(0), f'<matrix name="{name}" format="pp" JJ="{jj.group(1)}"/>')
    open(xml, "w").write(txt)
    run_ref("XsysmbsOMP", xml, name + ".x", work, 0, 0)
    with open(os.path.join(work, name + ".jt.log"), "w") as log:
        subprocess.run([os.path.join(ROOT, "oracle", "_ref", "XSHLJT"), xml, "-n", str(EM_STATES)], cwd=work,
                       stdin=subprocess.DEVNULL, stdout=log, stderr=subprocess.STDOUT, check=True)
    return xml


def em_case(work: str, manifest: dict) -> None:
    """The <transition> and <moment> nodes the reference XSHLEMB adds to the
    parent's states for every EM_RUNS operator, with the systems' <state>
    nodes and .EE files they were computed from."""
    arrays, entry, xmls = {}, {"runs": {}}, {}
    for name, sysd in EM_SYSTEMS:
        xmls[name] = em_xml(work, name, sysd)
        arrays[name + "_EE"] = np.fromfile(os.path.join(work, name + ".EE"), np.uint8)
        entry[name] = {"states": re.findall(r"<state [^>]*>\s*<wavefunction[^>]*/>\s*</state>",
                                            open(xmls[name]).read())}
    for run, spec in EM_RUNS.items():
        op, daughter, flags = spec[:3]
        parent = spec[3] if len(spec) > 3 else EM_SYSTEMS[0][0]
        xin = os.path.join(work, f"em_{run}.xml")
        open(xin, "w").write(open(xmls[parent]).read().replace("</cosmo>", op + "\n</cosmo>", 1))
        xout = os.path.join(work, f"em_{run}.out.xml")
        cmd = [os.path.join(ROOT, "oracle", "_ref", "XSHLEMB"), xin, "-o", xout] + flags
        if daughter:
            cmd += ["-f", xmls[daughter]]
        with open(os.path.join(work, f"em_{run}.log"), "w") as log:
            subprocess.run(cmd, cwd=work, stdin=subprocess.DEVNULL, stdout=log, stderr=subprocess.STDOUT, check=True)
        out = open(xout).read()
        entry["runs"][run] = {
            "operator": op, "daughter": daughter, "flags": flags, "parent": parent,
            "operator_out": re.search(r"<operator [^>]*/>", out).group(0),
            "states": re.findall(r"<state [^>]*>.*?</state>", out, re.S)}
    # occupation numbers (XSHLAO) of the same systems' states
    entry["xshlao"] = {}
    for name, _ in EM_SYSTEMS:
        xout = os.path.join(work, f"ao_{name}.out.xml")
        with open(os.path.join(work, f"ao_{name}.log"), "w") as log:
            subprocess.run([os.path.join(ROOT, "oracle", "_ref", "XSHLAO"), xmls[name], "-o", xout], cwd=work,
                           stdin=subprocess.DEVNULL, stdout=log, stderr=subprocess.STDOUT, check=True)
        entry["xshlao"][name] = re.findall(r"<state [^>]*>.*?</state>", open(xout).read(), re.S)
    # level listing (Xlevels) of two systems' states, one state with an
    # experimental <data Ex> child
    lv = []
    for k, name in enumerate(("sd22m0s1", "sd22m2s1")):
        txt = open(xmls[name]).read()
        if k == 0:
            st = re.findall(r"<state [^>]*>.*?</state>", txt, re.S)[1]
            txt = txt.replace(st, st.replace("</state>", '<data Ex="1.5"/>\n</state>'), 1)
        path = os.path.join(work, f"lv_{name}.xml")
        open(path, "w").write(txt)
        lv.append(path)
    r = subprocess.run([os.path.join(ROOT, "oracle", "_ref", "Xlevels")] + lv, cwd=work, stdin=subprocess.DEVNULL,
                       capture_output=True, text=True, check=True)
    entry["xlevels"] = {"data_state": 1, "data_ex": "1.5", "lines": r.stdout.splitlines()}
    manifest["em_sd22"] = entry
    np.savez_compressed(os.path.join(HERE, "em_sd22.npz"), **arrays)
    print("em", {r: sum(s.count("<transition") for s in v["states"]) for r, v in entry["runs"].items()})


def wide_em_case(work: str, manifest: dict) -> None:
    """E2 transitions among the lowest states of the spsdpf 0 hw window, as
    step 5 of the reference's 33Al example (XSHLEMB -w -u, en 0.5, ep 1.5):
    the reference's basis, Davidson vectors (.EE), XSHLJT <state> nodes and
    XSHLEMB output."""
    name = "spsdpf_0hw"
    xml = WIDE.write_case(work, name)
    txt = open(xml).read().replace("<system ", '<system A="33" ', 1)
    open(xml, "w").write(txt)
    run_ref("XsysmbsOMP", xml, name + ".x", work, 0, 0)
    run_ref("ref_dump", xml, name, work, EM_STATES, 0)
    txt = open(xml).read()
    jj = re.search(r'<matrix JJ="([^"]*)"/>', txt)
    open(xml, "w").write(txt.replace(jj.group(0), f'<matrix name="{name}" format="pp" JJ="{jj.group(1)}"/>'))
    with open(os.path.join(work, name + ".jt.log"), "w") as log:
        subprocess.run([os.path.join(ROOT, "oracle", "_ref", "XSHLJT"), xml, "-n", str(EM_STATES)], cwd=work,
                       stdin=subprocess.DEVNULL, stdout=log, stderr=subprocess.STDOUT, check=True)
    op, flags = '<operator name="E2" J="2" en="0.5" ep="1.5"/>', ["-w", "-u"]
    xin = os.path.join(work, "em_wide.xml")
    open(xin, "w").write(open(xml).read().replace("</cosmo>", op + "\n</cosmo>", 1))
    xout = os.path.join(work, "em_wide.out.xml")
    with open(os.path.join(work, "em_wide.log"), "w") as log:
        subprocess.run([os.path.join(ROOT, "oracle", "_ref", "XSHLEMB"), xin, "-o", xout] + flags, cwd=work,
                       stdin=subprocess.DEVNULL, stdout=log, stderr=subprocess.STDOUT, check=True)
    out = open(xout).read()
    manifest["em_wide"] = {
        "states": re.findall(r"<state [^>]*>\s*<wavefunction[^>]*/>\s*</state>", open(xml).read()),
        "operator": op, "flags": flags, "operator_out": re.search(r"<operator [^>]*/>", out).group(0),
        "out_states": re.findall(r"<state [^>]*>.*?</state>", out, re.S)}
    np.savez_compressed(os.path.join(HERE, "em_wide.npz"), EE=np.fromfile(os.path.join(work, name + ".EE"), np.uint8))
    print("em_wide", sum(st.count("<transition") for st in manifest["em_wide"]["out_states"]), "transitions")


def hh_case(name: str, work: str, xml: str, manifest: dict, keep_bytes: bool) -> None:
    """The reference's .HH file (XHH+JJ, PPMatrix::Write): sha256, and the bytes
    for one small case so the .HH reader can be pinned on a GPU."""
    with open(os.path.join(work, name + ".hh.log"), "w") as log:
        subprocess.run([os.path.join(ROOT, "oracle", "_ref", "XHH+JJ"), xml], cwd=work, stdin=subprocess.DEVNULL,
                       stdout=log, stderr=subprocess.STDOUT, check=True)
    hh = os.path.join(work, name + ".HH")
    manifest[name]["ref_hh_sha256"] = sha(hh)
    manifest[name]["ref_hh_bytes"] = os.path.getsize(hh)
    if keep_bytes:
        arrays = dict(np.load(os.path.join(HERE, name + ".npz")))
        arrays["ref_hh"] = np.fromfile(hh, np.uint8)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **arrays)
    print(name, "hh", manifest[name]["ref_hh_bytes"])


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("COSMO_REFERENCE"))
    ap.add_argument("--only", default=None)
    a = ap.parse_args()
    if not a.ref:
        ap.error("give the reference checkout with --ref or COSMO_REFERENCE")
    only = set(a.only.split(",")) if a.only else None

    def skip(name: str) -> bool:
        return only is not None and name not in only
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref", f"REF={a.ref}"], check=True)
    mpath = os.path.join(HERE, "manifest.json")
    manifest = json.load(open(mpath)) if os.path.exists(mpath) else {}
    work = tempfile.mkdtemp(prefix="cg_golden_")
    try:
        if not skip("sf_sd22_sd21"):
            sf_case(work, manifest)
        if not skip("em_sd22"):
            em_case(work, manifest)
        for name, (sysd, full, nst, it) in CASES.items():
            if skip(name):
                continue
            sysd.name = name
            _, xml = make_system(work, sysd)
            dump_case(name, work, xml, full, nst, it, manifest)
            manifest[name]["system"] = dict(space=sysd.space, nv=sysd.nv, zv=sysd.zv, twom=sysd.twom,
                                            parity=sysd.parity, jj=sysd.jj, seed=sysd.seed)
            if nst and full:
                jt_case(name, work, xml, nst, manifest, keep_vecs=full)
            if full:
                hh_case(name, work, xml, manifest, keep_bytes=(name == "sd22m0s1"))
        for name, sysd in BASIS_CASES.items():
            if skip(name):
                continue
            sysd.name = name
            _, xml = make_system(work, sysd)
            run_ref("XsysmbsOMP", xml, name, work, 0, 0)
            mbs = os.path.join(work, name + ".mbs")
            raw = open(mbs, "rb").read(12)
            manifest[name] = dict(n=int(np.frombuffer(raw[4:12], np.uint64)[0]),
                                  N=int(np.frombuffer(raw[:4], np.int32)[0]), mbs_sha256=sha(mbs),
                                  system=dict(space=sysd.space, nv=sysd.nv, zv=sysd.zv, twom=sysd.twom,
                                              parity=sysd.parity, jj=sysd.jj, seed=sysd.seed))
            print(name, manifest[name])
        # truncated bases (hw truncation, orbital rejections): the reference's .mbs
        for name in TRUNC.CASES:
            if skip(name):
                continue
            xml = TRUNC.write_case(work, name)
            run_ref("XsysmbsOMP", xml, name, work, 0, 0)
            mbs = os.path.join(work, name + ".mbs")
            raw = open(mbs, "rb").read()
            N = int(np.frombuffer(raw[:4], np.int32)[0])
            n = int(np.frombuffer(raw[4:12], np.uint64)[0])
            hw, rej = TRUNC.truncation(name)
            manifest[name] = dict(n=n, N=N, mbs_sha256=sha(mbs), truncation=dict(hw=hw, rejections=rej))
            np.savez_compressed(os.path.join(HERE, name + ".npz"),
                                mbs=np.frombuffer(raw[12:], np.uint16).reshape(n, N))
            print(name, manifest[name])
        # wide valence space (spsdpf, 40 m-states per species): the reference's
        # basis (XsysmbsOMP), its rows and Davidson on that basis (ref_dump reads
        # the .mbs), and <J-J+>, <T-T+> of its vectors
        for name, c in WIDE.CASES.items():
            if skip(name):
                continue
            xml = WIDE.write_case(work, name)
            run_ref("XsysmbsOMP", xml, name + ".x", work, 0, 0)
            dump_case(name, work, xml, c["full"], c["nstates"], 0, manifest)
            manifest[name]["truncation"] = dict(hw=list(c["hw"]) if c["hw"] else None, rejections=[])
            manifest[name]["system"] = dict(space="spsdpf", nv=c["nv"], zv=c["zv"], twom=c["twom"],
                                            parity=c["parity"], jj=0.0, seed=WIDE.SEED)
            if c["full"]:
                jt_case(name, work, xml, c["nstates"], manifest, keep_vecs=True)
            if name != "spsdpf_0hw":  # same interaction: its terms are pinned on the 0 hw case
                path = os.path.join(HERE, name + ".npz")
                arrays = {k: v for k, v in np.load(path).items() if not k.startswith(("esp_", "vspx_"))}
                np.savez_compressed(path, **arrays)
        if not skip("em_wide"):
            wide_em_case(work, manifest)
        if not skip("mg24usdb"):
            sysd = SyntheticSystem("sd", 4, 4, 0, "+", 0.0, 0, name="mg24usdb")
            xml = os.path.join(work, "mg24usdb.xml")
            write_xml(xml, sysd, os.path.join(a.ref, "interactions", "sd", "usdb.int"), USDB_ORBITS, hname="usdb")
            # no JJ shift in the example (EXAMPLE-24Mg-usdb.md:10)
            txt = open(xml).read().replace('<matrix JJ="0.0"/>', "")
            open(xml, "w").write(txt)
            dump_case("mg24usdb", work, xml, False, 10, 0, manifest, keep_terms=True)
            manifest["mg24usdb"]["system"] = dict(space="sd-usdb", nv=4, zv=4, twom=0, parity="+", jj=None)
            jt_case("mg24usdb", work, xml, 10, manifest, keep_vecs=False)
            # known answers printed in EXAMPLE-24Mg-usdb.md:29-38 (E, 4 decimals)
            manifest["mg24usdb"]["example_E"] = [-87.1044, -85.6021, -82.9883, -82.732, -82.0294, -81.2219,
                                                 -79.7662, -79.6227, -79.3076, -79.2863]
    finally:
        shutil.rmtree(work, ignore_errors=True)
    with open(mpath, "w") as f:
        json.dump(manifest, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
