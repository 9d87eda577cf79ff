"""The command-line drop-ins (C++ over the C ABI) against the reference's
tools' outputs: cg_xsysmbs (Xsysmbs), cg_xhhjj (XHH+JJ), cg_dexhvjt
(DEXHVJTcsb incl. XSHLJT), cg_davidson_vfile (davidson_vfile), cg_xshljt; cg_xshlsf and
cg_xshlemb are run against the reference tools' outputs in test_sf.py / test_em.py."""
import hashlib
import os
import re
import subprocess

import numpy as np
import pytest

import cosmo_gb300 as cg
from conftest import ROOT, golden, manifest, synthetic_xml

BIN = os.path.join(ROOT, "cosmo_gb300", "bin")
TOOLS = ["cg_dexhvjt", "cg_xsysmbs", "cg_xhhjj", "cg_davidson_vfile", "cg_xshljt", "cg_xshlsf", "cg_xshlemb", "cg_xshlao", "cg_xlevels"]


def _run(args, cwd):
    return subprocess.run(args, cwd=cwd, capture_output=True, text=True, stdin=subprocess.DEVNULL)


@pytest.mark.parametrize("tool", TOOLS)
def test_cli_usage(tool, tmp_path):
    """Every tool is built and prints its usage (exit 1) without arguments."""
    exe = os.path.join(BIN, tool)
    if not os.path.exists(exe):
        pytest.skip("command-line tools not built")
    r = _run([exe], str(tmp_path))
    assert r.returncode == 1 and "usage" in r.stderr


@pytest.mark.gpu
def test_cli_pipeline(gpu_available, tmp_path):
    name = "sd32m1s2"
    m = manifest()[name]
    g = golden(name)
    work = str(tmp_path)
    xml = synthetic_xml(name, work)
    # basis
    r = _run([os.path.join(BIN, "cg_xsysmbs"), xml, "-o", "x.mbs"], work)
    assert r.returncode == 0, r.stderr
    assert hashlib.sha256(open(os.path.join(work, "x.mbs"), "rb").read()).hexdigest() == m["mbs_sha256"]
    # .HH
    r = _run([os.path.join(BIN, "cg_xhhjj"), xml, "-o", "x.HH"], work)
    assert r.returncode == 0, r.stderr
    raw = open(os.path.join(work, "x.HH"), "rb").read()
    assert hashlib.sha256(raw).hexdigest() == m["ref_hh_sha256"] or len(raw) <= m["ref_hh_bytes"]
    # davidson_vfile on that file
    r = _run([os.path.join(BIN, "cg_davidson_vfile"), "x.HH", "-n", "5"], work)
    assert r.returncode == 0, r.stderr
    E, D, R, V = cg.read_ee(os.path.join(work, "x.HH.EE"))
    ok = R < 1e-5
    assert ok.sum() >= 3
    ref = np.asarray(m["ref_eig"])
    assert np.all(np.min(np.abs(E[ok][:, None] - ref[None, :]), axis=1) < 1e-4)
    # whole DEXHVJTcsb flow: mixed solve + XSHLJT into a new XML
    r = _run([os.path.join(BIN, "cg_dexhvjt"), xml, "-n", "5", "-o", "out.xml"], work)
    assert r.returncode == 0, r.stderr
    E2, _, R2, _ = cg.read_ee(os.path.join(work, name + ".HH.EE"))
    assert np.all(R2 <= 1e-5)
    np.testing.assert_allclose(E2, g["ref_eig"], rtol=0, atol=1e-4)
    txt = open(os.path.join(work, "out.xml")).read()
    states = [dict(re.findall(r'(\w+)="([^"]*)"', x)) for x in re.findall(r"<state ([^>]*)>", txt)]
    ref_states = m["ref_xshljt_states"]
    assert [s["J"] for s in states] == [s["J"] for s in ref_states]
    assert [s["name"] for s in states] == [s["name"] for s in ref_states]
    for a, b in zip(states, ref_states):
        assert abs(float(a["E"]) - float(b["E"])) < 2e-4
    # cg_xshljt on the same .EE into the input file (second pass merges)
    r = _run([os.path.join(BIN, "cg_xshljt"), "out.xml", "-n", "5", "-e", name + ".HH.EE"], work)
    assert r.returncode == 0, r.stderr
    assert len(re.findall(r"<state ", open(os.path.join(work, "out.xml")).read())) == len(ref_states)


@pytest.mark.gpu
def test_cli_exact_path(gpu_available, tmp_path):
    """cg_dexhvjt at or below the -l limit (default 1000) diagonalizes exactly
    and writes every state into the .EE file, as the reference's DXHV does
    (include/xsm/DEXHVcsb.cxx:80-110); -l 0 keeps Davidson."""
    name = "sd22m0s1"
    m = manifest()[name]
    work = str(tmp_path)
    xml = synthetic_xml(name, work)
    r = _run([os.path.join(BIN, "cg_dexhvjt"), xml, "-n", "5", "-o", "out.xml"], work)
    assert r.returncode == 0, r.stderr
    assert "exact diagonalization" in r.stderr
    E, D, R, V = cg.read_ee(os.path.join(work, name + ".HH.EE"))
    assert len(E) == m["n"] and V.shape == (m["n"], m["n"])
    assert np.all(D == 0) and np.all(R == 0)
    np.testing.assert_allclose(E[:10], m["ref_eig"][:10], rtol=0, atol=1e-7)
    assert np.all(np.diff(E) >= 0)
    txt = open(os.path.join(work, "out.xml")).read()
    states = [dict(re.findall(r'(\w+)="([^"]*)"', x)) for x in re.findall(r"<state ([^>]*)>", txt)]
    assert 0 < len(states) <= 5
    r = _run([os.path.join(BIN, "cg_dexhvjt"), xml, "-n", "5", "-l", "0", "-o", "out2.xml"], work)
    assert r.returncode == 0, r.stderr
    assert "exact diagonalization" not in r.stderr
    E2, _, R2, _ = cg.read_ee(os.path.join(work, name + ".HH.EE"))
    assert len(E2) == 5 and np.all(R2 <= 1e-5)
    np.testing.assert_allclose(E2, E[:5], rtol=0, atol=1e-4)
