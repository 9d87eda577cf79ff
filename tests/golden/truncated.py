"""Truncated-basis cases: the oscillator-quanta truncation (the system's
`hwmax` attribute or its <hwrejection HWMIN HWMAX> child) and the orbital-
occupation rejections (<rejection NMIN NMAX> with <orbital index type>
children) of the reference's basis tool, xmlshell/xmbs/XsysmbsOMP.cpp:214-300.
The p+sd valence spaces below mix two oscillator shells (0p: 2n+l = 1, sd: 2),
so the truncations select something.  Shared by the fixture script
(make_golden.py, which runs the reference on these XML files) and the tests
(which rebuild the same XML and compare the oracle's basis with the fixtures).
"""
from __future__ import annotations

import os

from cosmo_gb300.synthetic import SyntheticSystem, write_int, write_xml

# (name, n, l, 2j) in XML index order
PSD_ORBITS = [("0p3", 0, 1, 3), ("0p1", 0, 1, 1), ("0d5", 0, 2, 5), ("1s1", 1, 0, 1), ("0d3", 0, 2, 3)]
# sd listed before p: the reference's core quanta are the quanta of the first
# Nv (Zv) s.p. states in list order (include/sm/SingleParticleStates.cxx:
# 155-168 sorts an empty range), so here the core is counted in the sd shell
SDP_ORBITS = [("0d5", 0, 2, 5), ("1s1", 1, 0, 1), ("0d3", 0, 2, 3), ("0p3", 0, 1, 3), ("0p1", 0, 1, 1)]

CASES = {
    # 0 and 2 hw excitations above the p-shell core
    "psd22m0_hw2": dict(orbits=PSD_ORBITS, nv=2, zv=2, twom=0, parity="+", hwmax=2),
    # only 2 hw (HWMIN 1 drops 0 hw, parity drops 1 and 3 hw)
    "psd32m1_hwr13": dict(orbits=PSD_ORBITS, nv=3, zv=2, twom=1, parity="-", hwrej=(1, 3)),
    # hw truncation and at most one particle (either species) in 0d3/2
    "psd22m0_hw2_rej": dict(orbits=PSD_ORBITS, nv=2, zv=2, twom=0, parity="+", hwmax=2,
                            rej=[(0, 1, [5])]),
    # occupation rejection alone: 1 or 2 particles in 0p1/2 + 1s1/2
    "psd21m1_rej": dict(orbits=PSD_ORBITS, nv=2, zv=1, twom=1, parity="-", rej=[(1, 2, [2, 4])]),
    # the list-order core quanta (see SDP_ORBITS)
    "sdp22m0_hw2": dict(orbits=SDP_ORBITS, nv=2, zv=2, twom=0, parity="+", hwmax=2),
}


def truncation(name: str) -> tuple[tuple[int, int] | None, list[tuple[int, int, list[int]]]]:
    """(hwmin, hwmax) or None, and the rejections as (nmin, nmax, 0-based
    orbital levels, both species) of a case."""
    c = CASES[name]
    hw = None
    if "hwmax" in c:
        hw = (0, c["hwmax"])
    if "hwrej" in c:
        hw = c["hwrej"]
    rej = [(lo, hi, [i - 1 for i in idx]) for lo, hi, idx in c.get("rej", [])]
    return hw, rej


# larger cases for the on-the-fly product (no fixtures: checked against the
# stored matrix, which the cases above pin to the reference): lists of up to
# 260 rows over several 32-row slices, and lists far shorter than their class
LARGE = {
    "psd44m0_hw4": dict(orbits=PSD_ORBITS, nv=4, zv=4, twom=0, parity="+", hwmax=4),
    "psd44m0_hw4_rej": dict(orbits=PSD_ORBITS, nv=4, zv=4, twom=0, parity="+", hwmax=4,
                            rej=[(0, 2, [5])]),
    "psd66m0_hw2": dict(orbits=PSD_ORBITS, nv=6, zv=6, twom=0, parity="+", hwmax=2),
}


def write_case(workdir: str, name: str) -> str:
    """Write <name>.int and <name>.xml into workdir; returns the XML path."""
    c = CASES[name] if name in CASES else LARGE[name]
    os.makedirs(workdir, exist_ok=True)
    sysd = SyntheticSystem("psd", c["nv"], c["zv"], c["twom"], c["parity"], 0.0, 1, name=name)
    ip = os.path.join(workdir, name + ".int")
    xp = os.path.join(workdir, name + ".xml")
    write_int(ip, c["orbits"], -4.0, 1)
    write_xml(xp, sysd, os.path.abspath(ip), c["orbits"])
    txt = open(xp).read()
    if "hwmax" in c:
        txt = txt.replace("<system ", f'<system hwmax="{c["hwmax"]}" ', 1)
    kids = ""
    if "hwrej" in c:
        kids += f'<hwrejection HWMIN="{c["hwrej"][0]}" HWMAX="{c["hwrej"][1]}"/>'
    for lo, hi, idx in c.get("rej", []):
        kids += f'<rejection NMIN="{lo}" NMAX="{hi}">'
        kids += "".join(f'<orbital index="{i}" type="pn"/>' for i in idx) + "</rejection>"
    txt = txt.replace("<matrix JJ", kids + "<matrix JJ", 1)
    with open(xp, "w") as f:
        f.write(txt)
    return xp
