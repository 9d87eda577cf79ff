"""Wide valence-space cases: the spsdpf space of the reference's 33Al example
(0s, 0p, 1s0d, 1p0f in the order of the reference's interactions/int.xml:
40 m-states per species), 20 neutrons and 13 protons with 2Jz = 1, the 0 hw
positive-parity window (119 states) and the 1 hw negative-parity one (23,842
states) of the example, and an untruncated 2 neutrons + 1 proton system.  A seeded synthetic interaction stands in for fsu (the
bases are the example's, the spectra are not).  Shared by the fixture script
(make_golden.py, which runs the reference's XsysmbsOMP and ref_dump on these
XML files) and the tests (which rebuild the same XML)."""
from __future__ import annotations

import os

from cosmo_gb300.synthetic import SyntheticSystem, write_int, write_xml

SPSDPF_ORBITS = [("0s1", 0, 0, 1), ("0p3", 0, 1, 3), ("0p1", 0, 1, 1), ("0d5", 0, 2, 5), ("0d3", 0, 2, 3),
                 ("1s1", 1, 0, 1), ("0f7", 0, 3, 7), ("0f5", 0, 3, 5), ("1p3", 1, 1, 3), ("1p1", 1, 1, 1)]
SEED = 33

# name: system, the <hwrejection> window, reference Davidson states, full dumps
CASES = {
    "spsdpf_0hw": dict(nv=20, zv=13, twom=1, parity="+", hw=(0, 0), nstates=10, full=True),
    "spsdpf_1hw": dict(nv=20, zv=13, twom=1, parity="-", hw=(1, 1), nstates=5, full=False),
    # untruncated: every configuration of 2 neutrons and 1 proton in the 40 m-states
    "spsdpf_21": dict(nv=2, zv=1, twom=1, parity="-", hw=None, nstates=5, full=True),
}


def write_case(workdir: str, name: str) -> str:
    """Write the interaction and <name>.xml into workdir; returns the XML path."""
    c = CASES[name]
    os.makedirs(workdir, exist_ok=True)
    sysd = SyntheticSystem("spsdpf", c["nv"], c["zv"], c["twom"], c["parity"], 0.0, SEED, name=name)
    ip = os.path.join(workdir, f"spsdpf_s{SEED}.int")
    xp = os.path.join(workdir, name + ".xml")
    write_int(ip, SPSDPF_ORBITS, -8.0, SEED)
    write_xml(xp, sysd, os.path.abspath(ip), SPSDPF_ORBITS)
    txt = open(xp).read()
    if c["hw"] is not None:
        lo, hi = c["hw"]
        txt = txt.replace("<matrix JJ", f'<hwrejection HWMIN="{lo}" HWMAX="{hi}"/><matrix JJ', 1)
    with open(xp, "w") as f:
        f.write(txt)
    return xp


# The reference's own 33Al example (EXAMPLE-33Al-fsu.md) with its fsu9
# interaction files, which stay in the reference checkout: the system node
# the reference's XML creator writes (Av, Nv, Zv, A, Tz, Jz, P and the hw
# window), the fsu9 file list of the reference's interactions/int.xml (its
# formulascale element is read by no reference code), and the levels the
# example prints (Xlevels: name, T, Ex, E).
FSU9_FILES = [("spsdpfpb.int", ""),
              ("fsu9/spsdfp-fsu9.int", '<formulascale rank="2">(18/A)^0.3</formulascale>'),
              ("fsu9/0p1sd.int", ""), ("fsu9/0p3sd.int", ""), ("0s0f1p0.int", ""),
              ("spsdpfcm.int", '<scale rank="1">10.000000</scale><scale rank="2">10.000000</scale>')]
EXAMPLE_33AL = {"+": (0, 0, 119), "-": (1, 1, 23842)}
EXAMPLE_33AL_LEVELS = [("5/2+(1)", -303.079), ("1/2-(1)", -301.132), ("7/2-(1)", -299.928),
                       ("5/2-(1)", -299.874), ("3/2-(1)", -299.817)]


def write_33al(workdir: str, int_dir: str, parity: str) -> str:
    """The example's system of one parity with the fsu9 files read from
    int_dir (the reference's interactions/spsdpf); returns the XML path."""
    hwmin, hwmax, _ = EXAMPLE_33AL[parity]
    os.makedirs(workdir, exist_ok=True)
    out = ['<?xml version="1.0"?>', '<cosmo version="4.1">', ' <valencespace name="spsdpf">',
           '  <core name="0n" N="0" Z="0"/>']
    for i, (nm, n, l, tj) in enumerate(SPSDPF_ORBITS):
        j = f"{tj}/2"
        out.append(f'  <orbital name="{nm}" n="{n}" l="{l}" j="{j}" type="pn" index="{i + 1}"/>')
    out.append(" </valencespace>")
    out.append(' <hamiltonian name="fsu9" valencespace="spsdpf">')
    for f, extra in FSU9_FILES:
        out.append(f'  <file format="ascii"><name>{os.path.join(int_dir, f)}</name>{extra}</file>')
    out.append(" </hamiltonian>")
    name = f"33Al_fsu9_M1T7{parity}"
    out.append(f' <system Av="33" Nv="20" Zv="13" A="33" Tz="7/2" Jz="1/2" P="{parity}" name="{name}">'
               f'<hwrejection HWMAX="{hwmax}" HWMIN="{hwmin}"/></system>')
    out.append("</cosmo>")
    path = os.path.join(workdir, f"33Al_fsu9{parity}.xml")
    with open(path, "w") as f:
        f.write("\n".join(out) + "\n")
    return path
