"""CPU ORACLE — test infrastructure only.

A pure-Python restatement of the reference's problem setup, so that the CPU
side of the checks and of the timed CPU baseline needs nothing from the
product library:

* the XML system subset and the m-scheme single-particle table
  (SM::Make, include/xsm/xSingleParticleStates.cxx:26-104; system attributes
  as SM::MakeMBS2(XMLNode, sps), include/xsm/xManyBodyStates.cxx:22-91);
* the Oxbash reader with its repeated-line check (ReadXMLINT,
  include/xsm/xsphericalint.cxx:16-49; ReadOxbashINT and CheckSphericalINT,
  include/sm/sphericalint.cxx:43-84,145-246);
* the conversion to forward-ordered m-scheme operator terms: one-body ESP
  (MakeESPO, include/sm/MakeSPO.cxx:195-210), two-body VSPX (PPInteraction2sp,
  include/sm/spherical2sp.cxx:790-814, each line through AddPPVsp,
  include/sm/AddPPVsp.cxx:32-147) and the lambda J-J+ penalty (SPJJ,
  include/sm/spherical2sp.cxx:629-711 with SPSqrM and StripHermitianOperator,
  include/sm/cioperators.cxx:200-287), added as xReadSPInt does
  (include/xsm/xReadSPInt.cxx:58-73,273-287).

Clebsch-Gordan coefficients come from Racah's formula evaluated in exact
rational arithmetic (one rounding to double at the end).  TBMEs and s.p.
energies are rounded to single precision as the reference's std::stof does.
Pinned against the reference's own operator terms (tests/golden fixtures).
"""
from __future__ import annotations

import math
import os
import xml.etree.ElementTree as ET
from fractions import Fraction
from functools import lru_cache

import numpy as np


def _f32(text: str) -> float:
    """std::stof then widening to double."""
    return float(np.float32(float(text)))


def spin2(text: str) -> int:
    """Doubled spin of "5/2", "3" or "1.5" (the reference's spin(const char*),
    include/sm/spinclass.cxx:57-79)."""
    text = text.strip()
    if "/" in text:
        a, b = text.split("/")
        if b.strip() != "2":
            raise ValueError(f"bad spin {text}")
        return int(a)
    x = float(text)
    r = int(2 * x + 0.5) if x >= 0 else int(2 * x - 0.5)
    if abs(r - 2 * x) > 0.01:
        raise ValueError(f"spin {text} is not (half-)integer")
    return r


def _xml_value(node, key):
    """getXMLData: an attribute, else the text of a child element."""
    v = node.get(key)
    if v is None:
        c = node.find(key)
        if c is not None and c.text is not None:
            v = c.text.strip()
    return v


class System:
    """Parsed system: s.p. table rows (level n l 2j 2m 2t 2tz parity), neutrons
    first, and the system quantum numbers."""

    def __init__(self, xml_path: str, system_name: str | None = None):
        root = ET.parse(xml_path).getroot()
        if root.tag != "cosmo":
            raise ValueError("root element is not <cosmo>")
        self.xml_dir = os.path.dirname(os.path.abspath(xml_path))
        vs = root.find("valencespace")
        orbitals = sorted(vs.findall("orbital"), key=lambda o: int(o.get("index")))
        neutrons, protons = [], []
        for o in orbitals:
            idx = int(o.get("index"))
            j2 = spin2(o.get("j"))
            n = int(o.get("n", "0"))
            l = int(o.get("l", "0"))
            par = l & 1
            if o.get("P") is not None:
                par = 1 if o.get("P") in ("-", "1") else 0
            t2 = spin2(o.get("T")) if o.get("T") is not None else 1
            typ = o.get("type", "pn")
            for m2 in range(-j2, j2 + 1, 2):
                if typ in ("pn", "n"):
                    neutrons.append((idx - 1, n, l, j2, m2, t2, 1, par))
                if typ in ("pn", "p"):
                    protons.append((idx - 1, n, l, j2, m2, t2, -1, par))
        self.sps = np.array(neutrons + protons, dtype=np.int32)
        self.n_neutron_states = len(neutrons)
        systems = root.findall("system")
        if system_name:
            sn = [s for s in systems if s.get("name") == system_name][0]
        else:
            if len(systems) != 1:
                raise ValueError("several <system> nodes: give a system name")
            sn = systems[0]
        self.name = sn.get("name", "system")
        A = int(sn.get("Av"))
        if sn.get("Nv") is not None and sn.get("Zv") is not None:
            self.nv, self.zv = int(sn.get("Nv")), int(sn.get("Zv"))
        else:
            tz2 = spin2(sn.get("Tz"))
            self.zv, self.nv = (A - tz2) // 2, (A + tz2) // 2
        self.A = A
        self.twom = spin2(sn.get("Jz")) if sn.get("Jz") is not None else A % 2
        self.parity = 1 if sn.get("P", "+")[0] == "-" else 0
        self.truncated = (_xml_value(sn, "hwmax") is not None or sn.find("hwrejection") is not None
                          or sn.find("rejection") is not None)
        mx = sn.find("matrix")
        self.jj = float(mx.get("JJ")) if mx is not None and mx.get("JJ") is not None else None
        self.files = []
        for f in root.find("hamiltonian").findall("file"):
            scale = [1.0] * 10
            for s in f.findall("scale"):
                scale[int(s.get("rank"))] *= float(s.text)
            self.files.append((f.find("name").text.strip(), scale[1], scale[2]))

    def resolve(self, name: str) -> str:
        cands = [name, name + ".int"]
        if not os.path.isabs(name):
            cands += [os.path.join(self.xml_dir, name), os.path.join(self.xml_dir, name + ".int")]
        for c in cands:
            if os.path.exists(c):
                return c
        raise FileNotFoundError(name)


def read_oxbash(path: str, A: int, spescaling: float, vscaling: float):
    """ReadOxbashINT: s.p. energies per level and TBMEs keyed (c, d, a, b, J, T)
    (the file's a b c d become [2] [3] [0] [1], 0-based), repeated lines
    zeroed by CheckSphericalINT."""
    spe: list[float] = []
    tmp: dict[tuple, float] = {}
    linecount = 0
    with open(path) as fh:
        for line in fh:
            line = line.rstrip("\n").rstrip("\r")
            if not line:
                continue
            line = line.lstrip()
            if line and line[0] in "#!%/":
                continue
            tok = [t for t in line.replace(",", " ").split() if t]
            if linecount == 0:
                intlines = int(tok[0])
                words = len(tok) - 1 - (3 if intlines < 0 else 0)
                if len(spe) < words:
                    spe += [0.0] * (words - len(spe))
                for i in range(words):
                    spe[i] += _f32(tok[i + 1]) * spescaling
                if intlines < 0:
                    acore, ascale, spow = (_f32(tok[words + k]) for k in (1, 2, 3))
                    if A >= 0:
                        vscaling *= math.pow(ascale / (A + acore), spow)
            else:
                if len(tok) < 7:
                    linecount += 1
                    continue
                key = (int(tok[2]) - 1, int(tok[3]) - 1, int(tok[0]) - 1, int(tok[1]) - 1, int(tok[4]), int(tok[5]))
                tmp[key] = tmp.get(key, 0.0) + vscaling * _f32(tok[6])
            linecount += 1
    keys = sorted(tmp)

    def pairs(k):
        return tuple(sorted(k[0:2])) + tuple(sorted(k[2:4]))
    for i, k1 in enumerate(keys):
        a = pairs(k1)
        for k2 in keys[i + 1:]:
            if k1[4] != k2[4] or k1[5] != k2[5]:
                continue
            b = pairs(k2)
            if a == b or (a[0:2] == b[2:4] and a[2:4] == b[0:2]):
                tmp[k2] = 0.0
    return spe, tmp


@lru_cache(maxsize=None)
def clebsch_gordan(j1: int, m1: int, j2: int, m2: int, j3: int, m3: int) -> float:
    """<j1 m1 j2 m2 | j3 m3>, doubled arguments, Racah's formula in exact
    rational arithmetic: sqrt(P) * S with P and S rationals."""
    if m1 + m2 != m3 or abs(m1) > j1 or abs(m2) > j2 or abs(m3) > j3:
        return 0.0
    if (j1 + m1) % 2 or (j2 + m2) % 2 or (j3 + m3) % 2:
        return 0.0
    if j3 > j1 + j2 or j3 < abs(j1 - j2) or (j1 + j2 + j3) % 2:
        return 0.0
    f = math.factorial
    a, b, c = (j1 + j2 - j3) // 2, (j1 - j2 + j3) // 2, (-j1 + j2 + j3) // 2
    d = (j1 + j2 + j3) // 2 + 1
    P = Fraction((j3 + 1) * f(a) * f(b) * f(c) * f((j1 + m1) // 2) * f((j1 - m1) // 2) * f((j2 + m2) // 2)
                 * f((j2 - m2) // 2) * f((j3 + m3) // 2) * f((j3 - m3) // 2), f(d))
    S = Fraction(0)
    for k in range(d + 1):
        e = [(j1 + j2 - j3) // 2 - k, (j1 - m1) // 2 - k, (j2 + m2) // 2 - k, (j3 - j2 + m1) // 2 + k,
             (j3 - j1 - m2) // 2 + k]
        if min(e) < 0:
            continue
        den = f(k)
        for x in e:
            den *= f(x)
        S += Fraction(-1 if k % 2 else 1, den)
    if S == 0:
        return 0.0
    # sqrt(P) * S = sign(S) * sqrt(P * S^2), rounded once
    v = P * S * S
    return math.copysign(math.sqrt(v.numerator / v.denominator), S)


def add_pp_vsp(vsp: dict, sps: np.ndarray, ijk: tuple, V: float) -> None:
    """AddPPVsp (include/sm/AddPPVsp.cxx:32-147): every m-state combination of
    the four orbit levels with conserved 2m and 2tz, Clebsch-Gordan weights in
    J and T, 1/sqrt((1+d_ab)(1+d_cd)), sqrt(2) for a pn pair of separately
    indexed orbits, the pair-reordering fermion sign, forward pair order, /2
    for a line whose bra and ket orbit pairs coincide and x2 on the m-pair
    diagonal.  States visited in ascending index order (a0, a1, a2; a3 is the
    one state of its level that conserves 2m and 2tz)."""
    lvl = sps[:, 0]
    by = [np.flatnonzero(lvl == ijk[q]).tolist() for q in range(4)]
    if any(not b for b in by):
        return
    at = {(int(sps[i, 4]), int(sps[i, 6])): i for i in by[3]}
    L, T = 2 * ijk[4], 2 * ijk[5]
    norm = math.sqrt((float(ijk[0] == ijk[1]) + 1.0) * (float(ijk[2] == ijk[3]) + 1.0))

    def pn_pair(x, y):
        return (sps[x, 1] == sps[y, 1] and sps[x, 3] == sps[y, 3] and sps[x, 6] == -sps[y, 6]
                and sps[x, 7] == sps[y, 7])
    for a0 in by[0]:
        j0, m0, t0, z0 = (int(sps[a0, k]) for k in (3, 4, 5, 6))
        for a1 in by[1]:
            if (j0 & 1) and a1 == a0:
                continue
            j1, m1, t1, z1 = (int(sps[a1, k]) for k in (3, 4, 5, 6))
            cg01 = clebsch_gordan(j0, m0, j1, m1, L, m0 + m1)
            ct01 = clebsch_gordan(t0, z0, t1, z1, T, z0 + z1)
            for a2 in by[2]:
                j2, m2, t2, z2 = (int(sps[a2, k]) for k in (3, 4, 5, 6))
                a3 = at.get((m0 + m1 - m2, z0 + z1 - z2))
                if a3 is None:
                    continue
                if (j2 & 1) and a2 == a3:
                    continue
                j3, m3, t3, z3 = (int(sps[a3, k]) for k in (3, 4, 5, 6))
                h = cg01 * clebsch_gordan(j2, m2, j3, m3, L, m2 + m3)
                h *= ct01
                h *= clebsch_gordan(t2, z2, t3, z3, T, z2 + z3)
                if abs(h) < 1e-9:
                    continue
                h = h * V / norm
                if ijk[0] != ijk[1] and pn_pair(a0, a1):
                    h *= math.sqrt(2.0)
                if ijk[2] != ijk[3] and pn_pair(a2, a3):
                    h *= math.sqrt(2.0)
                b = [a0, a1, a2, a3]
                phase = False
                if b[0] > b[1]:
                    b[0], b[1] = b[1], b[0]
                    phase ^= bool(j0 & 1)
                if b[2] > b[3]:
                    b[2], b[3] = b[3], b[2]
                    phase ^= bool(j2 & 1)
                if (b[2], b[3]) < (b[0], b[1]):
                    b = [b[2], b[3], b[0], b[1]]
                if ijk[0] == ijk[2] and ijk[1] == ijk[3]:
                    h /= 2.0
                if b[0] == b[2] and b[1] == b[3]:
                    h *= 2.0
                k = tuple(b)
                vsp[k] = vsp.get(k, 0.0) + (-h if phase else h)


def j_minus_j_plus(sps: np.ndarray):
    """SPJJ: the one-body J+ (SPJPlus, q = sqrt((j-m)(j+m+2))/2 on jm -> jm+1,
    keyed (annihilated, created)), squared by SPSqrM into one-body and two-body
    parts, backward keys stripped (StripHermitianOperator)."""
    ns = len(sps)
    jo = {}
    for p0 in range(ns):
        for p1 in range(p0 + 1, ns):
            s0, s1 = sps[p0], sps[p1]
            if s0[0] != s1[0] or s0[6] != s1[6]:
                continue
            if s0[4] + 2 == s1[4]:
                jo[(p0, p1)] = math.sqrt((s0[3] - s0[4]) * (s0[3] + s0[4] + 2.0)) / 2.0
            elif s0[4] - 2 == s1[4]:
                jo[(p1, p0)] = math.sqrt((s1[3] - s1[4]) * (s1[3] + s1[4] + 2.0)) / 2.0
    items = sorted(jo.items())
    jsp, vsp = {}, {}
    for (i0, i1), iv in items:
        for (j0, j1), jv in items:
            h = iv * jv
            if abs(h) < 1e-8:
                continue
            if j1 == i1:
                jsp[(j0, i0)] = jsp.get((j0, i0), 0.0) + h
            aa = [j1, i0, j0, i1]
            if aa[0] > aa[1]:
                aa[0], aa[1] = aa[1], aa[0]
                h = -h
            if aa[2] > aa[3]:
                aa[2], aa[3] = aa[3], aa[2]
                h = -h
            k = tuple(aa)
            vsp[k] = vsp.get(k, 0.0) + h
    jsp = {k: v for k, v in jsp.items() if not k[1] < k[0]}
    vsp = {k: v for k, v in vsp.items() if not (k[2], k[3]) < (k[0], k[1])}
    return jsp, vsp


def operator_terms(xml_path: str, system_name: str | None = None):
    """(System, one-body keys (n, 2) int32, values, two-body keys (m, 4) int32,
    values): xReadSPInt's ESP and VSPX with lambda J-J+ added, keys sorted."""
    sysd = System(xml_path, system_name)
    sps = sysd.sps
    spe: list[float] = []
    tbme: dict[tuple, float] = {}
    for name, s1, s2 in sysd.files:
        e, t = read_oxbash(sysd.resolve(name), sysd.A, s1, s2)
        if len(spe) < len(e):
            spe += [0.0] * (len(e) - len(spe))
        for i, x in enumerate(e):
            spe[i] += x
        for k, v in t.items():
            if k[5] < 0:
                raise ValueError("Tz-resolved interactions are not restated")
            tbme[k] = tbme.get(k, 0.0) + v
    one: dict[tuple, float] = {}
    for i in range(len(sps)):
        one[(i, i)] = one.get((i, i), 0.0) + spe[int(sps[i, 0])]
    two: dict[tuple, float] = {}
    for k in sorted(tbme):
        add_pp_vsp(two, sps, k, tbme[k])
    if sysd.jj is not None:
        jsp, vjj = j_minus_j_plus(sps)
        for k, v in jsp.items():
            one[k] = one.get(k, 0.0) + v * sysd.jj
        for k, v in vjj.items():
            two[k] = two.get(k, 0.0) + v * sysd.jj
    k1 = sorted(one)
    k2 = sorted(two)
    return (sysd, np.array(k1, dtype=np.int32).reshape(-1, 2), np.array([one[k] for k in k1]),
            np.array(k2, dtype=np.int32).reshape(-1, 4), np.array([two[k] for k in k2]))
