"""Seeded synthetic shell-model inputs: an Oxbash ``.int`` file and a CoSMo
system XML.

The interaction recipe is the one the benchmark configurations describe:
isospin-coupled two-body matrix elements drawn from a seeded Gaussian
(mean 0, sigma 1 MeV) in every allowed (a, b, c, d, J, T) channel,
single-particle energies uniform in [spe_low, 0] MeV, both written with four
decimals, and ``matrix JJ=lambda`` for the J-J+ penalty.

The text layout is what the reference reader accepts
(``ReadOxbashINT``, include/sm/sphericalint.cxx:145-246): a first line with a
positive line count followed by the s.p. energies (so no mass scaling), then
one ``a b c d J T V`` line per unordered bra/ket pair with (c, d) >= (a, b) in
channel order, which keeps ``CheckSphericalINT`` (sphericalint.cxx:43-84)
from zeroing anything.  The XML carries the attributes the reference tools read
(``include/xsm/schema.h``): orbitals with ``n l j type index``, a
``hamiltonian/file/name`` and a ``system`` with ``Av Nv Zv Jz P`` and a
``matrix JJ`` child.
"""
from __future__ import annotations

import os
from dataclasses import dataclass
from fractions import Fraction

import numpy as np

# (name, n, l, 2j) in XML index order.
SD_ORBITS = [("0d5", 0, 2, 5), ("1s1", 1, 0, 1), ("0d3", 0, 2, 3)]
FP_ORBITS = [("0f7", 0, 3, 7), ("1p3", 1, 1, 3), ("0f5", 0, 3, 5), ("1p1", 1, 1, 1)]
SPACES = {"sd": (SD_ORBITS, -4.0), "fp": (FP_ORBITS, -8.0)}


def channel_lines(orbits):
    """All allowed (a, b, c, d, J, T) lines, 1-based orbit labels, in the
    generator's fixed order: for each T in (0, 1), each J, the pairs (a<=b)
    in lexicographic order and (c, d) >= (a, b)."""
    norb = len(orbits)
    pairs = [(a, b) for a in range(norb) for b in range(a, norb)]
    lines = []
    for T in (0, 1):
        jmax = max(orbits[a][3] + orbits[b][3] for a, b in pairs) // 2
        for J in range(0, jmax + 1):
            ok = []
            for (a, b) in pairs:
                ja, jb = orbits[a][3], orbits[b][3]
                if not (abs(ja - jb) // 2 <= J <= (ja + jb) // 2):
                    continue
                if a == b and (J + T) % 2 == 0:
                    continue
                ok.append((a, b))
            for i, (a, b) in enumerate(ok):
                pab = (orbits[a][2] + orbits[b][2]) & 1
                for (c, d) in ok[i:]:
                    if (orbits[c][2] + orbits[d][2]) & 1 != pab:
                        continue
                    lines.append((a + 1, b + 1, c + 1, d + 1, J, T))
    return lines


@dataclass
class SyntheticSystem:
    space: str
    nv: int          # valence neutrons
    zv: int          # valence protons
    twom: int = 0    # 2*Jz of the M-scheme sector
    parity: str = "+"
    jj: float = 0.5  # lambda of the J-J+ term
    seed: int = 0
    name: str = ""

    def label(self) -> str:
        return self.name or f"{self.space}{self.nv}{self.zv}m{self.twom}s{self.seed}"


def write_int(path: str, orbits, spe_low: float, seed: int) -> int:
    """Write the seeded Oxbash interaction; returns the number of TBME lines."""
    rng = np.random.Generator(np.random.PCG64(seed))
    spe = rng.uniform(spe_low, 0.0, len(orbits))
    lines = channel_lines(orbits)
    vals = rng.normal(0.0, 1.0, len(lines))
    with open(path, "w") as f:
        f.write("! synthetic seeded Gaussian TBME (cosmo_gb300.synthetic), seed %d\n" % seed)
        f.write(" %d " % len(lines) + " ".join("%.4f" % e for e in spe) + "\n")
        for (a, b, c, d, J, T), v in zip(lines, vals):
            f.write("%3d%3d%3d%3d %4d%3d %10.4f\n" % (a, b, c, d, J, T, v))
    return len(lines)


def _jstr(twoj: int) -> str:
    return f"{twoj}/2" if twoj % 2 else str(twoj // 2)


def write_xml(path: str, sysd: SyntheticSystem, int_path: str, orbits=None,
              mbs_name: str | None = None, hname: str = "syn") -> None:
    orbits = orbits if orbits is not None else SPACES[sysd.space][0]
    jz = _jstr(sysd.twom) if sysd.twom >= 0 else "-" + _jstr(-sysd.twom)
    out = ['<?xml version="1.0"?>', "<cosmo>", f' <valencespace name="{sysd.space}">']
    for i, (nm, n, l, tj) in enumerate(orbits):
        out.append(f'  <orbital name="{nm}" n="{n}" l="{l}" j="{_jstr(tj)}" type="pn" index="{i + 1}"/>')
    out.append(" </valencespace>")
    out.append(f' <hamiltonian name="{hname}"><file format="ascii"><name>{int_path}</name></file></hamiltonian>')
    mbs = f'<ManyBodyStates name="{mbs_name}"/>' if mbs_name else ""
    out.append(f' <system name="{sysd.label()}" Av="{sysd.nv + sysd.zv}" Nv="{sysd.nv}" Zv="{sysd.zv}"'
               f' Jz="{jz}" P="{sysd.parity}">{mbs}<matrix JJ="{sysd.jj}"/></system>')
    out.append("</cosmo>")
    with open(path, "w") as f:
        f.write("\n".join(out) + "\n")


def make_system(workdir: str, sysd: SyntheticSystem, mbs_name: str | None = None) -> tuple[str, str]:
    """Write ``<label>.int`` and ``<label>.xml`` into ``workdir``; returns both paths."""
    os.makedirs(workdir, exist_ok=True)
    orbits, spe_low = SPACES[sysd.space]
    ip = os.path.join(workdir, sysd.label() + ".int")
    xp = os.path.join(workdir, sysd.label() + ".xml")
    write_int(ip, orbits, spe_low, sysd.seed)
    write_xml(xp, sysd, os.path.abspath(ip), orbits, mbs_name)
    return ip, xp


def batched_sd_systems(count: int = 64, seed: int = 2024) -> list[SyntheticSystem]:
    """The 64-problem sd batch: A ~ U{2..12}, Z ~ U{max(0,A-12)..min(12,A)},
    2M in {0, 2} for even A and {1, 3} for odd A, each with its own seed."""
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    for k in range(count):
        a = int(rng.integers(2, 13))
        z = int(rng.integers(max(0, a - 12), min(12, a) + 1))
        twom = int(rng.integers(0, 2)) * 2 + (a & 1)
        out.append(SyntheticSystem("sd", a - z, z, twom, "+", 0.5, seed * 1000 + k,
                                   name=f"batch{k:02d}"))
    return out


def spin_fraction(twoj: int) -> Fraction:
    return Fraction(twoj, 2)
