"""CPU ORACLE — test infrastructure only.

A restatement of the reference's XSHLEMB (xmlshell/XSHLEMB.cpp:116-372): the
m-scheme one-body transition operators (include/sm/EMspherical2sp.cxx:
ElectricSPMultipole, MagneticSPMultipole, BetaJAMultipole with oscillator
radial integrals, ROperator_YS, ReducedToFull; SPTPlus and
Hermitian2FullOperator for the Fermi operator, include/sm/spherical2sp.cxx:
664-700, include/sm/cioperators.cxx:244-269), the overlap <D| O |P>
(PPMatrix::OverlapNH, include/sm/PPMatrix.cxx:275-302, with ActFermiOperator's
annihilate-then-create phases) and the B values, moments and unit conversions
the tool writes; and XSHLAO's occupation numbers (SM::occupation,
include/sm/occupation.cxx:55-70).  Angular-momentum coefficients and oscillator radial
integrals come from their closed forms (Racah; Lawson, Theory of the Nuclear
Shell Model, eq. 1.11a) in exact rational arithmetic, rounded once.  Pinned
against the reference XSHLEMB's own output (tests/golden, em_sd22).
"""
from __future__ import annotations

import math
from fractions import Fraction

import numpy as np

from .interaction import clebsch_gordan

HBARC = 197.327053
MU_P, MU_N = 2.792847351, -1.91304273

# s.p. table columns (interaction.System.sps)
LEVEL, N, L, J2, M2, T2, TZ2, PAR = range(8)


def _fact(n: int) -> int:
    return math.factorial(n) if n > 1 else 1


def _dfact(n: int) -> int:
    r = 1
    for i in range(3, n + 1, 2):
        r *= i
    return r


def ho_radial(L: int, n1: int, l1: int, n2: int, l2: int, origin_positive: bool = True) -> float:
    """<n1 l1| r^L |n2 l2> of oscillator functions (length 1), Lawson 1.11a;
    factorials of negative integers count as 1 (the reference's convention
    for the l-forbidden terms it keeps)."""
    t1, t2 = (l2 - l1 + L) // 2, (l1 - l2 + L) // 2
    qmin, qmax = max(0, n1 - t1, n2 - t2), min(n1, n2)
    if qmin > qmax:
        return 0.0
    S = Fraction(0)
    for q in range(qmin, qmax + 1):
        S += Fraction(_dfact(l1 + l2 + L + 2 * q + 1),
                      2 ** q * _fact(q) * _fact(n1 - q) * _fact(n2 - q) * _fact(q + t2 - n2) * _fact(q + t1 - n1))
    # R^2 = n1! n2! / (dfs) 2^(n1+n2-L) (t1! t2! S)^2
    e = n1 + n2 - L
    R2 = Fraction(_fact(n1) * _fact(n2), _dfact(2 * n1 + 2 * l1 + 1) * _dfact(2 * n2 + 2 * l2 + 1)) \
        * (Fraction(2) ** e) * (_fact(t1) * _fact(t2) * S) ** 2
    r = math.sqrt(R2.numerator / R2.denominator)
    return -r if (origin_positive and (n1 + n2) & 1) else r


def _delta2(a: int, b: int, c: int):
    if c > a + b or c < abs(a - b) or (a + b + c) % 2:
        return None
    return Fraction(_fact((a + b - c) // 2) * _fact((a - b + c) // 2) * _fact((-a + b + c) // 2),
                    _fact((a + b + c) // 2 + 1))


def six_j(a: int, b: int, c: int, d: int, e: int, f: int) -> float:
    """{a/2 b/2 c/2; d/2 e/2 f/2} by Racah's formula (doubled arguments)."""
    ds = [_delta2(a, b, c), _delta2(a, e, f), _delta2(d, b, f), _delta2(d, e, c)]
    if any(x is None for x in ds):
        return 0.0
    s = [(a + b + c) // 2, (a + e + f) // 2, (d + b + f) // 2, (d + e + c) // 2]
    p = [(a + b + d + e) // 2, (b + c + e + f) // 2, (c + a + f + d) // 2]
    S = Fraction(0)
    for t in range(max(s), min(p) + 1):
        den = 1
        for x in s:
            den *= _fact(t - x)
        for x in p:
            den *= _fact(x - t)
        S += Fraction((-1) ** t * _fact(t + 1), den)
    W = ds[0] * ds[1] * ds[2] * ds[3] * S * S
    return math.copysign(math.sqrt(W.numerator / W.denominator), S) if S else 0.0


def _sgn(a: int) -> float:
    return -1.0 if a & 1 else 1.0


def _y_sigma(f, i, q: int, K: int) -> float:
    """<f|| (Y_q sigma)_K ||i> (ROperator_YS) without the radial part."""
    if (i[PAR] - f[PAR] + q) & 1:
        return 0.0
    base = math.sqrt((i[J2] + 1.0) / math.pi) / 2.0
    lo = clebsch_gordan(i[J2], 1, 2 * K, 0, f[J2], 1)
    hi = clebsch_gordan(i[J2], -1, 2 * K, 2, f[J2], 1)
    ph = _sgn((f[J2] - 1) // 2 - f[L])
    if K - q == -1:
        return base * (_sgn((i[J2] - f[J2]) // 2 + K) * lo * math.sqrt(2 * K + 1.0) - hi * ph * math.sqrt(K))
    if K - q == 0:
        return base * ph * hi * math.sqrt(2 * K + 1.0)
    if K - q == 1:
        return base * (_sgn((i[J2] + f[J2]) // 2 + K) * lo * math.sqrt(K) - hi * ph * math.sqrt(K + 1.0))
    return 0.0


def _full(f, i, K: int, red: float) -> float:
    return red * clebsch_gordan(int(i[J2]), int(i[M2]), 2 * K, int(f[M2] - i[M2]), int(f[J2]), int(f[M2])) \
        / math.sqrt(f[J2] + 1.0)


def transition_terms(sps: np.ndarray, op: dict, kappa: int) -> list:
    """[(i, f, v)]: v a+_f a_i of the operator component with projection kappa.
    op: name (E2, M1, GT-, GT+, F), K, en, ep, mu_n, mu_p, gl_n, gl_p,
    origin_positive."""
    name, K = op["name"], op["K"]
    orig = op.get("origin_positive", True)
    out = []
    ns = len(sps)
    sps = [tuple(int(x) for x in r) for r in sps]
    if name[0] == "F":
        for a in range(ns):
            for b in range(a + 1, ns):
                x, y = sps[a], sps[b]
                if (x[M2], x[N], x[PAR], x[L], x[T2], x[J2]) != (y[M2], y[N], y[PAR], y[L], y[T2], y[J2]):
                    continue
                if abs(x[TZ2] - y[TZ2]) != 2:
                    continue
                ip, inn = (a, b) if x[TZ2] < y[TZ2] else (b, a)
                p = sps[ip]
                v = math.sqrt((p[T2] - p[TZ2]) * (p[T2] + p[TZ2] + 2.0)) / 2.0
                out += [(ip, inn, v), (inn, ip, v)]
        return out
    for fi in range(ns):
        for ii in range(ns):
            f, i = sps[fi], sps[ii]
            if i[M2] + 2 * kappa != f[M2]:
                continue
            if name[0] == "E":
                if f[TZ2] != i[TZ2] or (i[L] + K - f[L]) & 1:
                    continue
                v = op["en"] if f[TZ2] == 1 else op["ep"]
                v *= _sgn((i[J2] - f[J2]) // 2 + K)
                v *= math.sqrt((2 * K + 1.0) * (i[J2] + 1.0) / (4 * math.pi))
                v *= ho_radial(K, f[N], f[L], i[N], i[L], orig)
                v *= clebsch_gordan(i[J2], 1, 2 * K, 0, f[J2], 1)
            elif name[0] == "M":
                if f[TZ2] != i[TZ2] or (i[L] - f[L] + K - 1) & 1:
                    continue
                neutron = f[TZ2] == 1
                gl = op["gl_n"] if neutron else op["gl_p"]
                gs = 2.0 * (op["mu_n"] if neutron else op["mu_p"])
                a = _sgn((i[J2] + f[J2]) // 2 - K) * (f[J2] + 1.0) / 2.0 + (i[J2] + 1.0) / 2.0
                a = (a * _sgn(i[L] - (i[J2] - 1) // 2) / K + 1.0) * clebsch_gordan(i[J2], 1, 2 * K, 0, f[J2], 1)
                a *= K / 2.0 * (gs - 2.0 * gl / (K + 1.0))
                b = six_j(i[J2], 2, i[J2], 2 * K - 2, f[J2], 2 * K) * clebsch_gordan(i[J2], 1, 2 * K - 2, 0, f[J2], 1)
                b *= math.sqrt(K * (4.0 * K * K - 1) * i[J2] * (i[J2] + 2.0) * (i[J2] + 1)) * gl
                b *= _sgn((i[J2] + f[J2]) // 2 + K) / (K + 1.0)
                v = (a + b) * _sgn((i[J2] - f[J2]) // 2 + K - 1)
                v *= math.sqrt((2 * K + 1.0) * (i[J2] + 1.0) / (4 * math.pi))
                v *= ho_radial(K - 1, f[N], f[L], i[N], i[L], orig)
            elif name[0] == "G":
                plus = name == "GT+"
                if f[TZ2] != i[TZ2] + (2 if plus else -2) or (i[L] - f[L]) & 1:
                    continue
                v = _y_sigma(f, i, 0, K) * ho_radial(0, f[N], f[L], i[N], i[L], True)
                if v == 0.0:
                    continue
                v = _full(f, i, K, v)
                v *= (math.sqrt((i[T2] - i[TZ2]) * (i[T2] + i[TZ2] + 2.0)) / 2.0 if plus
                      else math.sqrt((i[T2] + i[TZ2]) * (i[T2] - i[TZ2] + 2.0)) / 2.0)
                out.append((ii, fi, v * math.sqrt(4 * math.pi)))
                continue
            else:
                raise ValueError(name)
            if v == 0.0:
                continue
            out.append((ii, fi, _full(f, i, K, v)))
    return out


def onebody_amplitudes(zp: np.ndarray, vp: np.ndarray, zd: np.ndarray, vd: np.ndarray, terms: list) -> np.ndarray:
    """amp[q, p] = <D_q| sum v a+_f a_i |P_p> (PPMatrix::OverlapNH of the
    operator): each term on every parent determinant, annihilation of i with
    the phase of the states of P below it, creation of f with the phase of the
    states of P - i below it, located in the daughter basis."""
    index = {tuple(int(x) for x in t): k for k, t in enumerate(zd)}
    vp = np.asarray(vp, dtype=np.float64).reshape(-1, len(zp))
    vd = np.asarray(vd, dtype=np.float64).reshape(-1, len(zd))
    w = np.zeros((len(zd), len(vp)))
    for pi, P in enumerate(zp):
        p = [int(x) for x in P]
        ps = set(p)
        for i, f, v in terms:
            if i not in ps:
                continue
            sign = p.index(i)
            rest = [x for x in p if x != i]
            if f in rest:
                continue
            sign += sum(1 for x in rest if x < f)
            k = index.get(tuple(sorted(rest + [f])))
            if k is None:
                continue
            w[k] += (-v if sign & 1 else v) * vp[:, pi]
    return vd @ w


def oscillator_b2(A: int) -> float:
    hw = 45.0 * A ** (-1.0 / 3.0) - 25.0 * A ** (-2.0 / 3.0)
    return HBARC * HBARC / (hw * 938.9186945)


def weisskopf(t: str, Lm: int, A: int, B: float) -> float:
    b = oscillator_b2(A)
    if t == "E":
        return b ** Lm * B / (1.2 ** (2 * Lm) * (3.0 / (Lm + 3.0)) ** 2 * A ** (2 * Lm / 3.0) / (4 * math.pi))
    if t == "M":
        return b ** (Lm - 1) * B / (10.0 * 1.2 ** (2 * Lm - 2) * (3.0 / (Lm + 3.0)) ** 2 * A ** ((2 * Lm - 2) / 3.0)
                                    / math.pi)
    return -1.0


def standard_units(t: str, Lm: int, A: int, B: float) -> float:
    b = oscillator_b2(A)
    return b ** Lm * B if t == "E" else (b ** (Lm - 1) * B if t == "M" else -1.0)


def transitions(op: dict, P: list, D: list, amp: np.ndarray, A: int = 1, flags=()) -> tuple:
    """The <transition> and <moment> records XSHLEMB writes: per parent state
    a list of dicts (final, B[, weisskopf, Bu, logft]) and a list of moments.
    P, D: state dicts (twoJ, twoJz, twoT, twoTz, E (from the .EE file), name).
    amp[q, p] = <D_q| O |P_p>."""
    K, t = op["K"], op["name"][0]
    trans, moms = [], []
    for pi, p in enumerate(P):
        tr, mo = [], []
        for qi, q in enumerate(D):
            jz = p["twoJz"] - q["twoJz"]
            c = clebsch_gordan(q["twoJ"], q["twoJz"], 2 * K, jz, p["twoJ"], p["twoJz"])
            if abs(c) < 1e-10:
                continue
            x = amp[qi, pi]
            B = (x / c) ** 2
            rec = {"final": q["name"], "B": B}
            if "-w" in flags and t in "EM":
                rec["weisskopf"] = weisskopf(t, K, A, B)
            if "-u" in flags and t in "EM":
                rec["Bu"] = standard_units(t, K, A, B)
            if "-ft" in flags:
                rec["logft"] = math.log(6145.0 / 1.27 / 1.27 / B) / math.log(10.0)
            tr.append(rec)
            if (abs(p["E"] - q["E"]) < 1e-5 and p["twoJ"] == q["twoJ"] and p["twoT"] == q["twoT"] and K < 3
                    and p["twoTz"] == q["twoTz"]):
                m = x / c * clebsch_gordan(q["twoJ"], q["twoJ"], 2 * K, 0, p["twoJ"], p["twoJ"]) \
                    * math.sqrt(4 * math.pi / (2 * K + 1)) * K
                mo.insert(0, {"m": m})
        trans.append(tr)
        moms.append(mo)
    return trans, moms


def occupations(z: np.ndarray, vecs: np.ndarray, ns: int) -> np.ndarray:
    """occ[k, s] = sum over the determinants holding s of psi_k^2."""
    vecs = np.asarray(vecs, dtype=np.float64).reshape(-1, len(z))
    occ = np.zeros((len(vecs), ns))
    p = vecs * vecs
    for col in range(z.shape[1]):
        for k in range(len(vecs)):
            occ[k] += np.bincount(z[:, col].astype(np.int64), weights=p[k], minlength=ns)
    return occ
