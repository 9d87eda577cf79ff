"""CPU ORACLE — test infrastructure only.

ctypes wrapper over oracle/_build/liboracle.so (cosmo_oracle.c,
oracle_davidson.c): a plain-C restatement of the reference algorithms used as
the parity reference in tests/ and smoke(), and as the timed CPU baseline in bench.py.
It is never imported by the product package.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle.so")
SRCS = ["cosmo_oracle.c", "oracle_davidson.c"]
REF_DIR = os.path.join(HERE, "_ref")


def build(force: bool = False) -> str:
    srcs = [os.path.join(HERE, s) for s in SRCS]
    if not force and os.path.exists(LIB) and all(os.path.getmtime(s) <= os.path.getmtime(LIB) for s in srcs):
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    tmp = LIB + ".tmp"
    cmd = ["gcc", "-O3", "-fopenmp", "-fPIC", "-shared", "-std=c11", "-o", tmp] + srcs + ["-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


def reference_root() -> str | None:
    """The reference checkout named by the COSMO_REFERENCE environment
    variable, or None when it is unset or does not hold the reference tree."""
    root = os.environ.get("COSMO_REFERENCE")
    if root and os.path.isdir(os.path.join(root, "include")):
        return root
    return None


def build_reference(ref_root: str | None = None) -> bool:
    """Compile the reference tools from the reference sources into oracle/_ref
    (only where the reference tree is given, by argument or COSMO_REFERENCE)."""
    ref_root = ref_root or reference_root()
    if not ref_root or not os.path.isdir(os.path.join(ref_root, "include")):
        return False
    subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={ref_root}"], check=True)
    return True


_lib = None
_P = C.c_void_p


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        L.oracle_basis.restype = C.c_uint64
        L.oracle_basis.argtypes = [C.c_int, _P, _P, _P, C.c_int, C.c_int, C.c_int, C.c_int, _P, C.c_uint64]
        L.oracle_build_upper.restype = C.c_int64
        L.oracle_build_upper.argtypes = [C.c_int, C.c_int64, _P, _P, C.c_int64, _P, _P, C.c_uint64, C.c_int, _P,
                                         _P, _P, _P, C.c_int]
        L.oracle_csb_from_upper.restype = _P
        L.oracle_csb_from_upper.argtypes = [C.c_uint64, _P, _P, _P]
        L.oracle_csb_free.argtypes = [_P]
        L.oracle_csb_times_matrix.argtypes = [_P, _P, _P, C.c_int, C.c_int]
        L.oracle_diagonal.argtypes = [C.c_uint64, _P, _P, _P, _P]
        L.oracle_davidson.restype = C.c_int
        L.oracle_davidson.argtypes = [_P, _P, C.c_uint64, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double,
                                      C.c_double, C.c_double, C.c_double, _P, _P, _P, _P, _P, _P, C.c_int,
                                      C.c_double, _P, _P, _P, _P]
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data if a is not None else None


def basis(sps: np.ndarray, N: int, twom: int, tz2: int, parity: int, cap: int | None = None) -> np.ndarray:
    """sps: rows (level n l 2j 2m 2t 2tz parity) as cosmo_gb300.Problem.sps()."""
    m2 = np.ascontiguousarray(sps[:, 4], dtype=np.int32)
    tz = np.ascontiguousarray(sps[:, 6], dtype=np.int32)
    pa = np.ascontiguousarray(sps[:, 7], dtype=np.int32)
    n = lib().oracle_basis(len(sps), _p(m2), _p(tz), _p(pa), N, twom, tz2, parity, None, 0)
    if cap is not None and n > cap:
        raise ValueError(f"basis of {n} states exceeds cap {cap}")
    z = np.zeros((n, N), dtype=np.uint16)
    lib().oracle_basis(len(sps), _p(m2), _p(tz), _p(pa), N, twom, tz2, parity, _p(z), n)
    return z


def basis_pruned(sps: np.ndarray, nv: int, zv: int, twom: int, parity: int,
                 hw: tuple[int, int] | None = None, rejections=()) -> np.ndarray:
    """The same truncated basis as basis_truncated, built without the
    untruncated one, so that it reaches spaces whose untruncated basis is out
    of reach (the spsdpf space: 20 neutrons in 40 m-states).

    XsysmbsOMP forms the occupation partitions of each species with quanta in
    [core, core + hwmax] before combining them (Partition::MakeQ,
    xmlshell/xmbs/PartitionClass.cxx:151-190); here each species' configurations
    are enumerated in lexicographic order by a depth-first search that leaves a
    branch once its quanta plus the least quanta the remaining particles can
    add exceed core + hwmax.  Neutron configurations in that order, each
    followed by the proton configurations that pass the determinant filters of
    basis_truncated (M, parity, hw window, rejections), is the order of the
    reference's sorted map (XsysmbsOMP.cpp:405-428)."""
    import sys as _sys
    sps = np.asarray(sps)
    neut = sps[:, 6] > 0
    q = (2 * sps[:, 1] + sps[:, 2]).astype(np.int64)
    m2 = sps[:, 4].astype(np.int64)
    par = sps[:, 7].astype(np.int64)
    nidx = np.where(neut)[0]
    pidx = np.where(~neut)[0]
    ncore = int(q[nidx][:nv].sum())
    pcore = int(q[pidx][:zv].sum())
    hwmin, hwmax = hw if hw is not None else (0, 0)

    def species(idx: np.ndarray, k: int, qlim: int | None) -> list[tuple[int, ...]]:
        qs = [int(x) for x in q[idx]]
        norb = len(qs)
        big = 1 << 40
        minsum = [[big] * (k + 1) for _ in range(norb + 1)]
        for i in range(norb + 1):
            rest = sorted(qs[i:])
            acc = 0
            minsum[i][0] = 0
            for r in range(1, min(k, len(rest)) + 1):
                acc += rest[r - 1]
                minsum[i][r] = acc
        out: list[tuple[int, ...]] = []
        cur: list[int] = []
        lim = big if qlim is None else qlim

        def go(start: int, left: int, Q: int) -> None:
            if left == 0:
                out.append(tuple(cur))
                return
            for c in range(start, norb - left + 1):
                Q2 = Q + qs[c]
                if Q2 + minsum[c + 1][left - 1] > lim:
                    continue
                cur.append(c)
                go(c + 1, left - 1, Q2)
                cur.pop()
        old = _sys.getrecursionlimit()
        _sys.setrecursionlimit(max(old, 4 * (k + 16)))
        try:
            if k <= norb:
                go(0, k, 0)
        finally:
            _sys.setrecursionlimit(old)
        return out

    nconf = species(nidx, nv, ncore + hwmax if hw is not None else None)
    pconf = species(pidx, zv, pcore + hwmax if hw is not None else None)
    P = np.array([[int(pidx[c]) for c in t] for t in pconf], dtype=np.int64).reshape(len(pconf), zv)
    pm = m2[P].sum(1) if zv else np.zeros(len(pconf), np.int64)
    pp = (par[P].sum(1) & 1) if zv else np.zeros(len(pconf), np.int64)
    pq = q[P].sum(1) - pcore if zv else np.zeros(len(pconf), np.int64)
    flags = [np.isin(sps[:, 0], levels) for _, _, levels in rejections]
    pc = [f[P].sum(1) if zv else np.zeros(len(pconf), np.int64) for f in flags]
    rows = []
    for t in nconf:
        Nn = np.array([int(nidx[c]) for c in t], dtype=np.int64)
        mn = int(m2[Nn].sum()) if nv else 0
        pn = int(par[Nn].sum() & 1) if nv else 0
        qn = int(q[Nn].sum()) - ncore if nv else -ncore
        keep = (pm == twom - mn) & (pp == (parity ^ pn))
        if hw is not None:
            if qn < 0 or qn > hwmax:
                continue
            keep &= (pq >= 0) & (pq <= hwmax) & (qn + pq >= hwmin) & (qn + pq <= hwmax)
        for (nmin, nmax, _), f, c in zip(rejections, flags, pc):
            cnt = int(f[Nn].sum()) + c
            keep &= (cnt >= nmin) & (cnt <= nmax)
        sel = P[keep]
        if len(sel):
            rows.append(np.hstack([np.broadcast_to(Nn, (len(sel), nv)), sel]))
    if not rows:
        return np.zeros((0, nv + zv), dtype=np.uint16)
    return np.vstack(rows).astype(np.uint16)


def basis_truncated(sps: np.ndarray, nv: int, zv: int, twom: int, parity: int,
                    hw: tuple[int, int] | None = None, rejections=()) -> np.ndarray:
    """The reference's truncated bases as a filter of the untruncated one.

    XsysmbsOMP (xmlshell/xmbs/XsysmbsOMP.cpp:214-300) builds occupation
    partitions per orbital level (neutron levels, then proton levels, :99-117),
    drops partitions, and writes the surviving determinants in the order of the
    untruncated basis (a sorted map, :405-428), so a filter of `basis` in order
    restates it:
    * hw (hwmin, hwmax): with Q = sum of 2n + l over occupied states, neutron
      partitions with Qn in [Ncore, Ncore + hwmax] and proton ones with Qp in
      [Pcore, Pcore + hwmax] (Partition::MakeQ, PartitionClass.cxx:151-190),
      then Qn + Qp in [Ncore + Pcore + hwmin, Ncore + Pcore + hwmax]
      (QuantaMinMaxPurge, :390-413).  Ncore (Pcore) is CoreQuanta
      (include/sm/SingleParticleStates.cxx:155-168): the quanta of the first
      nv neutron (zv proton) s.p. states in list order, since its sort covers
      an empty range.
    * rejections [(nmin, nmax, levels)]: the particles of both species in the
      listed 0-based orbital levels (type "pn") number nmin..nmax
      (TestRestriction, PartitionClass.cxx:23-40).
    sps: rows (level n l 2j 2m 2t 2tz parity) as cosmo_gb300.Problem.sps()."""
    sps = np.asarray(sps)
    z = basis(sps, nv + zv, twom, nv - zv, parity)
    keep = np.ones(len(z), dtype=bool)
    neut = sps[:, 6] > 0
    if hw is not None:
        hwmin, hwmax = hw
        q = 2 * sps[:, 1] + sps[:, 2]
        ncore = int(q[neut][:nv].sum())
        pcore = int(q[~neut][:zv].sum())
        qz = q[z.astype(np.int64)]
        nz = neut[z.astype(np.int64)]
        qn = np.where(nz, qz, 0).sum(1)
        qp = np.where(nz, 0, qz).sum(1)
        keep &= (qn >= ncore) & (qn <= ncore + hwmax) & (qp >= pcore) & (qp <= pcore + hwmax)
        keep &= (qn + qp >= ncore + pcore + hwmin) & (qn + qp <= ncore + pcore + hwmax)
    for nmin, nmax, levels in rejections:
        flag = np.isin(sps[:, 0], levels)
        cnt = flag[z.astype(np.int64)].sum(1)
        keep &= (cnt >= nmin) & (cnt <= nmax)
    return z[keep]


def build_upper(ns: int, k1, v1, k2, v2, z: np.ndarray, nthreads: int = 0):
    """Upper-triangle rows (CSR) of H from forward-ordered operator terms."""
    k1 = np.ascontiguousarray(k1, dtype=np.int32)
    v1 = np.ascontiguousarray(v1, dtype=np.float64)
    k2 = np.ascontiguousarray(k2, dtype=np.int32)
    v2 = np.ascontiguousarray(v2, dtype=np.float64)
    z = np.ascontiguousarray(z, dtype=np.uint16)
    n, N = z.shape
    rp = np.zeros(n + 1, dtype=np.uint64)
    r = lib().oracle_build_upper(ns, len(v1), _p(k1), _p(v1), len(v2), _p(k2), _p(v2), n, N, _p(z), _p(rp), None,
                                 None, nthreads)
    if r < 0:
        raise RuntimeError("oracle row buffer overflow")
    cols = np.zeros(int(rp[-1]), dtype=np.uint32)
    vals = np.zeros(int(rp[-1]))
    lib().oracle_build_upper(ns, len(v1), _p(k1), _p(v1), len(v2), _p(k2), _p(v2), n, N, _p(z), _p(rp), _p(cols),
                             _p(vals), nthreads)
    return rp, cols, vals


class CSB:
    """Reference-layout upper CSB (square blocks of floor(sqrt(n)) + 1)."""

    def __init__(self, rp, cols, vals):
        self.rp = np.ascontiguousarray(rp, dtype=np.uint64)
        self.cols = np.ascontiguousarray(cols, dtype=np.uint32)
        self.vals = np.ascontiguousarray(vals, dtype=np.float64)
        self.n = len(self.rp) - 1
        self._h = lib().oracle_csb_from_upper(self.n, _p(self.rp), _p(self.cols), _p(self.vals))

    def __del__(self):
        if getattr(self, "_h", None):
            lib().oracle_csb_free(self._h)
            self._h = None

    def times_matrix(self, x: np.ndarray, nthreads: int = 0) -> np.ndarray:
        x2 = np.asarray(x, dtype=np.float64).reshape(self.n, -1)
        m = x2.shape[1]
        xc = np.ascontiguousarray(x2.T)
        yc = np.zeros_like(xc)
        lib().oracle_csb_times_matrix(self._h, _p(xc), _p(yc), m, nthreads)
        return yc.T.reshape(np.shape(x))

    def diagonal(self) -> np.ndarray:
        d = np.zeros(self.n)
        lib().oracle_diagonal(self.n, _p(self.rp), _p(self.cols), _p(self.vals), _p(d))
        return d

    def davidson(self, nume: int = 10, block: int | None = None, lim: int | None = None, maxiter: int = 0,
                 crite=1e-15, critc=1e-12, critr=1e-8, ortho=1e-9, nthreads: int = 0, time_budget: float = 0.0,
                 want_vectors: bool = False):
        """dvdrvr2 restated.  Besides the eigenpairs, returns the end time of
        every iteration (iter_end, seconds from the start of the first) and the
        number of basis collapses."""
        block = block or nume
        lim = lim or nume + 20
        maxiter = maxiter or max(40 * nume, 200)
        d = self.diagonal()
        eig = np.zeros(nume); de = np.zeros(nume); res = np.zeros(nume)
        vecs = np.zeros((nume, self.n)) if want_vectors else None
        ends = np.zeros(maxiter)
        it = C.c_int(0); nmv = C.c_int64(0); per = C.c_double(0); t0 = C.c_double(0); ncol = C.c_int(0)
        ierr = lib().oracle_davidson(self._h, _p(d), self.n, nume, block, lim, maxiter, crite, critc, critr, ortho,
                                     _p(eig), _p(de), _p(res), _p(vecs), C.byref(it), C.byref(nmv), nthreads,
                                     time_budget, C.byref(per), C.byref(t0), _p(ends), C.byref(ncol))
        return dict(eig=eig, de=de, resid=res, vecs=vecs, iterations=it.value, matvecs=nmv.value, ierr=ierr,
                    seconds_per_iteration=per.value, iter_end=ends[:it.value].copy(), collapses=ncol.value)


def full_from_upper(rp, cols, vals):
    """scipy CSR of the full symmetric matrix from upper rows."""
    import scipy.sparse as sp
    n = len(rp) - 1
    rows = np.repeat(np.arange(n), np.diff(rp).astype(np.int64))
    U = sp.csr_matrix((vals, (rows, cols.astype(np.int64))), shape=(n, n))
    D = sp.diags(U.diagonal())
    return (U + U.T - D).tocsr()


def annihilation_amplitudes(zp: np.ndarray, vp: np.ndarray, zd: np.ndarray, vd: np.ndarray, ns: int) -> np.ndarray:
    """amp[q, p, s] = <D_q| a_s |P_p> for every s.p. state s: the overlap the
    reference's XSHLSF takes with PPMatrix::OverlapNH and the one-body
    operator a_s (xmlshell/XSHLSF.cpp:150-175, include/sm/PPMatrix.cxx:
    275-302).  zp, zd: parent and daughter bases (sorted tuples), vp, vd:
    their vectors (states x dimension).  For each daughter determinant D and
    each s outside it, P = D + s; SM::Annihilation removes s from P with the
    phase of the number of states of P below s (include/sm/operators.cxx:
    121-150)."""
    index = {tuple(int(x) for x in t): i for i, t in enumerate(zp)}
    vp = np.asarray(vp, dtype=np.float64).reshape(-1, len(zp))
    vd = np.asarray(vd, dtype=np.float64).reshape(-1, len(zd))
    amp = np.zeros((len(vd), len(vp), ns))
    for di, D in enumerate(zd):
        d = tuple(int(x) for x in D)
        for s in range(ns):
            if s in d:
                continue
            P = tuple(sorted(d + (s,)))
            i = index.get(P)
            if i is None:
                continue
            sign = -1.0 if P.index(s) & 1 else 1.0
            amp[:, :, s] += sign * np.outer(vd[:, di], vp[:, i])
    return amp
