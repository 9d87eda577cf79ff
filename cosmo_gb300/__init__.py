"""cosmo_gb300: GB300 (sm_103a) configuration-interaction hot path of CoSMo.

Python view of the C ABI in ``include/cosmo_gb300.h`` (ctypes over the in-tree
``libcosmo_gb300.so``).  The names follow the reference's objects:

* :class:`Problem`          system XML + s.p. states + ESP/VSPX operator terms
                            (``SM::Make``, ``xReadSPInt``)
* :class:`ManyBodyStates`   the M-scheme basis (``SM::Many_Body_States``,
                            ``MakeMBS2``/``Xsysmbs``, ``SM::locate``)
* :class:`Hamiltonian`      the stored H + lambda J-J+ (``PPMatrix2CSBBlk`` /
                            ``SparseMatrixCSB``, ``TimesMatrix``, ``ReadDiagonal``)
* :func:`davidson_diagonalization`  ``DavidsonDiagonalization``

Every failure raises :class:`CosmoError` carrying the C status code.  There is
no CPU fallback: without the built library or a CUDA device the calls fail.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libcosmo_gb300.so")

CG_OK = 0
CG_ERR_ARG = -1
CG_PREC_FP64, CG_PREC_FP32, CG_PREC_REFINE = 0, 1, 2
CG_FORMAT_ROWS, CG_FORMAT_TILED = 0, 1
STATUS_NAMES = {0: "CG_OK", -1: "CG_ERR_ARG", -2: "CG_ERR_IO", -3: "CG_ERR_PARSE", -4: "CG_ERR_CUDA",
                -5: "CG_ERR_NOMEM", -6: "CG_ERR_UNSUPPORTED", -7: "CG_ERR_NOT_CONVERGED",
                -8: "CG_ERR_TIMEOUT", -9: "CG_ERR_NO_DEVICE", -10: "CG_ERR_INTERNAL"}


class CosmoError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


class SpmmFormatInfo(C.Structure):
    _fields_ = [("format", C.c_int32), ("tiled_available", C.c_int32), ("warps", C.c_int32),
                ("stages", C.c_int32), ("slices_per_warp", C.c_int32), ("reserved", C.c_int32),
                ("entries", C.c_uint64), ("units", C.c_uint64),
                ("meta_bytes", C.c_uint64), ("device_bytes", C.c_uint64), ("ident_tiles", C.c_uint64),
                ("ident_entries", C.c_uint64)]


class ProblemInfo(C.Structure):
    _fields_ = [("n_sps", C.c_int32), ("n_neutron_sps", C.c_int32), ("nv", C.c_int32), ("zv", C.c_int32),
                ("twom", C.c_int32), ("parity", C.c_int32), ("has_jj", C.c_int32), ("jj", C.c_double),
                ("n_one_body", C.c_int64), ("n_two_body", C.c_int64)]


class ProblemDesc(C.Structure):
    _fields_ = [("n_sps", C.c_int32), ("n_neutron_sps", C.c_int32), ("sps", C.c_void_p), ("nv", C.c_int32),
                ("zv", C.c_int32), ("twom", C.c_int32), ("parity", C.c_int32), ("n_one_body", C.c_int64),
                ("one_keys", C.c_void_p), ("one_vals", C.c_void_p), ("n_two_body", C.c_int64),
                ("two_keys", C.c_void_p), ("two_vals", C.c_void_p)]


class HamiltonianInfo(C.Structure):
    _fields_ = [("n", C.c_uint64), ("nnz_full", C.c_uint64), ("nnz_upper", C.c_uint64), ("precision", C.c_int32),
                ("max_row", C.c_int32), ("device_bytes", C.c_uint64), ("build_seconds", C.c_double)]


class DavidsonParams(C.Structure):
    _fields_ = [("nstates", C.c_int32), ("block", C.c_int32), ("lim", C.c_int32), ("maxiter", C.c_int32),
                ("crite", C.c_double), ("critc", C.c_double), ("critr", C.c_double), ("ortho", C.c_double),
                ("tol_resid", C.c_double), ("switch_resid", C.c_double), ("precision", C.c_int32),
                ("verbose", C.c_int32), ("ortho_block", C.c_int32), ("algorithm", C.c_int32),
                ("keep", C.c_int32), ("precond", C.c_int32), ("refine_lim", C.c_int32),
                ("refine_keep", C.c_int32), ("ortho_pip", C.c_int32), ("refine_block", C.c_int32),
                ("refine_fp32_corrections", C.c_int32)]


class BatchParams(C.Structure):
    _fields_ = [("nstates", C.c_int32), ("block", C.c_int32), ("lim", C.c_int32), ("keep", C.c_int32),
                ("maxiter", C.c_int32), ("tol_resid", C.c_double), ("switch_resid", C.c_double),
                ("use_graph", C.c_int32)]


class BatchStats(C.Structure):
    _fields_ = [("iterations_fp32", C.c_int32), ("iterations_fp64", C.c_int32), ("graph_launches", C.c_uint64),
                ("graph_kernels", C.c_int32), ("launches", C.c_uint64), ("seconds", C.c_double),
                ("build_seconds", C.c_double), ("spmm_warps", C.c_int32), ("spmm_ctas_per_sm", C.c_int32),
                ("spmm_tune_seconds", C.c_double)]


class DavidsonStats(C.Structure):
    _fields_ = [("iterations", C.c_int32), ("refine_iterations", C.c_int32), ("matvecs", C.c_int64),
                ("restarts", C.c_int32), ("converged", C.c_int32), ("ierr", C.c_int32), ("seconds", C.c_double),
                ("spmm_seconds", C.c_double)]


# every symbol the header declares, with its ctypes signature
_P = C.c_void_p
_SIGS = {
    "cg_last_error": (C.c_char_p, []),
    "cg_version": (C.c_int32, []),
    "cg_device_count": (C.c_int32, []),
    "cg_launch_count": (C.c_uint64, []),
    "cg_problem_load_xml": (C.c_int32, [C.c_char_p, C.c_char_p, C.POINTER(_P)]),
    "cg_problem_create": (C.c_int32, [C.POINTER(ProblemDesc), C.POINTER(_P)]),
    "cg_problem_destroy": (None, [_P]),
    "cg_problem_get_info": (C.c_int32, [_P, C.POINTER(ProblemInfo)]),
    "cg_problem_sps": (C.c_int32, [_P, _P]),
    "cg_problem_one_body": (C.c_int32, [_P, _P, _P]),
    "cg_problem_two_body": (C.c_int32, [_P, _P, _P]),
    "cg_basis_build": (C.c_int32, [_P, C.POINTER(_P)]),
    "cg_basis_build_wide": (C.c_int32, [_P, C.POINTER(_P)]),
    "cg_basis_is_wide": (C.c_int32, [_P, C.POINTER(C.c_int32)]),
    "cg_basis_destroy": (None, [_P]),
    "cg_basis_dims": (C.c_int32, [_P, C.POINTER(C.c_uint64), C.POINTER(C.c_int32)]),
    "cg_basis_states": (C.c_int32, [_P, C.c_uint64, C.c_uint64, _P]),
    "cg_basis_locate": (C.c_int32, [_P, _P, C.c_uint64, _P]),
    "cg_basis_write_mbs": (C.c_int32, [_P, C.c_char_p]),
    "cg_hamiltonian_build": (C.c_int32, [_P, _P, C.c_int32, C.POINTER(_P)]),
    "cg_hamiltonian_destroy": (None, [_P]),
    "cg_hamiltonian_get_info": (C.c_int32, [_P, C.POINTER(HamiltonianInfo)]),
    "cg_hamiltonian_diagonal": (C.c_int32, [_P, _P]),
    "cg_hamiltonian_upper_rows": (C.c_int32, [_P, C.c_uint64, C.c_uint64, _P, _P, _P]),
    "cg_hamiltonian_write_hh": (C.c_int32, [_P, C.c_char_p]),
    "cg_hamiltonian_stream": (_P, [_P]),
    "cg_spmm": (C.c_int32, [_P, _P, _P, C.c_int32, C.c_int32]),
    "cg_spmm_device": (C.c_int32, [_P, _P, C.c_int32, _P, C.c_int32, C.c_int32, C.c_int32]),
    "cg_spmm_autotune": (C.c_int32, [_P, C.c_int32, C.c_int32, C.POINTER(C.c_int32), _P, _P, _P]),
    "cg_spmm_set_tuning": (C.c_int32, [_P, C.c_int32, C.c_int32]),
    "cg_spmm_refine_static": (C.c_int32, [_P, _P, C.c_int32, _P, C.c_int32, C.c_int32]),
    "cg_spmm_refine_static_max_rows": (C.c_int32, [C.POINTER(C.c_uint64)]),
    "cg_hamiltonian_build_virtual": (C.c_int32, [_P, _P, C.c_int32, C.POINTER(_P)]),
    "cg_hamiltonian_read_hh": (C.c_int32, [C.c_char_p, C.c_int32, C.POINTER(_P)]),
    "cg_hamiltonian_is_virtual": (C.c_int32, [_P, C.POINTER(C.c_int32)]),
    "cg_batch_create": (C.c_int32, [C.POINTER(_P), C.c_int32, C.POINTER(_P)]),
    "cg_batch_destroy": (None, [_P]),
    "cg_batch_defaults": (C.c_int32, [C.POINTER(BatchParams)]),
    "cg_batch_dims": (C.c_int32, [_P, _P]),
    "cg_batch_solve": (C.c_int32, [_P, C.POINTER(BatchParams), _P, _P, _P, C.POINTER(BatchStats)]),
    "cg_jt_expectations": (C.c_int32, [_P, _P, C.c_int32, _P, _P]),
    "cg_jj_spin": (C.c_int32, [C.c_double, C.c_int32]),
    "cg_sf_amplitudes": (C.c_int32, [_P, _P, C.c_int32, _P, _P, C.c_int32, _P]),
    "cg_xshlsf": (C.c_int32, [C.c_char_p, C.c_char_p, C.c_char_p, C.c_char_p, C.c_char_p, C.c_int32]),
    "cg_xshljt": (C.c_int32, [C.c_char_p, C.c_char_p, C.c_char_p, C.c_int32, C.c_char_p, C.POINTER(C.c_int32)]),
    "cg_dense_eigensolve": (C.c_int32, [_P, _P, _P]),
    "cg_occupations": (C.c_int32, [_P, _P, C.c_int32, _P]),
    "cg_xshlao": (C.c_int32, [C.c_char_p, C.c_char_p, C.c_char_p]),
    "cg_xlevels": (C.c_int32, [C.POINTER(C.c_char_p), C.c_int32, C.c_char_p]),
    "cg_transition_terms": (C.c_int32, [C.c_char_p, C.c_char_p, C.c_char_p, C.c_int32, C.c_int32, _P, _P, _P,
                                        C.c_int32, C.POINTER(C.c_int32)]),
    "cg_onebody_amplitudes": (C.c_int32, [_P, _P, C.c_int32, _P, _P, C.c_int32, _P, _P, _P, C.c_int32, _P]),
    "cg_xshlemb": (C.c_int32, [C.c_char_p, C.c_char_p, C.c_char_p, C.c_char_p, C.c_char_p, C.c_int32,
                               C.c_char_p]),
    "cg_gather_ceiling": (C.c_int32, [C.c_uint64, C.c_int32, C.POINTER(C.c_double)]),
    "cg_spmm_get_tuning": (C.c_int32, [_P, C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    "cg_spmm_set_format": (C.c_int32, [_P, C.c_int32]),
    "cg_spmm_get_format": (C.c_int32, [_P, _P]),
    "cg_spmm_set_tiled_shape": (C.c_int32, [_P, C.c_int32, C.c_int32]),
    "cg_davidson_defaults": (None, [C.POINTER(DavidsonParams), C.c_int32]),
    "cg_davidson": (C.c_int32, [_P, C.POINTER(DavidsonParams), _P, C.c_int32, _P, _P, _P, _P,
                                C.POINTER(DavidsonStats)]),
    "cg_write_ee": (C.c_int32, [C.c_char_p, C.c_int32, C.c_uint64, _P, _P, _P, _P]),
}

_lib = None


def lib() -> C.CDLL:
    """Load the in-tree library (fails loudly when it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise CosmoError(-10, f"{LIB_PATH} is missing: run `python -m cosmo_gb300.build`")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _check(status: int) -> None:
    if status != CG_OK:
        raise CosmoError(status, lib().cg_last_error().decode(errors="replace"))


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


def device_count() -> int:
    return int(lib().cg_device_count())


def gather_ceiling(rows: int, share: int = 1) -> float:
    """Random 32-byte gathers per second from a table of `rows` rows (device probe)."""
    g = C.c_double()
    _check(lib().cg_gather_ceiling(rows, share, C.byref(g)))
    return float(g.value)


class Batch:
    """Many independent problems solved together on the GPU (lockstep block
    Davidson under CUDA graphs; exact batched Jacobi for dimensions <= 64)."""

    def __init__(self, problems: list):
        arr = (_P * len(problems))(*[p._h for p in problems])
        h = _P()
        _check(lib().cg_batch_create(arr, len(problems), C.byref(h)))
        self._h = h
        self.count = len(problems)
        self._problems = problems

    def __del__(self):
        if getattr(self, "_h", None):
            lib().cg_batch_destroy(self._h)
            self._h = None

    def dims(self) -> np.ndarray:
        d = np.zeros(self.count, dtype=np.uint64)
        _check(lib().cg_batch_dims(self._h, _ptr(d)))
        return d

    def solve(self, nstates: int = 5, **kw):
        p = BatchParams()
        _check(lib().cg_batch_defaults(C.byref(p)))
        p.nstates = nstates
        p.block = max(p.block, nstates)
        for k, v in kw.items():
            if not hasattr(p, k):
                raise TypeError(f"unknown batch parameter {k}")
            setattr(p, k, v)
        eig = np.zeros((self.count, nstates))
        res = np.zeros((self.count, nstates))
        nconv = np.zeros(self.count, dtype=np.int32)
        st = BatchStats()
        _check(lib().cg_batch_solve(self._h, C.byref(p), _ptr(eig), _ptr(res), _ptr(nconv), C.byref(st)))
        return eig, res, nconv, st


def jt_expectations(basis: "ManyBodyStates", vecs) -> tuple[np.ndarray, np.ndarray]:
    """<J-J+> and <T-T+> of the rows of vecs (nstates x n), computed on the GPU
    (XSHLJT, include/xsm/XSHLJT.cxx:94-126)."""
    v = np.ascontiguousarray(np.asarray(vecs, dtype=np.float64).reshape(-1, basis.n))
    k = v.shape[0]
    jj = np.zeros(k)
    tt = np.zeros(k)
    _check(lib().cg_jt_expectations(basis._h, _ptr(v), k, _ptr(jj), _ptr(tt)))
    return jj, tt


def sf_amplitudes(parent: "ManyBodyStates", vp, daughter: "ManyBodyStates", vd) -> np.ndarray:
    """amp[q, p, s] = <D_q| a_s |P_p> for one-particle removal from the parent
    states (rows of vp) to the daughter states (rows of vd, at most 16),
    computed on the GPU (the overlaps of XSHLSF, xmlshell/XSHLSF.cpp:150-175)."""
    vp = np.ascontiguousarray(np.asarray(vp, dtype=np.float64).reshape(-1, parent.n))
    vd = np.ascontiguousarray(np.asarray(vd, dtype=np.float64).reshape(-1, daughter.n))
    amp = np.zeros((vd.shape[0], vp.shape[0], parent.n_sps))
    _check(lib().cg_sf_amplitudes(parent._h, _ptr(vp), vp.shape[0], daughter._h, _ptr(vd), vd.shape[0], _ptr(amp)))
    return amp


def xshlsf(parent_xml: str, out: str | None = None, daughter_xml: str | None = None, parent_system: str | None = None,
           daughter_system: str | None = None, full: bool = False) -> None:
    """The XSHLSF tool: spectroscopic factors between the parent's and the
    daughter's <state>s, table written to `out` (xmlshell/XSHLSF.cpp)."""
    enc = lambda x: x.encode() if x is not None else None  # noqa: E731
    _check(lib().cg_xshlsf(enc(parent_xml), enc(parent_system), enc(daughter_xml), enc(daughter_system), enc(out),
                           int(full)))


CG_EMB_WEISSKOPF, CG_EMB_UNITS, CG_EMB_LOGFT, CG_EMB_PHASE_INFINITY = 1, 2, 4, 8


def transition_terms(xml: str, system: str | None = None, operator: str | None = None, kappa: int = 0,
                     phase_infinity: bool = False) -> list:
    """[(i, f, v)]: the m-scheme terms v a+_f a_i of the <operator> node of an
    XML file (XSHLEMB's operators, include/sm/EMspherical2sp.cxx) for the
    projection kappa, on the system's s.p. states.  Host computation."""
    enc = lambda x: x.encode() if x is not None else None  # noqa: E731
    flags = CG_EMB_PHASE_INFINITY if phase_infinity else 0
    n = C.c_int32()
    _check(lib().cg_transition_terms(enc(xml), enc(system), enc(operator), kappa, flags, None, None, None, 0,
                                     C.byref(n)))
    i = np.zeros(max(n.value, 1), np.int32)
    f = np.zeros(max(n.value, 1), np.int32)
    v = np.zeros(max(n.value, 1), np.float64)
    _check(lib().cg_transition_terms(enc(xml), enc(system), enc(operator), kappa, flags, _ptr(i), _ptr(f), _ptr(v),
                                     n.value, C.byref(n)))
    return [(int(i[k]), int(f[k]), float(v[k])) for k in range(n.value)]


def onebody_amplitudes(parent: "ManyBodyStates", vp, daughter: "ManyBodyStates", vd, terms) -> np.ndarray:
    """amp[q, p] = <D_q| sum v a+_f a_i |P_p> for the (i, f, v) terms, parent
    states the rows of vp, daughter states the rows of vd (at most 16), on the
    GPU (the overlaps of XSHLEMB, PPMatrix::OverlapNH)."""
    vp = np.ascontiguousarray(np.asarray(vp, dtype=np.float64).reshape(-1, parent.n))
    vd = np.ascontiguousarray(np.asarray(vd, dtype=np.float64).reshape(-1, daughter.n))
    ti = np.ascontiguousarray([t[0] for t in terms] or [0], dtype=np.int32)
    tf = np.ascontiguousarray([t[1] for t in terms] or [0], dtype=np.int32)
    tv = np.ascontiguousarray([t[2] for t in terms] or [0.0], dtype=np.float64)
    amp = np.zeros((vd.shape[0], vp.shape[0]))
    _check(lib().cg_onebody_amplitudes(parent._h, _ptr(vp), vp.shape[0], daughter._h, _ptr(vd), vd.shape[0],
                                       _ptr(ti), _ptr(tf), _ptr(tv), len(terms), _ptr(amp)))
    return amp


def xshlemb(parent_xml: str, out: str | None = None, daughter_xml: str | None = None,
            parent_system: str | None = None, daughter_system: str | None = None, operator: str | None = None,
            weisskopf: bool = False, units: bool = False, logft: bool = False,
            phase_infinity: bool = False) -> None:
    """The XSHLEMB tool: B values of the parent XML's <operator> between the
    parent's and the daughter's <state>s, written as <transition>/<moment>
    children of the parent's states into `out` (the parent XML when None)."""
    enc = lambda x: x.encode() if x is not None else None  # noqa: E731
    flags = ((CG_EMB_WEISSKOPF if weisskopf else 0) | (CG_EMB_UNITS if units else 0) | (CG_EMB_LOGFT if logft else 0)
             | (CG_EMB_PHASE_INFINITY if phase_infinity else 0))
    _check(lib().cg_xshlemb(enc(parent_xml), enc(parent_system), enc(daughter_xml), enc(daughter_system), enc(out),
                            flags, enc(operator)))


def occupations(basis: "ManyBodyStates", vecs) -> np.ndarray:
    """occ[k, s] = <psi_k| n_s |psi_k> for the rows of vecs (XSHLAO's
    SM::occupation), on the GPU."""
    v = np.ascontiguousarray(np.asarray(vecs, dtype=np.float64).reshape(-1, basis.n))
    occ = np.zeros((v.shape[0], basis.n_sps))
    _check(lib().cg_occupations(basis._h, _ptr(v), v.shape[0], _ptr(occ)))
    return occ


def xshlao(xml: str, out: str | None = None, system: str | None = None) -> None:
    """The XSHLAO tool: orbital occupation numbers of the system's <state>s
    as <occupation> nodes, into `out` (the input XML when None)."""
    enc = lambda x: x.encode() if x is not None else None  # noqa: E731
    _check(lib().cg_xshlao(enc(xml), enc(system), enc(out)))


def xlevels(files, out: str | None = None) -> None:
    """The Xlevels tool: the levels of the <state>s of the XML files organized
    together and listed on stdout (host only)."""
    arr = (C.c_char_p * len(files))(*[f.encode() for f in files])
    _check(lib().cg_xlevels(arr, len(files), out.encode() if out else None))


def jj_spin(x: float, two_m: int) -> int:
    """2J from <J-J+> and 2M (SM::JJSpin); -1 if not a valid spin."""
    return int(lib().cg_jj_spin(float(x), int(two_m)))


def xshljt(xml: str, ee: str, nstates: int = 0, out: str | None = None, system: str | None = None) -> int:
    """Spin/isospin analysis of an .EE file into <state> nodes of the system XML
    (XSHLJT); returns the number of states recorded."""
    k = C.c_int32()
    _check(lib().cg_xshljt(xml.encode(), system.encode() if system else None, ee.encode(), nstates,
                           out.encode() if out else None, C.byref(k)))
    return int(k.value)


def launch_count() -> int:
    """Kernel launches issued by the library so far in this process."""
    return int(lib().cg_launch_count())


def _device_name() -> str:
    try:
        import subprocess
        out = subprocess.run(["nvidia-smi", "--query-gpu=name", "--format=csv,noheader", "-i", "0"],
                             capture_output=True, text=True, timeout=10).stdout.strip()
        return out or "cuda"
    except Exception:
        return "cuda"


class Problem:
    """System XML -> s.p. table and forward-ordered m-scheme operator terms."""

    def __init__(self, xml_path: str | None = None, system: str | None = None, _handle=None):
        if _handle is None:
            h = _P()
            _check(lib().cg_problem_load_xml(xml_path.encode(), system.encode() if system else None, C.byref(h)))
        else:
            h = _handle
        self._h = h
        inf = ProblemInfo()
        _check(lib().cg_problem_get_info(h, C.byref(inf)))
        self.info = inf

    @classmethod
    def from_terms(cls, sps: np.ndarray, n_neutron_sps: int, nv: int, zv: int, twom: int, parity: int,
                   one_keys, one_vals, two_keys, two_vals) -> "Problem":
        """Problem from an explicit s.p. table and forward-ordered operator terms."""
        keep = [np.ascontiguousarray(sps, dtype=np.int32), np.ascontiguousarray(one_keys, dtype=np.int32),
                np.ascontiguousarray(one_vals, dtype=np.float64), np.ascontiguousarray(two_keys, dtype=np.int32),
                np.ascontiguousarray(two_vals, dtype=np.float64)]
        d = ProblemDesc(len(keep[0]), n_neutron_sps, _ptr(keep[0]), nv, zv, twom, parity, len(keep[2]),
                        _ptr(keep[1]), _ptr(keep[2]), len(keep[4]), _ptr(keep[3]), _ptr(keep[4]))
        h = _P()
        _check(lib().cg_problem_create(C.byref(d), C.byref(h)))
        return cls(_handle=h)

    def __del__(self):
        if getattr(self, "_h", None):
            lib().cg_problem_destroy(self._h)
            self._h = None

    def sps(self) -> np.ndarray:
        t = np.zeros((self.info.n_sps, 8), dtype=np.int32)
        _check(lib().cg_problem_sps(self._h, _ptr(t)))
        return t

    def one_body(self) -> tuple[np.ndarray, np.ndarray]:
        k = np.zeros((self.info.n_one_body, 2), dtype=np.int32)
        v = np.zeros(self.info.n_one_body)
        _check(lib().cg_problem_one_body(self._h, _ptr(k), _ptr(v)))
        return k, v

    def two_body(self) -> tuple[np.ndarray, np.ndarray]:
        k = np.zeros((self.info.n_two_body, 4), dtype=np.int32)
        v = np.zeros(self.info.n_two_body)
        _check(lib().cg_problem_two_body(self._h, _ptr(k), _ptr(v)))
        return k, v


class ManyBodyStates:
    """GPU-resident M-scheme basis in the reference's lexicographic order.
    wide=True builds the wide representation (64-bit species masks, binary
    search locate) even where the bitstring one applies."""

    def __init__(self, problem: Problem, wide: bool = False):
        h = _P()
        _check((lib().cg_basis_build_wide if wide else lib().cg_basis_build)(problem._h, C.byref(h)))
        self._h = h
        w = C.c_int32()
        _check(lib().cg_basis_is_wide(h, C.byref(w)))
        self.wide = bool(w.value)
        n = C.c_uint64()
        N = C.c_int32()
        _check(lib().cg_basis_dims(h, C.byref(n), C.byref(N)))
        self.n = int(n.value)
        self.N = int(N.value)
        self.n_sps = int(problem.info.n_sps)

    def __del__(self):
        if getattr(self, "_h", None):
            lib().cg_basis_destroy(self._h)
            self._h = None

    def states(self, first: int = 0, count: int | None = None) -> np.ndarray:
        count = self.n - first if count is None else count
        z = np.zeros((count, self.N), dtype=np.uint16)
        _check(lib().cg_basis_states(self._h, first, count, _ptr(z)))
        return z

    def locate(self, tuples: np.ndarray) -> np.ndarray:
        t = np.ascontiguousarray(tuples, dtype=np.uint16).reshape(-1, self.N)
        out = np.zeros(len(t), dtype=np.uint64)
        _check(lib().cg_basis_locate(self._h, _ptr(t), len(t), _ptr(out)))
        return out

    def write_mbs(self, path: str) -> None:
        _check(lib().cg_basis_write_mbs(self._h, path.encode()))


class Hamiltonian:
    """H + lambda J-J+ on the GPU: stored (both triangles, row-sliced), or with
    ``virtual=True`` regenerated on the fly by every product (SM::PPMatrix)."""

    def __init__(self, problem: Problem, basis: ManyBodyStates, precision: int = CG_PREC_FP64,
                 virtual: bool = False):
        h = _P()
        build = lib().cg_hamiltonian_build_virtual if virtual else lib().cg_hamiltonian_build
        _check(build(problem._h, basis._h, precision, C.byref(h)))
        self._h = h
        self.virtual = bool(virtual)
        self.refresh_info()

    @classmethod
    def from_hh(cls, path: str, precision: int = CG_PREC_FP64) -> "Hamiltonian":
        """Stored H read from a .HH file (the davidson_vfile input)."""
        self = cls.__new__(cls)
        h = _P()
        _check(lib().cg_hamiltonian_read_hh(path.encode(), precision, C.byref(h)))
        self._h = h
        self.virtual = False
        self.refresh_info()
        return self

    def refresh_info(self):
        inf = HamiltonianInfo()
        _check(lib().cg_hamiltonian_get_info(self._h, C.byref(inf)))
        self.info = inf
        self.n = int(inf.n)
        self.precision = int(inf.precision)

    def __del__(self):
        if getattr(self, "_h", None):
            lib().cg_hamiltonian_destroy(self._h)
            self._h = None

    @property
    def stream(self) -> int:
        return int(lib().cg_hamiltonian_stream(self._h) or 0)

    def diagonal(self) -> np.ndarray:
        d = np.zeros(self.n)
        _check(lib().cg_hamiltonian_diagonal(self._h, _ptr(d)))
        return d

    def dense_eigensolve(self, want_vectors: bool = True):
        """Every eigenpair of the stored matrix by exact FP64 diagonalization
        (the reference DXHV's path for small dimensions): (eig, vecs[n, n])."""
        eig = np.zeros(max(self.n, 1))
        vecs = np.zeros((self.n, self.n)) if want_vectors else None
        _check(lib().cg_dense_eigensolve(self._h, _ptr(eig), _ptr(vecs) if want_vectors else None))
        return eig[:self.n], vecs

    def upper_rows(self, row0: int = 0, nrows: int | None = None):
        nrows = self.n - row0 if nrows is None else nrows
        rp = np.zeros(nrows + 1, dtype=np.uint64)
        _check(lib().cg_hamiltonian_upper_rows(self._h, row0, nrows, _ptr(rp), None, None))
        cols = np.zeros(int(rp[-1]), dtype=np.uint32)
        vals = np.zeros(int(rp[-1]))
        _check(lib().cg_hamiltonian_upper_rows(self._h, row0, nrows, _ptr(rp), _ptr(cols), _ptr(vals)))
        return rp, cols, vals

    def write_hh(self, path: str) -> None:
        _check(lib().cg_hamiltonian_write_hh(self._h, path.encode()))

    def times_matrix(self, x: np.ndarray, precision: int | None = None) -> np.ndarray:
        """y = H x for the columns of x (n x m), like SparseMatrixCSB::TimesMatrix."""
        x = np.asarray(x, dtype=np.float64)
        x2 = x.reshape(self.n, -1)
        m = x2.shape[1]
        xc = np.ascontiguousarray(x2.T)  # vector k at k*n
        yc = np.zeros_like(xc)
        prec = self.precision if precision is None else precision
        _check(lib().cg_spmm(self._h, _ptr(xc), _ptr(yc), m, prec))
        return yc.T.reshape(x.shape)

    def spmm_device(self, x_ptr: int, ldx: int, y_ptr: int, ldy: int, m: int, precision: int) -> None:
        _check(lib().cg_spmm_device(self._h, x_ptr, ldx, y_ptr, ldy, m, precision))

    def autotune(self, nvec: int = 8, reps: int = 3, cache: str | None = None) -> dict:
        """Choose the FP32 product's launch shape for this matrix (timed on the
        device).  With `cache` (a JSON file) a previous choice for the same
        matrix size, vector count and device is reused instead of re-timing."""
        import json
        key = f"n={self.n},nnz={int(self.info.nnz_full)},nvec={nvec},dev={_device_name()}"
        if cache and os.path.exists(cache):
            with open(cache) as f:
                db = json.load(f)
            if key in db:
                w, c = db[key]["warps"], db[key]["ctas_per_sm"]
                _check(lib().cg_spmm_set_tuning(self._h, w, c))
                fmt = db[key].get("format", CG_FORMAT_ROWS)
                if fmt == CG_FORMAT_TILED and not self.format()[1]:
                    fmt = CG_FORMAT_ROWS
                if self.format()[1]:
                    self.set_format(fmt)
                    if "tiled_shape" in db[key]:
                        self.set_tiled_shape(*db[key]["tiled_shape"])
                return {"warps": w, "ctas_per_sm": c, "format": fmt, "cached": True}
        cap = C.c_int32(64)
        w = np.zeros(64, dtype=np.int32)
        c = np.zeros(64, dtype=np.int32)
        ms = np.zeros(64, dtype=np.float32)
        _check(lib().cg_spmm_autotune(self._h, nvec, reps, C.byref(cap), _ptr(w), _ptr(c), _ptr(ms)))
        k = int(cap.value)
        bw, bc, _ = self.tuning()
        fmt = self.format()[0]
        res = {"warps": bw, "ctas_per_sm": bc, "format": fmt, "cached": False,
               "candidates": [(int(w[i]), int(c[i]), float(ms[i])) for i in range(k)]}
        if cache:
            db = {}
            if os.path.exists(cache):
                with open(cache) as f:
                    db = json.load(f)
            db[key] = {"warps": bw, "ctas_per_sm": bc, "format": fmt, "ms": float(min(ms[:k]))}
            fi = self.format_info()
            if fi["tiled_available"]:
                db[key]["tiled_shape"] = [fi["slices_per_warp"], fi["stages"]]
            with open(cache, "w") as f:
                json.dump(db, f, indent=1, sort_keys=True)
        return res

    def tuning(self):
        w, c, t = C.c_int32(), C.c_int32(), C.c_int32()
        _check(lib().cg_spmm_get_tuning(self._h, C.byref(w), C.byref(c), C.byref(t)))
        return int(w.value), int(c.value), bool(t.value)

    def set_format(self, fmt: int) -> None:
        """Storage the FP32 product of up to 8 vectors reads: CG_FORMAT_ROWS
        (row-wise) or CG_FORMAT_TILED (neutron-block tiles)."""
        _check(lib().cg_spmm_set_format(self._h, fmt))

    def format(self):
        """(format in use, tiled copy present, tiled entries incl. padding)."""
        i = self.format_info()
        return i["format"], i["tiled_available"], i["entries"]

    def set_tiled_shape(self, slices_per_warp: int, stages: int) -> None:
        """Launch shape of the tiled product: slices per consumer warp, ring slots."""
        _check(lib().cg_spmm_set_tiled_shape(self._h, slices_per_warp, stages))

    def format_info(self) -> dict:
        i = SpmmFormatInfo()
        _check(lib().cg_spmm_get_format(self._h, C.byref(i)))
        d = {k: getattr(i, k) for k, _ in SpmmFormatInfo._fields_}
        d["tiled_available"] = bool(d["tiled_available"])
        return d


@dataclass
class DavidsonResult:
    eig: np.ndarray
    de: np.ndarray
    resid: np.ndarray
    vecs: np.ndarray | None
    stats: DavidsonStats


def davidson_params(nstates: int, **kw) -> DavidsonParams:
    p = DavidsonParams()
    lib().cg_davidson_defaults(C.byref(p), nstates)
    for k, v in kw.items():
        if not hasattr(p, k):
            raise TypeError(f"unknown Davidson parameter {k}")
        setattr(p, k, v)
    return p


def davidson_diagonalization(h: Hamiltonian, nstates: int = 10, want_vectors: bool = True,
                             init: np.ndarray | None = None, **kw) -> DavidsonResult:
    """Lowest eigenpairs of h (DavidsonDiagonalization, include/kdav/davidson.cxx:168).

    Keyword arguments set :class:`DavidsonParams` fields (block, lim, maxiter,
    crite, critc, critr, ortho, tol_resid, switch_resid, precision, verbose,
    ortho_block, algorithm, keep, precond, refine_lim, refine_keep, ortho_pip, refine_block,
    refine_fp32_corrections).  precision
    defaults to the matrix precision."""
    kw.setdefault("precision", h.precision)
    p = davidson_params(nstates, **kw)
    eig = np.zeros(nstates)
    de = np.zeros(nstates)
    res = np.zeros(nstates)
    vecs = np.zeros((nstates, h.n)) if want_vectors else None
    st = DavidsonStats()
    ninit = 0
    ip = None
    if init is not None:
        init = np.ascontiguousarray(np.asarray(init, dtype=np.float64).reshape(-1, h.n))
        ninit = init.shape[0]
        ip = _ptr(init)
    _check(lib().cg_davidson(h._h, C.byref(p), ip, ninit, _ptr(eig), _ptr(de), _ptr(res),
                             _ptr(vecs) if vecs is not None else None, C.byref(st)))
    return DavidsonResult(eig, de, res, vecs, st)


def write_ee(path: str, eig, de, resid, vecs) -> None:
    """Write a .EE eigenpair file (Davidson::Save, include/kdav/cdavidson.cpp:327-368)."""
    eig = np.ascontiguousarray(eig, dtype=np.float64)
    de = np.ascontiguousarray(de, dtype=np.float64)
    resid = np.ascontiguousarray(resid, dtype=np.float64)
    vecs = np.ascontiguousarray(vecs, dtype=np.float64)
    _check(lib().cg_write_ee(path.encode(), len(eig), vecs.shape[1], _ptr(eig), _ptr(de), _ptr(resid), _ptr(vecs)))


def read_ee(path: str):
    """Read a .EE file: returns (E, dE, resid, vectors)."""
    with open(path, "rb") as f:
        cnt = int(np.frombuffer(f.read(4), dtype=np.uint32)[0])
        E, dE, R, V = [], [], [], []
        for _ in range(cnt):
            e, d, r = np.frombuffer(f.read(24), dtype=np.float64)
            n = int(np.frombuffer(f.read(8), dtype=np.uint64)[0])
            V.append(np.frombuffer(f.read(8 * n), dtype=np.float64).copy())
            E.append(e); dE.append(d); R.append(r)
    return np.array(E), np.array(dE), np.array(R), np.array(V)


def read_mbs(path: str) -> np.ndarray:
    """Read a .mbs basis file (Many_Body_States::Read, include/sm/ManyBodyStates.cxx:209)."""
    with open(path, "rb") as f:
        N = int(np.frombuffer(f.read(4), dtype=np.int32)[0])
        n = int(np.frombuffer(f.read(8), dtype=np.uint64)[0])
        z = np.frombuffer(f.read(2 * N * n), dtype=np.uint16).reshape(n, N)
    return z
