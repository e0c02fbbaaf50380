"""Python host binding of libgainls.so (the C ABI declared in include/gain_ls.h).

The library is the product; this module only marshals arguments through ctypes.  It never
falls back to a CPU implementation: if the shared library is missing, every call raises.

    import gainls
    eng = gainls.Engine(jmax=11, nsym=4, maxdeg=1)
    gainls.upload_problem(eng, problem)          # a synth.Problem
    stats = eng.run_pair(job, gainls.PATH_SPLIT)
"""
from __future__ import annotations

import ctypes
import os
from typing import Optional, Sequence

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
# GAINLS_LIBRARY selects another build of the same C ABI (e.g. an instrumented one)
LIB_PATH = os.environ.get("GAINLS_LIBRARY") or os.path.join(HERE, "lib", "libgainls.so")
HEADER = os.path.join(os.path.dirname(HERE), "include", "gain_ls.h")

PATH_PLAIN_FP64 = 0
PATH_SPLIT = 1

OK, ERR_INVALID_ARG, ERR_OOM, ERR_CUDA, ERR_TIMEOUT, ERR_TOL_NOT_MET, ERR_NOT_READY, ERR_UNSUPPORTED = range(8)

_ip = ctypes.POINTER(ctypes.c_int)
_dp = ctypes.POINTER(ctypes.c_double)
_vp = ctypes.c_void_p


class GainError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{_status_name(status)}: {message}")
        self.status = status


class PairJob(ctypes.Structure):
    _fields_ = [("jindI", ctypes.c_int), ("gammaI", ctypes.c_int), ("jindF", ctypes.c_int),
                ("gammaF", ctypes.c_int), ("nlower", ctypes.c_int), ("lower_levels", _ip),
                ("nupper", ctypes.c_int), ("upper_levels", _ip)]


class SplitOpts(ctypes.Structure):
    _fields_ = [("tol", ctypes.c_double), ("slices", ctypes.c_int), ("beta", ctypes.c_int),
                ("kchunks", ctypes.c_int), ("s_floor", ctypes.c_double)]


class Stats(ctypes.Structure):
    _fields_ = [("device_ms", ctypes.c_double), ("rows", ctypes.c_longlong), ("cols", ctypes.c_longlong),
                ("refined", ctypes.c_longlong), ("uncertified", ctypes.c_longlong),
                ("uncertified_weak", ctypes.c_longlong), ("inexact", ctypes.c_longlong),
                ("amp_max", ctypes.c_double),
                ("beta1", ctypes.c_int), ("slices1", ctypes.c_int), ("chunks1", ctypes.c_int),
                ("beta2", ctypes.c_int), ("slices2", ctypes.c_int), ("chunks2", ctypes.c_int),
                ("products1", ctypes.c_int), ("products2", ctypes.c_int),
                ("kernel_launches", ctypes.c_int),
                ("gemm1_ms", ctypes.c_double), ("gemm2_ms", ctypes.c_double),
                ("tensor_flops", ctypes.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class PlanStats(ctypes.Structure):
    _fields_ = [("device_ms", ctypes.c_double), ("gemm1_ms", ctypes.c_double), ("gemm2_ms", ctypes.c_double),
                ("transitions", ctypes.c_longlong), ("refined", ctypes.c_longlong),
                ("uncertified", ctypes.c_longlong), ("jobs", ctypes.c_int), ("failed_jobs", ctypes.c_int),
                ("graph_nodes", ctypes.c_int), ("kernel_launches", ctypes.c_int), ("gemm1_tiles", ctypes.c_int),
                ("gemm2_tiles", ctypes.c_int), ("units", ctypes.c_int), ("pair", ctypes.c_int),
                ("captures", ctypes.c_int), ("tuned", ctypes.c_int), ("tune_ms", ctypes.c_double),
                ("tensor_flops", ctypes.c_double), ("beta2", ctypes.c_int * 4), ("slices2", ctypes.c_int * 4),
                ("digits_ms", ctypes.c_double), ("middle_ms", ctypes.c_double), ("refine_ms", ctypes.c_double),
                ("shared_lower", ctypes.c_int), ("shared_upper", ctypes.c_int)]

    def as_dict(self):
        d = {k: getattr(self, k) for k, _ in self._fields_}
        d["beta2"], d["slices2"] = list(self.beta2), list(self.slices2)
        return d


class LineParams(ctypes.Structure):
    _fields_ = [("temperature", ctypes.c_double), ("q_part", ctypes.c_double), ("zpe", ctypes.c_double),
                ("thresh", ctypes.c_double), ("freq_lo", ctypes.c_double), ("freq_hi", ctypes.c_double),
                ("gnsF", ctypes.c_double), ("ndegI", ctypes.c_int), ("ndegF", ctypes.c_int),
                ("reduced", ctypes.c_int)]


class State(ctypes.Structure):
    _fields_ = [("energy", ctypes.c_double), ("J", ctypes.c_int), ("jind", ctypes.c_int),
                ("gamma", ctypes.c_int), ("ndeg", ctypes.c_int), ("ilevel", ctypes.c_int)]


class Filters(ctypes.Structure):
    _fields_ = [("nsym", ctypes.c_int), ("gns", _dp), ("isym_pairs", _ip), ("igamma_pair", _ip),
                ("sym_degen", _ip), ("erange_lower", ctypes.c_double * 2), ("erange_upper", ctypes.c_double * 2),
                ("freq_window", ctypes.c_double * 2), ("zpe", ctypes.c_double), ("maxJ", ctypes.c_int),
                ("reduced", ctypes.c_int), ("symmetry_type", ctypes.c_int)]


class TroveState(ctypes.Structure):
    _fields_ = [("energy", ctypes.c_double), ("irec", ctypes.c_int), ("ilevel", ctypes.c_int),
                ("krot", ctypes.c_int), ("taurot", ctypes.c_int), ("rec_len", ctypes.c_int)]


def make_filters(gns, isym_pairs, igamma_pair, sym_degen, erange_lower, erange_upper,
                 freq_window=(-1e9, 1e9), zpe=0.0, maxJ=0, reduced=False, symmetry_type=1):
    """A Filters struct plus the arrays it points to (kept alive on the struct)."""
    arrs = [np.ascontiguousarray(gns, np.float64), np.ascontiguousarray(isym_pairs, np.int32),
            np.ascontiguousarray(igamma_pair, np.int32), np.ascontiguousarray(sym_degen, np.int32)]
    f = Filters(len(arrs[0]), arrs[0].ctypes.data_as(_dp), arrs[1].ctypes.data_as(_ip),
                arrs[2].ctypes.data_as(_ip), arrs[3].ctypes.data_as(_ip),
                (ctypes.c_double * 2)(*erange_lower), (ctypes.c_double * 2)(*erange_upper),
                (ctypes.c_double * 2)(*freq_window), zpe, maxJ, int(reduced), symmetry_type)
    f._keep = arrs
    return f


def state_table(energy, J, jind, gamma, ndeg, ilevel):
    n = len(energy)
    arr = (State * n)()
    for i in range(n):
        arr[i] = State(float(energy[i]), int(J[i]), int(jind[i]), int(gamma[i]), int(ndeg[i]), int(ilevel[i]))
    return arr


def filter_intensity(f: Filters, I: State, F: State) -> bool:
    return bool(lib().gain_filter_intensity(ctypes.byref(f), ctypes.byref(I), ctypes.byref(F)))


def filter_lower(f: Filters, I: State) -> bool:
    return bool(lib().gain_filter_lower(ctypes.byref(f), ctypes.byref(I)))


def degeneracy_filter(f: Filters, gI, gF, idegI, idegF) -> bool:
    return bool(lib().gain_degeneracy_filter(ctypes.byref(f), gI, gF, idegI, idegF))


def transition_details(f: Filters, table):
    a, b, c = ctypes.c_int(), ctypes.c_longlong(), ctypes.c_int()
    check(lib().gain_transition_details(ctypes.byref(f), table, len(table), ctypes.byref(a), ctypes.byref(b),
                                        ctypes.byref(c)))
    return a.value, b.value, c.value


def plan_pairs(f: Filters, table):
    """[(jindI, gammaI, jindF, gammaF, lower_levels, upper_levels), ...]"""
    npairs, nlev = ctypes.c_int(), ctypes.c_longlong()
    check(lib().gain_plan_pairs(ctypes.byref(f), table, len(table), ctypes.byref(npairs), None, None,
                                ctypes.byref(nlev), None))
    pairs = np.zeros(4 * npairs.value, np.int32)
    offs = np.zeros(2 * npairs.value + 1, np.int32)
    levels = np.zeros(max(nlev.value, 1), np.int32)
    check(lib().gain_plan_pairs(ctypes.byref(f), table, len(table), ctypes.byref(npairs), _p(pairs, _ip),
                                _p(offs, _ip), ctypes.byref(nlev), _p(levels, _ip)))
    out = []
    for p in range(npairs.value):
        out.append((*[int(x) for x in pairs[4 * p:4 * p + 4]], levels[offs[2 * p]:offs[2 * p + 1]].tolist(),
                    levels[offs[2 * p + 1]:offs[2 * p + 2]].tolist()))
    return out


_lib = None


def _status_name(s: int) -> str:
    names = ["GAIN_OK", "GAIN_ERR_INVALID_ARG", "GAIN_ERR_OOM", "GAIN_ERR_CUDA", "GAIN_ERR_TIMEOUT",
             "GAIN_ERR_TOL_NOT_MET", "GAIN_ERR_NOT_READY", "GAIN_ERR_UNSUPPORTED"]
    return names[s] if 0 <= s < len(names) else f"status {s}"


def lib():
    """Load libgainls.so; raise if it has not been built (there is no fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: build it with gain-mpi_gb300/build.py "
                               "(or __graft_entry__.build()); there is no CPU fallback")
        L = ctypes.CDLL(LIB_PATH)
        _declare(L)
        _lib = L
    return _lib


def _declare(L):
    I, D, S = ctypes.c_int, ctypes.c_double, ctypes.c_int
    L.gain_last_error_string.restype = ctypes.c_char_p
    L.gain_status_string.restype = ctypes.c_char_p
    L.gain_status_string.argtypes = [I]
    L.gain_abi_version.restype = I
    L.gain_hls_kblock.argtypes = [I, I, I, I, I, _vp, _vp, _vp, _vp, I, I, I, I, I, I, _vp, _vp, _vp,
                                  _vp, _vp, I, I, _vp]
    L.gain_expand.argtypes = [I, I, I, I, I, I, _vp, _vp, _vp, _vp, _vp, _vp, _vp]
    L.gain_hls_rotsym.argtypes = [I, I, I, I, I, _vp, _vp, _vp, _vp, _vp, _vp, I, I, I, _vp, _vp, _vp, _vp, I, _vp]
    L.gain_dot.argtypes = [I, _vp, _vp, _vp, _vp]
    L.gain_threej_table.argtypes = [I, _dp]
    L.gain_engine_create.argtypes = [I, I, I, I, ctypes.POINTER(_vp)]
    L.gain_engine_destroy.argtypes = [_vp]
    L.gain_upload_basis.argtypes = [_vp, I, I, I, _ip, _ip, _ip, _ip, _ip]
    L.gain_upload_inflation.argtypes = [_vp, I, _ip, _ip, I, I, I, ctypes.POINTER(_ip), ctypes.POINTER(_dp),
                                        _ip, _ip]
    L.gain_upload_dipole.argtypes = [_vp, _dp, I, I, I, I]
    L.gain_upload_eigvecs.argtypes = [_vp, I, I, I, I, _dp]
    L.gain_selftest_bounded_wait.argtypes = [_vp, D]
    L.gain_selftest_bounded_wait.restype = S
    L.gain_upload_dipole_pieces.argtypes = [_vp, I, ctypes.POINTER(_dp), I, _ip, _ip]
    L.gain_upload_dipole_pieces.restype = S
    L.gain_upload_wigner.argtypes = [_vp, I, I, I, I, I, _dp]
    L.gain_adjoint_pair.argtypes = [_vp, ctypes.POINTER(PairJob), _dp, _dp, ctypes.POINTER(Stats)]
    L.gain_adjoint_pair_prec.argtypes = [_vp, ctypes.POINTER(PairJob), _dp, _dp, ctypes.c_int, ctypes.POINTER(Stats)]
    L.gain_adjoint_pair_degenerate.argtypes = [_vp, ctypes.POINTER(PairJob), ctypes.POINTER(Filters), _dp, _dp,
                                               ctypes.c_int, ctypes.POINTER(Stats)]
    L.gain_plan_create.argtypes = [_vp, ctypes.POINTER(PairJob), I, ctypes.POINTER(SplitOpts), I, ctypes.POINTER(_vp)]
    L.gain_plan_run.argtypes = [_vp, ctypes.POINTER(Stats), ctypes.POINTER(PlanStats)]
    L.gain_plan_select.argtypes = [_vp, I]
    L.gain_plan_amp_device.argtypes = [_vp, I, ctypes.POINTER(ctypes.c_void_p), _ip]
    L.gain_plan_destroy.argtypes = [_vp]
    for name in ("gain_plan_create", "gain_plan_run", "gain_plan_select", "gain_plan_amp_device", "gain_plan_destroy"):
        getattr(L, name).restype = S
    L.gain_run_plan.argtypes = [ctypes.POINTER(_vp), ctypes.c_int, ctypes.POINTER(PairJob), ctypes.c_int, ctypes.c_int,
                                ctypes.POINTER(SplitOpts), JOB_DONE_FN, _vp, ctypes.POINTER(Stats)]
    L.gain_run_pair_component.argtypes = [_vp, ctypes.POINTER(PairJob), ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                          ctypes.POINTER(SplitOpts), ctypes.POINTER(Stats)]
    L.gain_run_pair_degenerate.argtypes = [_vp, ctypes.POINTER(PairJob), ctypes.POINTER(Filters), ctypes.c_int,
                                           ctypes.POINTER(SplitOpts), ctypes.POINTER(Stats)]
    L.gain_upload_eigvecs_async.argtypes = [_vp, I, I, I, I, _dp]
    L.gain_release_eigvecs.argtypes = [_vp, I, I]
    L.gain_release_eigvecs.restype = S
    L.gain_run_pair.argtypes = [_vp, ctypes.POINTER(PairJob), I, ctypes.POINTER(SplitOpts), ctypes.POINTER(Stats)]
    L.gain_pair_amp_device.argtypes = [_vp, ctypes.POINTER(ctypes.c_void_p), _ip]
    L.gain_fetch_amp.argtypes = [_vp, _dp]
    L.gain_pair_lines.argtypes = [_vp, ctypes.POINTER(LineParams), _dp, _dp, I, I, _dp, _dp, _dp,
                                  ctypes.POINTER(ctypes.c_ubyte), ctypes.POINTER(ctypes.c_longlong)]
    L.gain_pair_lines_async.argtypes = [_vp, ctypes.POINTER(LineParams), _dp, _dp, I, I, _dp, _dp, _dp,
                                  ctypes.POINTER(ctypes.c_ubyte), ctypes.POINTER(ctypes.c_longlong)]
    L.gain_lines_wait.argtypes = [_vp]
    L.gain_lines_threshold_refined.argtypes = [_vp, ctypes.POINTER(ctypes.c_longlong)]
    L.gain_lines_intensity_host.argtypes = [_vp, ctypes.POINTER(ctypes.c_longlong)]
    L.gain_format_line.argtypes = [ctypes.c_char_p, ctypes.c_size_t, D, I, I, I, I, I, I, D, I, D, _dp, I]
    L.gain_format_line.restype = I
    L.gain_format_line_native.argtypes = [ctypes.c_char_p, ctypes.c_size_t, D, I, I, I, I, I, I, D, I, D, _dp, I]
    L.gain_format_line_native.restype = I
    L.gain_line_length_native.argtypes = [D, I, I, I, I, I, I, D, I, D, _dp, I]
    L.gain_line_length_native.restype = ctypes.c_long
    L.gain_format_value.argtypes = [ctypes.c_char_p, ctypes.c_size_t, D, I, I, I]
    L.gain_format_value.restype = I
    U64 = ctypes.c_ulonglong
    L.gain_pair_lines_text.argtypes = [_vp, ctypes.POINTER(LineParams), _dp, _dp, I, I, I, I, I,
                                       ctypes.POINTER(U64), ctypes.POINTER(ctypes.c_longlong)]
    L.gain_fetch_lines_text.argtypes = [_vp, ctypes.c_void_p, U64]
    L.gain_pair_lines_text_host.argtypes = [_vp, ctypes.POINTER(LineParams), _dp, _dp, I, I, I, I, I,
                                            ctypes.c_void_p, U64, ctypes.POINTER(U64), ctypes.POINTER(ctypes.c_longlong)]
    L.gain_lines_text_device.argtypes = [_vp, ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(U64)]
    L.gain_format_values_device.argtypes = [_dp, ctypes.c_longlong, I, I, I, ctypes.c_char_p, I, _ip]
    FP, SP = ctypes.POINTER(Filters), ctypes.POINTER(State)
    L.gain_filter_lower.argtypes = [FP, SP]
    L.gain_filter_lower.restype = I
    L.gain_filter_intensity.argtypes = [FP, SP, SP]
    L.gain_filter_intensity.restype = I
    L.gain_degeneracy_filter.argtypes = [FP, I, I, I, I]
    L.gain_degeneracy_filter.restype = I
    L.gain_transition_details.argtypes = [FP, SP, I, _ip, ctypes.POINTER(ctypes.c_longlong), _ip]
    L.gain_transition_details.restype = S
    L.gain_plan_pairs.argtypes = [FP, SP, I, _ip, _ip, _ip, ctypes.POINTER(ctypes.c_longlong), _ip]
    L.gain_plan_pairs.restype = S
    L.gain_trove_basis_read.argtypes = [ctypes.c_char_p, I, I, _ip, I, ctypes.POINTER(_vp)]
    L.gain_trove_basis_free.argtypes = [_vp]
    L.gain_trove_basis_free.restype = None
    L.gain_trove_basis_info.argtypes = [_vp, _ip, _ip, _ip, _ip, _ip]
    L.gain_trove_basis_arrays.argtypes = [_vp, _ip, _ip, _ip, _ip, _ip, _ip, _ip]
    L.gain_trove_basis_repres.argtypes = [_vp, I, _ip, _dp]
    L.gain_trove_basis_upload.argtypes = [_vp, I, _vp]
    L.gain_trove_dipole_read.argtypes = [ctypes.c_char_p, ctypes.c_ulonglong, ctypes.POINTER(_vp)]
    L.gain_trove_dipole_free.argtypes = [_vp]
    L.gain_trove_dipole_free.restype = None
    L.gain_trove_dipole_info.argtypes = [_vp, _ip, _ip]
    L.gain_trove_dipole_block.argtypes = [_vp, I, _ip, _ip, _ip, ctypes.POINTER(_dp)]
    L.gain_trove_states_read.argtypes = [ctypes.c_char_p, I, I, ctypes.POINTER(Filters), _ip,
                                         ctypes.POINTER(TroveState), _ip]
    L.gain_trove_vectors_read.argtypes = [ctypes.c_char_p, I, _ip, I, _dp]
    for name in ("gain_trove_basis_read", "gain_trove_basis_info", "gain_trove_basis_arrays",
                 "gain_trove_basis_repres", "gain_trove_basis_upload", "gain_trove_dipole_read",
                 "gain_trove_dipole_info", "gain_trove_dipole_block", "gain_trove_states_read",
                 "gain_trove_vectors_read"):
        getattr(L, name).restype = S
    for name in ("gain_hls_kblock", "gain_hls_rotsym", "gain_expand", "gain_dot", "gain_threej_table", "gain_engine_create",
                 "gain_engine_destroy", "gain_upload_basis", "gain_upload_inflation", "gain_upload_dipole",
                 "gain_upload_eigvecs", "gain_upload_eigvecs_async", "gain_upload_wigner", "gain_adjoint_pair",
                 "gain_adjoint_pair_prec", "gain_run_pair", "gain_run_pair_component", "gain_run_pair_degenerate",
                 "gain_run_plan", "gain_adjoint_pair_degenerate", "gain_pair_amp_device", "gain_fetch_amp",
                 "gain_pair_lines", "gain_pair_lines_async", "gain_lines_wait", "gain_lines_threshold_refined", "gain_lines_intensity_host",
                 "gain_pair_lines_text", "gain_pair_lines_text_host", "gain_fetch_lines_text",
                 "gain_lines_text_device",
                 "gain_format_values_device"):
        getattr(L, name).restype = S


def check(status: int):
    if status != OK:
        msg = lib().gain_last_error_string().decode(errors="replace")
        raise GainError(status, msg)


def declared_symbols() -> list[str]:
    """Every function name the C headers include/gain_ls.h and include/gain_trove.h declare."""
    import re
    text = open(HEADER).read() + open(os.path.join(os.path.dirname(HEADER), "gain_trove.h")).read()
    return sorted(set(re.findall(r"\b(gain_[a-z0-9_]+)\s*\(", text)))


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _p(a, t):
    return a.ctypes.data_as(t)


# --------------------------------------------------------------------------- layer 1
def threej_table(jmax: int) -> np.ndarray:
    t = np.zeros((jmax + 1) * (jmax + 1) * 9, np.float64)
    check(lib().gain_threej_table(jmax, _p(t, _dp)))
    return t


def hls_kblock(dimenF, dimenI, jI, jF, kF, tauI, tauF, icorrI, icorrF, startF_idx, startI_idx,
               startFblock, endFblock, ncontrF, kFBlocksize, kblock_size, dipole_me, vector, threej,
               half_ls, jmax, dip_stride, stream=0):
    """Drop-in K-block kernel; pointer arguments are device addresses (ints)."""
    check(lib().gain_hls_kblock(dimenF, dimenI, jI, jF, kF, tauI, tauF, icorrI, icorrF, startF_idx,
                                startI_idx, startFblock, endFblock, ncontrF, kFBlocksize, kblock_size,
                                dipole_me, vector, threej, half_ls, jmax, dip_stride, stream))


def expand(dimenI, igammaI, maxcoeff, idegI, sdeg, Ntot, ijterms, icontr, N, repres, vecI, vec, stream=0):
    check(lib().gain_expand(dimenI, igammaI, maxcoeff, idegI, sdeg, Ntot, ijterms, icontr, N, repres,
                            vecI, vec, stream))


def hls_rotsym(dimenF, dimenI, nlevelI, nlevelF, sym_max_degen, kI, kF, ktauI, ktauF, icorrI, icorrF,
               startFblock, endFblock, ncontrF, dipole_me, wigner, vector, half_ls, dip_stride, stream=0):
    """gain_hls_rotsym on device pointers (ints)."""
    check(lib().gain_hls_rotsym(dimenF, dimenI, nlevelI, nlevelF, sym_max_degen, kI, kF, ktauI, ktauF, icorrI,
                                icorrF, startFblock, endFblock, ncontrF, dipole_me, wigner, vector, half_ls,
                                dip_stride, stream))


def dot(n, x, y, result, stream=0):
    check(lib().gain_dot(n, x, y, result, stream))


def format_line_native(nu, indexF, jF, gammaF, indexI, jI, gammaI, A, intensity=None, amps=None) -> str:
    """The same line through the library's own conversions (the device kernels' code)."""
    buf = ctypes.create_string_buffer(4096)
    a = _f64(amps) if amps is not None else None
    n = lib().gain_format_line_native(buf, 4096, nu, indexF, jF, gammaF, indexI, jI, gammaI, A,
                                      int(intensity is not None), 0.0 if intensity is None else intensity,
                                      _p(a, _dp) if a is not None else None, 0 if a is None else len(a))
    assert n > 0
    return buf.raw[:n].decode()


def line_length_native(nu, indexF, jF, gammaF, indexI, jI, gammaI, A, intensity=None, amps=None) -> int:
    a = _f64(amps) if amps is not None else None
    return int(lib().gain_line_length_native(nu, indexF, jF, gammaF, indexI, jI, gammaI, A,
                                             int(intensity is not None), 0.0 if intensity is None else intensity,
                                             _p(a, _dp) if a is not None else None, 0 if a is None else len(a)))


def format_value(x: float, conv: str, width: int, prec: int) -> str:
    """x through the library's "%<width>.<prec>E" / "%<width>.<prec>f" conversion (host build)."""
    buf = ctypes.create_string_buffer(512)
    n = lib().gain_format_value(buf, 512, x, ord(conv), width, prec)
    assert n > 0, n
    return buf.raw[:n].decode()


def format_values_device(values, conv: str, width: int, prec: int, stride: int = 400) -> list:
    """values through the device conversion kernel (one GPU launch)."""
    v = _f64(values)
    out = ctypes.create_string_buffer(max(1, v.size * stride))
    lens = np.zeros(v.size, np.int32)
    check(lib().gain_format_values_device(_p(v, _dp), v.size, ord(conv), width, prec, out, stride, _p(lens, _ip)))
    raw = out.raw
    return [raw[i * stride:i * stride + int(n)].decode() for i, n in enumerate(lens)]


def format_line(nu, indexF, jF, gammaF, indexI, jI, gammaI, A, intensity=None, amps=None) -> str:
    buf = ctypes.create_string_buffer(4096)
    a = _f64(amps) if amps is not None else None
    n = lib().gain_format_line(buf, 4096, nu, indexF, jF, gammaF, indexI, jI, gammaI, A,
                               int(intensity is not None), 0.0 if intensity is None else intensity,
                               _p(a, _dp) if a is not None else None, 0 if a is None else len(a))
    return buf.raw[:n].decode()


# --------------------------------------------------------------------------- layer 2
class Engine:
    def __init__(self, jmax: int, nsym: int, maxdeg: int = 1, device: int = 0):
        h = _vp()
        check(lib().gain_engine_create(device, jmax, nsym, maxdeg, ctypes.byref(h)))
        self.h = h
        self.nsym = nsym
        self._keep = {}

    def close(self):
        if self.h:
            lib().gain_engine_destroy(self.h)
            self.h = _vp()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def upload_basis(self, jind, J, K, tau, vib, kblock, kstart):
        K, tau, vib, kblock, kstart = map(_i32, (K, tau, vib, kblock, kstart))
        check(lib().gain_upload_basis(self.h, jind, J, len(K), _p(K, _ip), _p(tau, _ip), _p(vib, _ip),
                                      _p(kblock, _ip), _p(kstart, _ip)))

    def upload_inflation(self, jind, icontr, ijterms, dimen, maxcoeff, matsize, N, repres, Ntot, sdeg):
        icontr, ijterms, Ntot, sdeg = map(_i32, (icontr, ijterms, Ntot, sdeg))
        Ns = [_i32(x) for x in N]
        Rs = [_f64(x) for x in repres]
        Np = (_ip * len(Ns))(*[_p(x, _ip) for x in Ns])
        Rp = (_dp * len(Rs))(*[_p(x, _dp) for x in Rs])
        check(lib().gain_upload_inflation(self.h, jind, _p(icontr, _ip), _p(ijterms, _ip), dimen, maxcoeff,
                                          matsize, Np, Rp, _p(Ntot, _ip), _p(sdeg, _ip)))

    def upload_dipole(self, piece, N, startF, endF, ncontrF):
        piece = _f64(piece)
        check(lib().gain_upload_dipole(self.h, _p(piece, _dp), N, startF, endF, ncontrF))

    def upload_dipole_pieces(self, pieces, N):
        """pieces: [(startF, endF, piece[3*N*(endF-startF)]), ...] kept in host memory (the
        arrays stay referenced by the engine); runs loop over them."""
        arrs = [_f64(a) for (_, _, a) in pieces]
        self._keep["dipole_pieces"] = arrs
        ptrs = (_dp * len(arrs))(*[_p(a, _dp) for a in arrs])
        s, e = _i32([x[0] for x in pieces]), _i32([x[1] for x in pieces])
        check(lib().gain_upload_dipole_pieces(self.h, len(arrs), ptrs, N, _p(s, _ip), _p(e, _ip)))

    def upload_eigvecs(self, jind, gamma, vecs):
        vecs = _f64(vecs)
        check(lib().gain_upload_eigvecs(self.h, jind, gamma, vecs.shape[0], vecs.shape[1], _p(vecs, _dp)))

    def upload_wigner(self, jindI, jindF, nlevelsI, nlevelsF, maxdeg, rot):
        rot = _f64(rot)
        assert rot.size == 3 * nlevelsI * nlevelsF * maxdeg * maxdeg
        check(lib().gain_upload_wigner(self.h, jindI, jindF, nlevelsI, nlevelsF, maxdeg, _p(rot, _dp)))

    def upload_eigvecs_device(self, jind, gamma, ptr: int, nlevels: int, nsize: int):
        """gain_upload_eigvecs from device memory (ptr: a device address of nlevels x nsize
        doubles, e.g. a torch tensor's data_ptr()).  The engine copies on its own stream, so
        torch's current stream (which may still be writing the tensor) is synchronised first."""
        try:
            import torch
            if torch.cuda.is_available():
                torch.cuda.current_stream().synchronize()
        except ImportError:
            pass
        check(lib().gain_upload_eigvecs(self.h, jind, gamma, nlevels, nsize, ctypes.cast(ptr, _dp)))

    def release_eigvecs(self, jind, gamma):
        check(lib().gain_release_eigvecs(self.h, jind, gamma))

    def upload_eigvecs_async(self, jind, gamma, vecs):
        """Queue the copy of page-locked vecs (C-contiguous float64, kept unchanged until the
        next run_pair returns); pageable arrays are copied synchronously."""
        assert vecs.dtype == np.float64 and vecs.flags.c_contiguous and vecs.ndim == 2
        check(lib().gain_upload_eigvecs_async(self.h, jind, gamma, vecs.shape[0], vecs.shape[1], _p(vecs, _dp)))

    def run_pair(self, jindI, gammaI, jindF, gammaF, lower_levels: Sequence[int],
                 upper_levels: Sequence[int], path: int = PATH_SPLIT, tol: float = 0.0,
                 slices: int = 0, beta: int = 0, kchunks: int = 0, s_floor: float = 0.0,
                 raise_on_error: bool = True, components=None, filters=None) -> dict:
        """Amplitudes of one block pair.  components=(idegI, idegF): that degenerate component
        pair, kept in its slot (gain_run_pair_component); filters: every component pair
        passing the degeneracy filter (gain_run_pair_degenerate)."""
        lo, up = _i32(lower_levels), _i32(upper_levels)
        job = PairJob(jindI, gammaI, jindF, gammaF, len(lo), _p(lo, _ip), len(up), _p(up, _ip))
        opts = SplitOpts(tol, slices, beta, kchunks, s_floor)
        st = Stats()
        if filters is not None:
            s = lib().gain_run_pair_degenerate(self.h, ctypes.byref(job), ctypes.byref(filters), path,
                                               ctypes.byref(opts), ctypes.byref(st))
        elif components is not None:
            s = lib().gain_run_pair_component(self.h, ctypes.byref(job), int(components[0]), int(components[1]), path,
                                              ctypes.byref(opts), ctypes.byref(st))
        else:
            s = lib().gain_run_pair(self.h, ctypes.byref(job), path, ctypes.byref(opts), ctypes.byref(st))
        self._shape = (len(lo), len(up))
        out = st.as_dict()
        out["status"] = s
        if s != OK:
            out["error"] = lib().gain_last_error_string().decode(errors="replace")
            if raise_on_error:
                check(s)
        return out

    def adjoint(self, jindI, gammaI, jindF, gammaF, lower_levels, upper_levels, dL_dS, dL_dmu=None,
                precision="f64", filters=None):
        """dL/dmu (the dipole piece's layout [3][N][ncontrF], accumulated into dL_dmu if given)
        of a loss with gradient dL_dS [nlower, nupper] over the pair's line strengths;
        precision "f64", "f32" (SIMT chains) or "split" (both products as tensor-core digit
        GEMMs) is the arithmetic of the adjoint chain."""
        prec = {"f64": 0, "f32": 1, "split": 2}[precision]
        lo, up = _i32(lower_levels), _i32(upper_levels)
        g = _f64(dL_dS)
        assert g.size == len(lo) * len(up)
        if dL_dmu is None:
            raise ValueError("dL_dmu: a float64 array of the uploaded dipole piece's size")
        assert dL_dmu.dtype == np.float64 and dL_dmu.flags.c_contiguous
        job = PairJob(jindI, gammaI, jindF, gammaF, len(lo), _p(lo, _ip), len(up), _p(up, _ip))
        st = Stats()
        if filters is not None:   # degenerate symmetries: every passing component pair
            check(lib().gain_adjoint_pair_degenerate(self.h, ctypes.byref(job), ctypes.byref(filters), _p(g, _dp),
                                                     _p(dL_dmu, _dp), prec, ctypes.byref(st)))
        else:
            check(lib().gain_adjoint_pair_prec(self.h, ctypes.byref(job), _p(g, _dp), _p(dL_dmu, _dp), prec,
                                               ctypes.byref(st)))
        self.last_adjoint_stats = st
        self._shape = (len(lo), len(up))
        return dL_dmu

    def lines_wait(self) -> int:
        """Wait for the copies of the last asynchronous lines call; returns its n_lines."""
        check(lib().gain_lines_wait(self.h))
        pend = getattr(self, "_pending_lines", None)
        self._pending_lines = None
        return pend[0].value if pend else 0

    def threshold_refined(self) -> int:
        """Lines the last line assembly / text call recomputed in FP64 because their A lay
        within its certified bound of THRESH_LINE."""
        n = ctypes.c_longlong()
        check(lib().gain_lines_threshold_refined(self.h, ctypes.byref(n)))
        return n.value

    def intensity_host(self) -> int:
        """Lines of the last text call whose intensity was evaluated on the host."""
        n = ctypes.c_longlong()
        check(lib().gain_lines_intensity_host(self.h, ctypes.byref(n)))
        return n.value

    def amp_device(self):
        p, ld = ctypes.c_void_p(), ctypes.c_int()
        check(lib().gain_pair_amp_device(self.h, ctypes.byref(p), ctypes.byref(ld)))
        return p.value, ld.value

    def fetch_amp(self, out: Optional[np.ndarray] = None) -> np.ndarray:
        if out is None:
            out = np.empty(self._shape, np.float64)
        assert out.dtype == np.float64 and out.flags.c_contiguous and out.size == self._shape[0] * self._shape[1]
        check(lib().gain_fetch_amp(self.h, _p(out, _dp)))
        return out.reshape(self._shape)

    def lines(self, eI, eF, jI, jF, temperature=296.0, q_part=1.0, zpe=0.0, thresh=0.0,
              freq=(-1e9, 1e9), gnsF=1.0, intensity=True, want=("S", "A", "I", "keep"),
              out_S=None, out_A=None, ndeg=(1, 1), reduced=False, asynchronous=False):
        """S, A (and I, keep) of the last run; out_S / out_A may be preallocated (e.g. pinned)
        contiguous float64 arrays of nlower*nupper elements.  ndeg=(ndegI, ndegF) above 1
        combines the component slots of the last job.  asynchronous=True queues the copies
        (gain_pair_lines_async): the arrays and n_lines are complete after lines_wait()."""
        eI, eF = _f64(eI), _f64(eF)
        n = self._shape[0] * self._shape[1]
        prm = LineParams(temperature, q_part, zpe, thresh, freq[0], freq[1], gnsF, ndeg[0], ndeg[1], int(reduced))
        S = (out_S.reshape(-1) if out_S is not None else np.empty(n)) if "S" in want else None
        A = (out_A.reshape(-1) if out_A is not None else np.empty(n)) if "A" in want else None
        I = np.empty(n) if (intensity and "I" in want) else None
        K = np.empty(n, np.uint8) if "keep" in want else None
        nl = ctypes.c_longlong()
        fn = lib().gain_pair_lines_async if asynchronous else lib().gain_pair_lines
        if asynchronous:
            self._pending_lines = (nl, eI, eF)   # kept alive until the copies land
        check(fn(self.h, ctypes.byref(prm), _p(eI, _dp), _p(eF, _dp), jI, jF,
                                    _p(S, _dp) if S is not None else None,
                                    _p(A, _dp) if A is not None else None,
                                    _p(I, _dp) if I is not None else None,
                                    K.ctypes.data_as(ctypes.POINTER(ctypes.c_ubyte)) if K is not None else None,
                                    ctypes.byref(nl)))
        shp = self._shape
        return {"S": None if S is None else S.reshape(shp), "A": None if A is None else A.reshape(shp),
                "I": None if I is None else I.reshape(shp), "keep": None if K is None else K.reshape(shp),
                "n_lines": nl.value}


def _lines_text(self, eI, eF, jI, jF, gammaI, gammaF, temperature=296.0, q_part=1.0, zpe=0.0, thresh=0.0,
                freq=(-1e9, 1e9), gnsF=1.0, intensity=True, amplitudes=False, out=None, ndeg=(1, 1),
                reduced=False):
    """The line-list text of the last run, built on the device (gain_pair_lines_text) and
    copied into out (a uint8 array of at least the text's size, e.g. pinned) or a new bytes
    object.  Returns (text, n_lines)."""
    eI, eF = _f64(eI), _f64(eF)
    prm = LineParams(temperature, q_part, zpe, thresh, freq[0], freq[1], gnsF, ndeg[0], ndeg[1], int(reduced))
    nb, nl = ctypes.c_ulonglong(), ctypes.c_longlong()
    flags = (TEXT_INTENSITY if intensity else 0) | (TEXT_AMPLITUDES if amplitudes else 0)
    check(lib().gain_pair_lines_text(self.h, ctypes.byref(prm), _p(eI, _dp), _p(eF, _dp), jI, jF, gammaI, gammaF,
                                     flags, ctypes.byref(nb), ctypes.byref(nl)))
    if out is None:
        buf = np.empty(max(1, nb.value), np.uint8)
        check(lib().gain_fetch_lines_text(self.h, buf.ctypes.data, buf.size))
        return buf[:nb.value].tobytes(), nl.value
    assert out.dtype == np.uint8 and out.flags.c_contiguous and out.size >= nb.value
    check(lib().gain_fetch_lines_text(self.h, out.ctypes.data, out.size))
    return memoryview(out)[:nb.value], nl.value


def _lines_text_host(self, eI, eF, jI, jF, gammaI, gammaF, out, temperature=296.0, q_part=1.0, zpe=0.0,
                     thresh=0.0, freq=(-1e9, 1e9), gnsF=1.0, intensity=True, amplitudes=False, ndeg=(1, 1),
                     reduced=False):
    """gain_pair_lines_text_host: the text formed on the device and copied into out (a uint8
    array, page-locked for the overlap) part by part.  Returns (text view, n_lines)."""
    eI, eF = _f64(eI), _f64(eF)
    assert out.dtype == np.uint8 and out.flags.c_contiguous
    prm = LineParams(temperature, q_part, zpe, thresh, freq[0], freq[1], gnsF, ndeg[0], ndeg[1], int(reduced))
    nb, nl = ctypes.c_ulonglong(), ctypes.c_longlong()
    flags = (TEXT_INTENSITY if intensity else 0) | (TEXT_AMPLITUDES if amplitudes else 0)
    check(lib().gain_pair_lines_text_host(self.h, ctypes.byref(prm), _p(eI, _dp), _p(eF, _dp), jI, jF, gammaI,
                                          gammaF, flags, out.ctypes.data, out.size, ctypes.byref(nb),
                                          ctypes.byref(nl)))
    return memoryview(out)[:nb.value], nl.value


JOB_DONE_FN = ctypes.CFUNCTYPE(None, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int)


def run_plan(engines, jobs, path=PATH_SPLIT, tol=0.0, on_done=None):
    """gain_run_plan: jobs = [(jindI, gammaI, jindF, gammaF, lower_levels, upper_levels)] over
    the engines (each holding the uploads the jobs need).  on_done(job, engine, status) runs in
    the worker's thread after each job (the engine's amplitudes are that job's meanwhile; the
    engine argument is the matching Engine).  Returns the per-job stats dicts."""
    keep = []
    arr = (PairJob * max(1, len(jobs)))()
    for i, (jI, gI, jF, gF, lo, up) in enumerate(jobs):
        lo, up = _i32(lo), _i32(up)
        keep += [lo, up]
        arr[i] = PairJob(jI, gI, jF, gF, len(lo), _p(lo, _ip), len(up), _p(up, _ip))
    hs = (_vp * len(engines))(*[e.h for e in engines])
    by_handle = {(e.h.value if isinstance(e.h, ctypes.c_void_p) else e.h): e for e in engines}
    st = (Stats * max(1, len(jobs)))()
    cb = JOB_DONE_FN(0)
    errors = []
    if on_done is not None:
        def _done(user, job, eh, status):
            eng = by_handle[eh]
            lo_n, up_n = arr[job].nlower, arr[job].nupper
            eng._shape = (lo_n, up_n)
            try:
                on_done(job, eng, status)
            except Exception as exc:   # never raise through the C frames
                errors.append(exc)
        cb = JOB_DONE_FN(_done)
    opts = SplitOpts(tol, 0, 0, 0, 0.0)
    check(lib().gain_run_plan(hs, len(engines), arr, len(jobs), path, ctypes.byref(opts), cb, None, st))
    if errors:
        raise errors[0]
    return [st[i].as_dict() for i in range(len(jobs))]


PLAN_AUTOTUNE = 1


class Plan:
    """gain_plan_*: block pairs run as one unit (two grouped tensor-core launches in a CUDA
    graph) on one engine.  jobs = [(jindI, gammaI, jindF, gammaF, lower_levels, upper_levels)]."""

    def __init__(self, eng: "Engine", jobs, tol: float = 0.0, autotune: bool = False, beta: int = 0,
                 slices: int = 0):
        self.eng = eng
        self.shapes = []
        keep = []
        arr = (PairJob * len(jobs))()
        for i, (jI, gI, jF, gF, lo, up) in enumerate(jobs):
            lo, up = _i32(lo), _i32(up)
            keep += [lo, up]
            arr[i] = PairJob(jI, gI, jF, gF, len(lo), _p(lo, _ip), len(up), _p(up, _ip))
            self.shapes.append((len(lo), len(up)))
        opts = SplitOpts(tol, slices, beta, 0, 0.0)
        self.h = _vp()
        check(lib().gain_plan_create(eng.h, arr, len(jobs), ctypes.byref(opts), PLAN_AUTOTUNE if autotune else 0,
                                     ctypes.byref(self.h)))
        self.n = len(jobs)

    def run(self, raise_on_error: bool = True):
        """Replay the plan; returns (plan stats dict, [job stats dicts], status)."""
        js = (Stats * self.n)()
        ps = PlanStats()
        s = lib().gain_plan_run(self.h, js, ctypes.byref(ps))
        if s != OK and raise_on_error:
            check(s)
        return ps.as_dict(), [js[i].as_dict() for i in range(self.n)], s

    def select(self, job: int):
        """Make job's amplitudes the engine's last run (fetch_amp, lines, lines_text...)."""
        check(lib().gain_plan_select(self.h, job))
        self.eng._shape = self.shapes[job]

    def amp(self, job: int) -> np.ndarray:
        self.select(job)
        return self.eng.fetch_amp().copy()

    def close(self):
        if getattr(self, "h", None):
            lib().gain_plan_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


Engine.lines_text = _lines_text
Engine.lines_text_host = _lines_text_host
TEXT_INTENSITY, TEXT_AMPLITUDES = 1, 2


def upload_problem(eng: Engine, p, dipole_block=None, blocks=None):
    """Upload a synth.Problem: bases, expansion tables, dipole piece, eigenvectors."""
    for jind, b in enumerate(p.bases):
        eng.upload_basis(jind, b.J, b.K, b.tau, b.vib, b.kblock, b.kstart)
        inf = p.infl[jind]
        eng.upload_inflation(jind, inf.icontr, inf.ijterms, b.dimen, inf.maxcoeff, inf.matsize, inf.N, inf.repres,
                             inf.Ntot, inf.sdeg)
    nv = p.dipole.shape[-1]
    if dipole_block is None:
        eng.upload_dipole(p.dipole.reshape(-1), nv, 0, nv, nv)
    else:
        s, e = dipole_block
        piece = np.ascontiguousarray(p.dipole[:, :, s:e])
        eng.upload_dipole(piece.reshape(-1), nv, s, e, e - s)
    for (jind, g), blk in p.blocks.items():
        if blocks is None or (jind, g) in blocks:
            eng.upload_eigvecs(jind, g, blk.vecs)
    if p.rule == "c4r":   # rotational-symmetry form: the Wigner table of every |dJ| <= 1 pair
        import synth
        for jI, bI in enumerate(p.bases):
            for jF, bF in enumerate(p.bases):
                if abs(bF.J - bI.J) <= 1:
                    eng.upload_wigner(jI, jF, synth.rotsym_levels(bI.J), synth.rotsym_levels(bF.J), 1,
                                      synth.make_wigner(bI.J, bF.J, 1))


# ----------------------------------------------------------------------------- TROVE files
def trove_basis(dirpath: str, J: int, nsym: int, sym_degen, rotsym: bool = False) -> dict:
    """The basis of J read from j0eigen_quanta<J>.chk (with the J=0 file) in dirpath."""
    h = _vp()
    sd = _i32(sym_degen)
    check(lib().gain_trove_basis_read(dirpath.encode(), J, nsym, _p(sd, _ip), int(rotsym), ctypes.byref(h)))
    try:
        j, d, mc, ms = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        Ntot = np.zeros(nsym, np.int32)
        check(lib().gain_trove_basis_info(h, ctypes.byref(j), ctypes.byref(d), ctypes.byref(mc), ctypes.byref(ms),
                                          _p(Ntot, _ip)))
        d, mc = d.value, mc.value
        out = {k: np.zeros(n, np.int32) for k, n in (("K", d), ("tau", d), ("vib", d), ("kblock", J + 1),
                                                      ("kstart", J + 1), ("icontr", 2 * d), ("ijterms", mc * nsym))}
        check(lib().gain_trove_basis_arrays(h, *[_p(out[k], _ip) for k in
                                                 ("K", "tau", "vib", "kblock", "kstart", "icontr", "ijterms")]))
        out["N"], out["repres"] = [], []
        for g in range(nsym):
            N = np.zeros(mc, np.int32)
            R = np.zeros(int(Ntot[g]) * int(sd[g]) * ms.value, np.float64)
            check(lib().gain_trove_basis_repres(h, g, _p(N, _ip), _p(R, _dp)))
            out["N"].append(N)
            out["repres"].append(R)
        out.update(J=j.value, dimen=d, maxcoeff=mc, matsize=ms.value, Ntot=Ntot, sdeg=sd)
        return out
    finally:
        lib().gain_trove_basis_free(h)


def trove_upload_basis(eng: "Engine", jind: int, dirpath: str, J: int, nsym: int, sym_degen, rotsym=False):
    h = _vp()
    sd = _i32(sym_degen)
    check(lib().gain_trove_basis_read(dirpath.encode(), J, nsym, _p(sd, _ip), int(rotsym), ctypes.byref(h)))
    try:
        check(lib().gain_trove_basis_upload(eng.h, jind, h))
    finally:
        lib().gain_trove_basis_free(h)


def trove_dipole(path: str, max_bytes: int = 1 << 62):
    """(ncontr, [(startF, endF, ncontrF, piece[3*ncontr*ncontrF]), ...]) of j0_extfield.chk."""
    h = _vp()
    check(lib().gain_trove_dipole_read(path.encode(), max_bytes, ctypes.byref(h)))
    try:
        n, nb = ctypes.c_int(), ctypes.c_int()
        check(lib().gain_trove_dipole_info(h, ctypes.byref(n), ctypes.byref(nb)))
        pieces = []
        for b in range(nb.value):
            s, e, c, ptr = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), _dp()
            check(lib().gain_trove_dipole_block(h, b, ctypes.byref(s), ctypes.byref(e), ctypes.byref(c),
                                                ctypes.byref(ptr)))
            size = 3 * n.value * c.value
            arr = np.ctypeslib.as_array(ptr, shape=(size,)).copy() if size else np.zeros(0)
            pieces.append((s.value, e.value, c.value, arr))
        return n.value, pieces
    finally:
        lib().gain_trove_dipole_free(h)


def trove_states(dirpath: str, J: int, gamma: int, f: Filters):
    """States of j0eigen_descr<J>_<gamma+1>.chk passing the filters: (structured array, dim_basis)."""
    n, dim = ctypes.c_int(), ctypes.c_int()
    check(lib().gain_trove_states_read(dirpath.encode(), J, gamma, ctypes.byref(f), ctypes.byref(n), None,
                                       ctypes.byref(dim)))
    arr = (TroveState * max(1, n.value))()
    check(lib().gain_trove_states_read(dirpath.encode(), J, gamma, ctypes.byref(f), ctypes.byref(n), arr,
                                       ctypes.byref(dim)))
    dt = np.dtype([("energy", np.float64), ("irec", np.int32), ("ilevel", np.int32), ("krot", np.int32),
                   ("taurot", np.int32), ("rec_len", np.int32)], align=True)
    assert dt.itemsize == ctypes.sizeof(TroveState)
    out = np.frombuffer(bytes(arr), dtype=dt, count=n.value).copy()
    return out, dim.value


def trove_vectors(path: str, rec_len: int, records) -> np.ndarray:
    r = _i32(records)
    out = np.zeros((len(r), rec_len), np.float64)
    check(lib().gain_trove_vectors_read(path.encode(), rec_len, _p(r, _ip), len(r), _p(out, _dp)))
    return out
