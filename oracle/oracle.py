"""ORACLE (test infrastructure only): Python side of the CPU restatement.

* builds and loads the C restatement (gain_oracle.c) through ctypes;
* restates the state-selection rules of BaseClasses/States.cpp:41-116 and the line-list
  text of BaseClasses/Output.cpp:52-112 in plain Python (small loops only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may import this
module, and only as the checker.
"""
from __future__ import annotations

import ctypes
import os
import platform
import subprocess
import sys
from typing import Sequence

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build", platform.machine())
LIB = os.path.join(BUILD, "libgainoracle.so")
# The same source built for speed, used only as the timed CPU baseline: -O3 and the
# compiler's default floating-point contraction (fused multiply-adds where it finds them).
# No -march=native: the same host code must build and behave alike on x86_64 and aarch64.
LIB_FAST = os.path.join(BUILD, "libgainoracle_fast.so")
SRC = os.path.join(HERE, "gain_oracle.c")
FAST_FLAGS = ["-O3", "-fopenmp"]

REF, DD = 0, 1

_lib = None
_lib_fast = None


def _stale(target: str) -> bool:
    return not os.path.exists(target) or os.path.getmtime(target) < max(
        os.path.getmtime(SRC), os.path.getmtime(os.path.join(HERE, "gain_oracle.h")))


def build(force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    if force or _stale(LIB):
        # parity build: no contraction, so every product and sum rounds as written
        cmd = ["gcc", "-O2", "-fPIC", "-shared", "-std=c11", "-ffp-contract=off", "-fopenmp",
               SRC, "-o", LIB + ".tmp", "-lm"]
        subprocess.run(cmd, check=True)
        os.replace(LIB + ".tmp", LIB)
    if force or _stale(LIB_FAST):
        cmd = ["gcc"] + FAST_FLAGS + ["-fPIC", "-shared", "-std=c11", SRC, "-o", LIB_FAST + ".tmp", "-lm"]
        subprocess.run(cmd, check=True)
        os.replace(LIB_FAST + ".tmp", LIB_FAST)
    return LIB


def lib(fast: bool = False):
    """The parity build, or (fast=True) the speed build the CPU baseline times."""
    global _lib, _lib_fast
    if fast:
        if _lib_fast is None:
            build()
            _lib_fast = ctypes.CDLL(LIB_FAST)
            _declare(_lib_fast)
        return _lib_fast
    if _lib is None:
        build()
        _lib = ctypes.CDLL(LIB)
        _declare(_lib)
    return _lib


_ip = ctypes.POINTER(ctypes.c_int)
_dp = ctypes.POINTER(ctypes.c_double)


class OrcPair(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int) for n in ("jI", "jF", "jmax", "dimenI", "dimenF")] + \
        [(n, _ip) for n in ("tauI", "tauF", "icorrI", "icorrF", "kstartI", "kblockI",
                            "kstartF", "kblockF")] + \
        [(n, ctypes.c_int) for n in ("gammaI", "gammaF", "maxcoeffI", "maxcoeffF", "NtotI", "NtotF")] + \
        [("ijtermsI", _ip), ("icontrI", _ip), ("NI", _ip), ("represI", _dp),
         ("ijtermsF", _ip), ("icontrF", _ip), ("NF", _ip), ("represF", _dp),
         ("dipole_me", _dp)] + \
        [(n, ctypes.c_int) for n in ("dip_stride", "startFblock", "endFblock", "ncontrF")] + \
        [("threej", _dp), ("nlower", ctypes.c_int), ("nupper", ctypes.c_int),
         ("vec_lower", _dp), ("vec_upper", _dp)] + \
        [(n, ctypes.c_int) for n in ("idegI", "idegF", "sdegI", "sdegF")]


def _declare(L):
    I, D = ctypes.c_int, ctypes.c_double
    L.orc_hls_kblock.argtypes = [I, I, I, I, I, _ip, _ip, _ip, _ip, I, I, I, I, I, _ip, _dp, I,
                                 _dp, _dp, I, _dp, I]
    L.orc_hls_kblock.restype = None
    L.orc_half_ls.argtypes = [I, I, I, I, _ip, _ip, _ip, _ip, _ip, _ip, _ip, _ip, I, I, I, _dp, I,
                              _dp, _dp, I, _dp, I]
    L.orc_half_ls.restype = None
    L.orc_hls_rotsym.argtypes = [I, I, I, I, I, _ip, _ip, _ip, _ip, _ip, _ip, I, I, I, _dp, I, _dp, _dp,
                                 _dp, I]
    L.orc_hls_rotsym.restype = None
    L.orc_expand.argtypes = [I, I, I, I, I, I, _ip, _ip, _ip, _dp, _dp, _dp, I]
    L.orc_expand.restype = None
    L.orc_dot.argtypes = [I, _dp, _dp, I]
    L.orc_dot.restype = D
    L.orc_run_pair.argtypes = [ctypes.POINTER(OrcPair), I, I, _dp]
    L.orc_run_pair.restype = I
    L.orc_line.argtypes = [_dp, ctypes.POINTER(ctypes.c_ubyte), I, I, I, I, D, D, D, I, I, D, D, D,
                           D, _dp, _dp, _dp]
    L.orc_line.restype = I
    L.orc_line_list.argtypes = [I, I, _dp, ctypes.c_long, _dp, _dp, _ip, _ip, I, I, I, I, D, D, D, D, D, D, D, I,
                                I, ctypes.c_char_p, ctypes.c_longlong, ctypes.POINTER(ctypes.c_longlong)]
    L.orc_line_list.restype = ctypes.c_longlong


def _i(a):
    a = np.ascontiguousarray(a, np.int32)
    return a, a.ctypes.data_as(_ip)


def _d(a):
    a = np.ascontiguousarray(a, np.float64)
    return a, a.ctypes.data_as(_dp)


# ----------------------------------------------------------------------------- kernels

def hls_kblock(dimenF, dimenI, jI, jF, kF, tauI, tauF, icorrI, icorrF, startF_idx, startI_idx,
               startFblock, endFblock, ncontrF, kblock_size, dipole_me, dip_stride, vector,
               threej, jmax, half_ls, mode=REF):
    keep = []
    args = []
    for a in (tauI, tauF, icorrI, icorrF):
        arr, p = _i(a); keep.append(arr); args.append(p)
    kb, kbp = _i(kblock_size)
    dm, dmp = _d(dipole_me)
    vec, vecp = _d(vector)
    tj, tjp = _d(threej)
    assert half_ls.dtype == np.float64 and half_ls.flags.c_contiguous
    lib().orc_hls_kblock(dimenF, dimenI, jI, jF, kF, *args, startF_idx, startI_idx, startFblock,
                         endFblock, ncontrF, kbp, dmp, dip_stride, vecp, tjp, jmax,
                         half_ls.ctypes.data_as(_dp), mode)
    return half_ls


def hls_rotsym(bI, bF, nlevelI, nlevelF, maxdeg, dipole_piece, dip_stride, block, wigner, vector,
               half_ls, mode=REF):
    """Rotsym half_ls of one primitive lower vector (synth.Basis inputs, rotsym field meaning:
    K = degeneracy index, tau = level index); entries outside the dipole block untouched."""
    startF, endF, ncontrF = block
    keep = []

    def I(a):
        arr, p = _i(a); keep.append(arr); return p

    def D(a):
        arr, p = _d(a); keep.append(arr); return p

    assert half_ls.dtype == np.float64 and half_ls.flags.c_contiguous and half_ls.size >= bF.dimen
    lib().orc_hls_rotsym(bF.dimen, bI.dimen, nlevelI, nlevelF, maxdeg, I(bI.K), I(bF.K), I(bI.tau), I(bF.tau),
                         I(bI.vib), I(bF.vib), startF, endF, ncontrF, D(dipole_piece), dip_stride, D(wigner),
                         D(vector), half_ls.ctypes.data_as(_dp), mode)
    return half_ls


def half_ls(bI, bF, prim_vec, dipole, threej, jmax, mode=REF, block=None):
    """Whole half_ls (dimen of J') for one primitive lower vector (synth.Basis inputs)."""
    nv = dipole.shape[-1]
    startF, endF, ncontrF = block if block is not None else (0, nv, nv)
    out = np.zeros(bF.dimen, np.float64)
    keep = [_i(x) for x in (bI.tau, bF.tau, bI.vib, bF.vib, bI.kstart, bI.kblock, bF.kstart,
                            bF.kblock)]
    dm, dmp = _d(dipole.reshape(-1))
    pv, pvp = _d(prim_vec)
    tj, tjp = _d(threej)
    lib().orc_half_ls(bI.J, bF.J, bI.dimen, bF.dimen, *[k[1] for k in keep], startF, endF,
                      ncontrF, dmp, nv, pvp, tjp, jmax, out.ctypes.data_as(_dp), mode)
    return out


def expand(infl, gamma, vec_sym, ideg=0, mode=REF):
    dimen = infl.icontr.shape[0] // 2
    out = np.zeros(dimen, np.float64)
    ij, ijp = _i(infl.ijterms)
    ic, icp = _i(infl.icontr)
    N, Np = _i(infl.N[gamma])
    rp, rpp = _d(infl.repres[gamma])
    v, vp = _d(vec_sym)
    lib().orc_expand(dimen, gamma, infl.maxcoeff, ideg, int(infl.sdeg[gamma]),
                     int(infl.Ntot[gamma]), ijp, icp, Np, rpp, vp, out.ctypes.data_as(_dp), mode)
    return out


def dot(x, y, mode=REF):
    a, ap = _d(x)
    b, bp = _d(y)
    return lib().orc_dot(a.shape[0], ap, bp, mode)


def run_pair(problem, jindI, gammaI, jindF, gammaF, lower_levels: Sequence[int],
             upper_levels: Sequence[int], threej, jmax, mode=REF, nthreads=1,
             dipole_block=None, components=(0, 0), fast=False):
    """amp[l, u] through the reference's plain loop order for one block pair.

    lower_levels / upper_levels are level indices inside the (J, Gamma) blocks; components =
    (idegI, idegF), the degenerate components of the lower and upper vectors.  fast=True runs
    the speed build (the CPU baseline's timing only; its roundings may differ)."""
    p = problem
    bI, bF = p.bases[jindI], p.bases[jindF]
    iI, iF = p.infl[jindI], p.infl[jindF]
    vl = np.ascontiguousarray(p.blocks[(jindI, gammaI)].vecs[np.asarray(lower_levels, int)])
    vu = np.ascontiguousarray(p.blocks[(jindF, gammaF)].vecs[np.asarray(upper_levels, int)])
    nv = p.dipole.shape[-1]
    startF, endF = dipole_block if dipole_block is not None else (0, nv)
    ncontrF = endF - startF
    keep = []

    def I(a):
        arr, ptr = _i(a); keep.append(arr); return ptr

    def D(a):
        arr, ptr = _d(a); keep.append(arr); return ptr

    s = OrcPair()
    s.jI, s.jF, s.jmax = bI.J, bF.J, jmax
    s.dimenI, s.dimenF = bI.dimen, bF.dimen
    s.tauI, s.tauF, s.icorrI, s.icorrF = I(bI.tau), I(bF.tau), I(bI.vib), I(bF.vib)
    s.kstartI, s.kblockI, s.kstartF, s.kblockF = I(bI.kstart), I(bI.kblock), I(bF.kstart), I(bF.kblock)
    s.gammaI, s.gammaF = gammaI, gammaF
    s.maxcoeffI, s.maxcoeffF = iI.maxcoeff, iF.maxcoeff
    s.NtotI, s.NtotF = int(iI.Ntot[gammaI]), int(iF.Ntot[gammaF])
    s.ijtermsI, s.icontrI, s.NI, s.represI = I(iI.ijterms), I(iI.icontr), I(iI.N[gammaI]), D(iI.repres[gammaI])
    s.ijtermsF, s.icontrF, s.NF, s.represF = I(iF.ijterms), I(iF.icontr), I(iF.N[gammaF]), D(iF.repres[gammaF])
    piece = p.dipole if dipole_block is None else np.ascontiguousarray(p.dipole[:, :, startF:endF])
    s.dipole_me = D(piece.reshape(-1))
    s.dip_stride, s.startFblock, s.endFblock, s.ncontrF = nv, startF, endF, ncontrF
    s.threej = D(threej)
    s.nlower, s.nupper = vl.shape[0], vu.shape[0]
    s.vec_lower, s.vec_upper = D(vl), D(vu)
    s.idegI, s.idegF = int(components[0]), int(components[1])
    s.sdegI, s.sdegF = int(iI.sdeg[gammaI]), int(iF.sdeg[gammaF])
    amp = np.zeros((vl.shape[0], vu.shape[0]), np.float64)
    rc = lib(fast).orc_run_pair(ctypes.byref(s), nthreads, mode, amp.ctypes.data_as(_dp))
    if rc != 0:
        raise MemoryError("oracle run_pair failed")
    return amp


# ------------------------------------------------------------------- selection rules
class Filters:
    """The intensity-block parameters (TroveClasses/TroveInput.cpp:239-326) the filters read."""

    def __init__(self, jvals, gns, isym_pairs, igamma_pair, sym_degen, erange_lower,
                 erange_upper, freq_window=(-1e9, 1e9), zpe=0.0, reduced=False,
                 symmetry_type=1, temperature=296.0, q_part=1.0, thresh=0.0):
        self.gns = list(map(float, gns))
        self.isym_do = [g >= 1e-15 for g in self.gns]      # TroveInput.cpp:300-304
        self.isym_pairs = list(isym_pairs)
        self.igamma_pair = list(igamma_pair)
        self.sym_degen = list(sym_degen)
        self.erange_lower = tuple(erange_lower)
        self.erange_upper = tuple(erange_upper)
        self.freq_window = tuple(freq_window)
        self.zpe = zpe
        self.reduced = reduced
        self.symmetry_type = symmetry_type
        self.maxJ = max(jvals)
        self.temperature = temperature
        self.q_part = q_part
        self.thresh = thresh

    # States.cpp:46-53
    def filter_lower(self, energy, g):
        return (energy - self.zpe) <= self.erange_lower[1] and \
            (energy - self.zpe) >= self.erange_lower[0] and self.isym_do[g]

    def filter_upper(self, energy, g):
        return (energy - self.zpe) <= self.erange_upper[1] and \
            (energy - self.zpe) >= self.erange_upper[0] and self.isym_do[g]

    # States.cpp:54-76
    def filter_intensity(self, eI, gI, jI, eF, gF, jF):
        nu = eF - eI
        return (self.gns[gI] > 0.0 and self.gns[gF] > 0.0 and
                nu >= self.freq_window[0] and nu <= self.freq_window[1] and
                self.filter_lower(eI, gI) and self.filter_upper(eF, gF) and
                (jF != self.maxJ or jI != self.maxJ) and
                self.isym_pairs[gI] == self.isym_pairs[gF] and
                self.igamma_pair[gI] == gF and abs(jF - jI) <= 1 and jI + jF >= 1)

    # States.cpp:95-116
    def degeneracy_filter(self, gI, gF, idegI, idegF):
        if self.sym_degen[gI] == 1 or self.sym_degen[gF] == 1:
            return True
        if not self.reduced:
            return True
        if self.symmetry_type == 1:
            return True
        if self.symmetry_type == 2:
            return idegI == 1 and idegF == 0
        if self.symmetry_type == 3:
            if gI == 3 and gF == 4 and idegI == 1 and idegF == 0:
                return True
            if gI == 4 and gF == 3 and idegI == 2 and idegF == 0:
                return True
            if gI == 2 and gF == 2 and idegI == 1 and idegF == 0:
                return True
        return False


def transitions(problem, flt: Filters):
    """(I, F) global state pairs in the reference's order (main.cpp:238-296, one rank)."""
    p = problem
    out = []
    n = len(p.st_energy)
    for I in range(n):
        if not flt.filter_lower(p.st_energy[I], p.st_gamma[I]):
            continue
        for F in range(n):
            if F == I:
                continue
            if flt.filter_intensity(p.st_energy[I], p.st_gamma[I], p.st_J[I],
                                    p.st_energy[F], p.st_gamma[F], p.st_J[F]):
                out.append((I, F))
    return out


def line(amp_slots, degmask, maxdeg, ndegI, ndegF, flt: Filters, eI, eF, jI, jF, gF):
    a, ap = _d(amp_slots)
    m = np.ascontiguousarray(degmask, np.uint8)
    S, A, Iv = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
    ok = lib().orc_line(ap, m.ctypes.data_as(ctypes.POINTER(ctypes.c_ubyte)), maxdeg, ndegI, ndegF,
                        int(flt.reduced), eI, eF, flt.zpe, jI, jF, flt.gns[gF], flt.temperature,
                        flt.q_part, flt.thresh, ctypes.byref(S), ctypes.byref(A), ctypes.byref(Iv))
    return (S.value, A.value, Iv.value) if ok else None


def line_list(amp, eI, eF, levI, levF, jI, jF, gI, gF, gnsF=1.0, temperature=296.0, q_part=1.0, zpe=0.0,
              thresh=0.0, freq=(-1e9, 1e9), intensity=True, amplitudes=False):
    """(text bytes, n_lines) of one block pair as the reference writes it (orc_line_list)."""
    a, ap = _d(amp)
    rows, cols = a.shape
    ei, eip = _d(eI)
    ef, efp = _d(eF)
    li, lip = _i(levI)
    lf, lfp = _i(levF)
    nl = ctypes.c_longlong()
    args = (rows, cols, ap, cols, eip, efp, lip, lfp, jI, jF, gI, gF, gnsF, temperature, q_part, zpe, thresh,
            freq[0], freq[1], int(intensity), int(amplitudes))
    n = lib().orc_line_list(*args, None, 0, ctypes.byref(nl))
    buf = ctypes.create_string_buffer(max(1, n))
    lib().orc_line_list(*args, buf, n, ctypes.byref(nl))
    return buf.raw[:n], nl.value


def line_text(nu, indexF, jF, gF, indexI, jI, gI, A, intens=None, amps=None):
    """Output.cpp:99-111 text of one line."""
    s = "%12.6f %8d %4d %4d <- %8d %4d %4d %16.9E " % (nu, indexF + 1, jF, gF + 1, indexI + 1,
                                                        jI, gI + 1, A)
    if intens is not None:
        s += "%16.9E " % intens
    if amps is not None:
        s += "[ %s ] " % "".join(" %16.9E" % x for x in amps)
    return s + " || \n"   # fprintf(output, "%s || \n", buffer), Output.cpp:111
