"""ORACLE (test infrastructure only): Python side of ref_harness.cu.

Runs the reference's own unmodified kernels (oracle/_ref/dipole_GPU.cubin, compiled from
the reference tree by oracle/build_ref.sh) on the GPU, driven like GpuManager drives them.
Used to make golden fixtures and to pin the oracle; never part of the product path.
"""
from __future__ import annotations

import ctypes
import os
import platform
import shutil
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build", platform.machine())
LIB = os.path.join(BUILD, "libgainrefh.so")
SRC = os.path.join(HERE, "ref_harness.cu")
CUBIN = os.path.join(HERE, "_ref", "dipole_GPU.cubin")

_lib = None
_ip = ctypes.POINTER(ctypes.c_int)
_dp = ctypes.POINTER(ctypes.c_double)


class RefhPair(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int) for n in ("jI", "jF", "jmax", "dimenI", "dimenF")] + \
        [(n, _ip) for n in ("tauI", "tauF", "icorrI", "icorrF", "kstartI", "kblockI", "kstartF", "kblockF")] + \
        [(n, ctypes.c_int) for n in ("gammaI", "gammaF", "maxcoeffI", "maxcoeffF", "NtotI", "NtotF",
                                     "nsymI", "nsymF", "matsizeI", "matsizeF")] + \
        [("ijtermsI", _ip), ("icontrI", _ip), ("NI", _ip), ("represI", _dp),
         ("ijtermsF", _ip), ("icontrF", _ip), ("NF", _ip), ("represF", _dp), ("dipole_me", _dp)] + \
        [(n, ctypes.c_int) for n in ("dip_stride", "startFblock", "endFblock", "ncontrF")] + \
        [("threej", _dp), ("nlower", ctypes.c_int), ("nupper", ctypes.c_int), ("vec_lower", _dp),
         ("vec_upper", _dp)] + \
        [(n, ctypes.c_int) for n in ("idegI", "idegF", "sdegI", "sdegF")]


def available() -> bool:
    return os.path.exists(CUBIN)


def build() -> str:
    os.makedirs(BUILD, exist_ok=True)
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(SRC):
        nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
        cmd = [nvcc, "-O2", "-shared", "-Xcompiler", "-fPIC", SRC, "-o", LIB + ".tmp", "-lcublas", "-lcuda"]
        stub = "/usr/local/cuda/lib64/stubs"
        if os.path.isdir(stub):
            cmd += ["-L", stub]
        subprocess.run(cmd, check=True)
        os.replace(LIB + ".tmp", LIB)
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        L.refh_init.argtypes = [ctypes.c_char_p]
        L.refh_init.restype = ctypes.c_int
        L.refh_error.restype = ctypes.c_char_p
        L.refh_run_pair.argtypes = [ctypes.POINTER(RefhPair), _dp, _dp, _dp]
        L.refh_run_pair.restype = ctypes.c_int
        I = ctypes.c_int
        L.refh_hls_rotsym.argtypes = [I, I, I, I, I, _ip, _ip, _ip, _ip, _ip, _ip, I, I, I, _dp, I, _dp, _dp, _dp]
        L.refh_hls_rotsym.restype = ctypes.c_int
        if L.refh_init(CUBIN.encode()) != 0:
            raise RuntimeError("reference harness: " + L.refh_error().decode())
        _lib = L
    return _lib


def run_pair(problem, jindI, gammaI, jindF, gammaF, lower_levels, upper_levels, threej, jmax,
             dipole_block=None, vec_lower=None, vec_upper=None, components=(0, 0)):
    """(amp [nl, nu], half_ls [nl, dimenF], seconds of the per-transition loop); components =
    (idegI, idegF), the degenerate components the expansions take."""
    p = problem
    bI, bF = p.bases[jindI], p.bases[jindF]
    iI, iF = p.infl[jindI], p.infl[jindF]
    vl = vec_lower if vec_lower is not None else p.blocks[(jindI, gammaI)].vecs[np.asarray(lower_levels, int)]
    vu = vec_upper if vec_upper is not None else p.blocks[(jindF, gammaF)].vecs[np.asarray(upper_levels, int)]
    vl = np.ascontiguousarray(vl, np.float64)
    vu = np.ascontiguousarray(vu, np.float64)
    nv = p.dipole.shape[-1]
    if dipole_block is None:
        startF, endF = 0, nv
        piece = np.ascontiguousarray(p.dipole)
    else:
        startF, endF = dipole_block
        piece = np.ascontiguousarray(p.dipole[:, :, startF:endF])
    keep = []

    def I(a):
        a = np.ascontiguousarray(a, np.int32); keep.append(a); return a.ctypes.data_as(_ip)

    def D(a):
        a = np.ascontiguousarray(a, np.float64); keep.append(a); return a.ctypes.data_as(_dp)

    s = RefhPair()
    s.jI, s.jF, s.jmax, s.dimenI, s.dimenF = bI.J, bF.J, jmax, bI.dimen, bF.dimen
    s.tauI, s.tauF, s.icorrI, s.icorrF = I(bI.tau), I(bF.tau), I(bI.vib), I(bF.vib)
    s.kstartI, s.kblockI, s.kstartF, s.kblockF = I(bI.kstart), I(bI.kblock), I(bF.kstart), I(bF.kblock)
    s.gammaI, s.gammaF = gammaI, gammaF
    s.maxcoeffI, s.maxcoeffF = iI.maxcoeff, iF.maxcoeff
    s.NtotI, s.NtotF = int(iI.Ntot[gammaI]), int(iF.Ntot[gammaF])
    s.nsymI, s.nsymF = len(iI.N), len(iF.N)
    s.matsizeI, s.matsizeF = int(getattr(iI, "matsize", 1)), int(getattr(iF, "matsize", 1))
    s.idegI, s.idegF = int(components[0]), int(components[1])
    s.sdegI, s.sdegF = int(iI.sdeg[gammaI]), int(iF.sdeg[gammaF])
    if not (0 <= s.idegI < s.sdegI and 0 <= s.idegF < s.sdegF):
        raise ValueError("components outside the degeneracies")
    # every expansion entry the reference kernel reads lies inside the uploaded tables
    for inf, g, b, ms, sd in ((iI, gammaI, bI, s.matsizeI, s.sdegI), (iF, gammaF, bF, s.matsizeF, s.sdegF)):
        d = b.dimen
        irow, ib = np.asarray(inf.icontr[:d]), np.asarray(inf.icontr[d:2 * d])
        n = np.asarray(inf.N[g])[irow]
        it = np.asarray(inf.ijterms)[irow + g * inf.maxcoeff]
        used = n > 0
        if (np.any(irow < 0) or np.any(irow >= inf.maxcoeff) or np.any(ib[used] >= ms) or np.any(ib < 0)
                or np.any(it[used] + n[used] > int(inf.Ntot[g])) or len(inf.repres[g]) < int(inf.Ntot[g]) * sd * ms):
            raise ValueError("expansion tables outside their ranges")
    s.ijtermsI, s.icontrI, s.NI, s.represI = I(iI.ijterms), I(iI.icontr), I(iI.N[gammaI]), D(iI.repres[gammaI])
    s.ijtermsF, s.icontrF, s.NF, s.represF = I(iF.ijterms), I(iF.icontr), I(iF.N[gammaF]), D(iF.repres[gammaF])
    s.dipole_me = D(piece.reshape(-1))
    s.dip_stride, s.startFblock, s.endFblock, s.ncontrF = nv, startF, endF, endF - startF
    s.threej = D(threej)
    s.nlower, s.nupper = vl.shape[0], vu.shape[0]
    s.vec_lower, s.vec_upper = D(vl), D(vu)
    amp = np.zeros((vl.shape[0], vu.shape[0]), np.float64)
    hls = np.zeros((vl.shape[0], bF.dimen), np.float64)
    secs = ctypes.c_double()
    if lib().refh_run_pair(ctypes.byref(s), amp.ctypes.data_as(_dp), hls.ctypes.data_as(_dp),
                           ctypes.byref(secs)) != 0:
        raise RuntimeError("reference harness: " + lib().refh_error().decode())
    return amp, hls, secs.value


def hls_rotsym(bI, bF, nlevelI, nlevelF, maxdeg, dipole, block, wigner, vector):
    """The reference's rotsym half line strength of one primitive lower vector (dimen of J'),
    zeros outside the dipole block; dipole is the full [3][N][N] flipped array."""
    nv = dipole.shape[-1]
    startF, endF = block
    piece = np.ascontiguousarray(dipole[:, :, startF:endF])
    keep = []

    def I(a):
        a = np.ascontiguousarray(a, np.int32); keep.append(a); return a.ctypes.data_as(_ip)

    def D(a):
        a = np.ascontiguousarray(a, np.float64); keep.append(a); return a.ctypes.data_as(_dp)

    out = np.zeros(bF.dimen, np.float64)
    if lib().refh_hls_rotsym(bF.dimen, bI.dimen, nlevelI, nlevelF, maxdeg, I(bI.K), I(bF.K), I(bI.tau), I(bF.tau),
                             I(bI.vib), I(bF.vib), startF, endF, endF - startF, D(piece.reshape(-1)), nv,
                             D(wigner), D(vector), out.ctypes.data_as(_dp)) != 0:
        raise RuntimeError("reference harness: " + lib().refh_error().decode())
    return out
