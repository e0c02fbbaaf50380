"""The C++ host mirror of GpuManager (include/gain_gpu_manager.hpp), driven by a
main.cpp-style loop (tests/cpp/manager_driver.cpp), against the reference kernels' golden
amplitudes."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, ROOT

pytestmark = pytest.mark.gpu


def _write_input(path, d):
    import synth
    nv, jvals, rule = int(d["nv"]), [int(x) for x in d["jvals"]], str(d["rule"])
    JI, JF, gI, gF = int(d["JI"]), int(d["JF"]), int(d["gI"]), int(d["gF"])
    s, e = (int(x) for x in d["block"])
    nsym = synth.nsym_of(rule)
    ints = [nv, int(d["jmax"]), nsym, JI, JF, gI, gF, d["vec_lower"].shape[0], d["vec_upper"].shape[0], s, e]
    with open(path, "wb") as f:
        f.write(np.asarray(ints, np.int32).tobytes())
        for J in (JI, JF):
            b = synth.make_basis(J, nv)
            inf = synth.make_inflation(b, synth.classes_of(b, rule), nsym)
            f.write(np.asarray([b.dimen], np.int32).tobytes())
            for a in (b.K, b.tau, b.vib, b.kblock, b.kstart, inf.icontr, inf.ijterms):
                f.write(np.ascontiguousarray(a, np.int32).tobytes())
            for g in range(nsym):
                f.write(np.ascontiguousarray(inf.N[g], np.int32).tobytes())
            f.write(np.ascontiguousarray(inf.Ntot, np.int32).tobytes())
        f.write(np.ascontiguousarray(d["dipole"][:, :, s:e]).tobytes())
        f.write(np.ascontiguousarray(d["vec_lower"]).tobytes())
        f.write(np.ascontiguousarray(d["vec_upper"]).tobytes())


@pytest.fixture(scope="module")
def driver(built_lib, tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    out = str(tmp_path_factory.mktemp("drv") / "manager_driver")
    lib = os.path.join(ROOT, "gain-mpi_gb300", "lib")
    subprocess.run([nvcc, "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "manager_driver.cpp"), "-o", out, "-L", lib, "-lgainls",
                    "-Xlinker", "-rpath", "-Xlinker", lib], check=True)
    return out


def _write_rotsym_input(path, p, jI, gI, jF, gF, nlower, nupper, block):
    """A rotsym block pair of a synth problem (rule c4r), with the Wigner table record."""
    import synth
    bI, bF = p.bases[jI], p.bases[jF]
    s, e = block
    nv = p.dipole.shape[-1]
    ints = [nv, 11, p.nsym, bI.J, bF.J, gI, gF, nlower, nupper, s, e]
    with open(path, "wb") as f:
        f.write(np.asarray(ints, np.int32).tobytes())
        for jind in (jI, jF):
            b, inf = p.bases[jind], p.infl[jind]
            f.write(np.asarray([b.dimen], np.int32).tobytes())
            for a in (b.K, b.tau, b.vib, b.kblock, b.kstart, inf.icontr, inf.ijterms):
                f.write(np.ascontiguousarray(a, np.int32).tobytes())
            for g in range(p.nsym):
                f.write(np.ascontiguousarray(inf.N[g], np.int32).tobytes())
            f.write(np.ascontiguousarray(inf.Ntot, np.int32).tobytes())
        f.write(np.ascontiguousarray(p.dipole[:, :, s:e]).tobytes())
        f.write(np.ascontiguousarray(p.blocks[(jI, gI)].vecs[:nlower]).tobytes())
        f.write(np.ascontiguousarray(p.blocks[(jF, gF)].vecs[:nupper]).tobytes())
        nI, nF = synth.rotsym_levels(bI.J), synth.rotsym_levels(bF.J)
        f.write(np.asarray([1, nI, nF], np.int32).tobytes())
        f.write(np.ascontiguousarray(synth.make_wigner(bI.J, bF.J, 1)).tobytes())


@pytest.mark.parametrize("block", [None, (3, 10)])
def test_manager_rotsym_loop_matches_oracle(driver, tmp_path, block):
    """GpuManager(rotsym=true): TransferWigner after each basis set, ExecuteHalfLs through the
    rotsym drop-in, against the oracle's reference-order restatement of the same loop."""
    import oracle
    import synth
    p = synth.make_problem(12, [2, 3], "c4r", blocks=[(2, 0), (3, 1)])
    blk = block or (0, 12)
    nlower, nupper = 6, 12
    inp, outp = str(tmp_path / "in.bin"), str(tmp_path / "out.bin")
    _write_rotsym_input(inp, p, 0, 0, 1, 1, nlower, nupper, blk)
    subprocess.run([driver, inp, outp], check=True, timeout=120)
    amp = np.fromfile(outp, np.float64).reshape(nlower, nupper)
    bI, bF, iI, iF = p.bases[0], p.bases[1], p.infl[0], p.infl[1]
    s, e = blk
    piece = np.ascontiguousarray(p.dipole[:, :, s:e]).reshape(-1)
    wig = synth.make_wigner(bI.J, bF.J, 1)
    ref = np.zeros_like(amp)
    for l in range(nlower):
        prim = oracle.expand(iI, 0, p.blocks[(0, 0)].vecs[l])
        h = np.zeros(bF.dimen)
        oracle.hls_rotsym(bI, bF, synth.rotsym_levels(bI.J), synth.rotsym_levels(bF.J), 1, piece, 12, (s, e, e - s),
                          wig, prim, h)
        for u in range(nupper):
            ref[l, u] = oracle.dot(oracle.expand(iF, 1, p.blocks[(1, 1)].vecs[u]), h)
    assert np.max(np.abs(amp - ref)) <= 1e-14 * np.abs(ref).max()


@pytest.mark.parametrize("name", ["c4_dJp1", "c4_dJm1", "full_blocked", "c4_highJ"])
def test_manager_loop_matches_reference(driver, tmp_path, name):
    d = np.load(os.path.join(GOLDEN, name + ".npz"))
    inp, outp = str(tmp_path / "in.bin"), str(tmp_path / "out.bin")
    _write_input(inp, d)
    subprocess.run([driver, inp, outp], check=True, timeout=120)
    amp = np.fromfile(outp, np.float64).reshape(d["ref_amp"].shape)
    ref = d["ref_amp"]
    # same half_ls bits as the reference; the dot's summation order differs from cublasDdot
    assert np.max(np.abs(amp - ref)) <= 1e-14 * np.abs(ref).max() + 1e-300


@pytest.mark.parametrize("nblocks", [2, 3])
def test_manager_dipole_blocks_match_reference(driver, tmp_path, nblocks):
    """The dipole split into blocks (TroveDipole's pieces), SwitchDipoleBlock between the
    half line strength calls of each lower state (MultiGpuManager.cpp:240-262): the same
    golden amplitudes as the whole dipole (each block writes its own upper functions)."""
    d = np.load(os.path.join(GOLDEN, "c4_dJp1.npz"))
    nv = int(d["nv"])
    assert tuple(int(x) for x in d["block"]) == (0, nv)
    inp, outp = str(tmp_path / "in.bin"), str(tmp_path / "out.bin")
    _write_input(inp, d)
    subprocess.run([driver, inp, outp, str(nblocks)], check=True, timeout=120)
    amp = np.fromfile(outp, np.float64).reshape(d["ref_amp"].shape)
    ref = d["ref_amp"]
    assert np.max(np.abs(amp - ref)) <= 1e-14 * np.abs(ref).max() + 1e-300
