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
