"""The C ABI without a GPU: the library loads, exports every declared entry point, rejects
bad arguments on the host with a status (never aborting), and prints lines exactly as the
reference's Output::OutputLinestrength does."""
import ctypes
import os

import numpy as np
import pytest

from conftest import has_gpu


def test_library_exports_every_declared_symbol(built_lib):
    import gainls
    L = gainls.lib()
    names = gainls.declared_symbols()
    assert "gain_hls_kblock" in names and "gain_run_pair" in names
    for n in names:
        assert hasattr(L, n), n
    assert L.gain_abi_version() == 1


def test_status_strings(built_lib):
    import gainls
    L = gainls.lib()
    for s in range(8):
        assert L.gain_status_string(s).decode().startswith("GAIN_")


@pytest.mark.skipif(has_gpu(), reason="checks the no-GPU error path")
def test_engine_without_gpu_reports_status(built_lib):
    import gainls
    with pytest.raises(gainls.GainError) as e:
        gainls.Engine(11, 4, 1)
    assert e.value.status in (gainls.ERR_CUDA, gainls.ERR_INVALID_ARG)


def test_engine_rejects_bad_arguments(built_lib):
    import gainls
    h = ctypes.c_void_p()
    assert gainls.lib().gain_engine_create(0, -1, 4, 1, ctypes.byref(h)) == gainls.ERR_INVALID_ARG
    assert gainls.lib().gain_engine_create(0, 11, 0, 1, ctypes.byref(h)) == gainls.ERR_INVALID_ARG
    assert "bad argument" in gainls.lib().gain_last_error_string().decode()
    assert gainls.lib().gain_run_pair(None, None, 0, None, None) == gainls.ERR_INVALID_ARG
    assert gainls.lib().gain_engine_create(0, 11, 4, 4, ctypes.byref(h)) == gainls.ERR_INVALID_ARG   # maxdeg 1..3


def test_new_entry_points_reject_bad_arguments_on_the_host(built_lib):
    """The plan executor, the component runs, the asynchronous lines and the adjoints check
    their arguments before touching a device."""
    import gainls
    L = gainls.lib()
    assert L.gain_run_plan(None, 1, None, 0, 0, None, gainls.JOB_DONE_FN(0), None, None) == gainls.ERR_INVALID_ARG
    engines = (ctypes.c_void_p * 2)(None, None)
    assert L.gain_run_plan(engines, 2, None, 0, 0, None, gainls.JOB_DONE_FN(0), None, None) == gainls.ERR_INVALID_ARG
    assert "NULL" in L.gain_last_error_string().decode()
    assert L.gain_run_pair_component(None, None, 0, 0, 0, None, None) == gainls.ERR_INVALID_ARG
    assert L.gain_run_pair_degenerate(None, None, None, 0, None, None) == gainls.ERR_INVALID_ARG
    assert L.gain_pair_lines_async(None, None, None, None, 0, 0, None, None, None, None, None) == gainls.ERR_INVALID_ARG
    assert L.gain_lines_wait(None) == gainls.ERR_INVALID_ARG
    assert L.gain_adjoint_pair_prec(None, None, None, None, 7, None) == gainls.ERR_INVALID_ARG
    assert "precision" in L.gain_last_error_string().decode()
    assert L.gain_adjoint_pair_degenerate(None, None, None, None, None, 0, None) == gainls.ERR_INVALID_ARG


def test_dropin_validation_is_host_side(built_lib):
    import gainls
    # |jI - jF| > 1, negative sizes, kF > jF: all rejected before touching any pointer
    bad = [
        dict(jI=1, jF=3, kF=0, dimenF=4),
        dict(jI=2, jF=2, kF=3, dimenF=4),
        dict(jI=2, jF=2, kF=0, dimenF=-1),
    ]
    for b in bad:
        with pytest.raises(gainls.GainError) as e:
            gainls.hls_kblock(b["dimenF"], 4, b["jI"], b["jF"], b["kF"], 1, 1, 1, 1, 0, 0, 0, 4, 4, 4, 1, 1,
                              1, 1, 1, 11, 4)
        assert e.value.status == gainls.ERR_INVALID_ARG
    with pytest.raises(gainls.GainError):
        gainls.expand(4, 0, 0, 0, 1, 4, 1, 1, 1, 1, 1, 1)


@pytest.mark.parametrize("args", [
    (1234.5678901, 3, 1, 0, 0, 0, 0, 1.23456789e-5, None, None),
    (0.000001, 11999, 11, 1, 1999, 10, 0, 3.5e-300, 1.0e-30, None),
    (8000.0, 0, 31, 3, 5, 30, 2, 0.0, 0.0, [0.1, -0.25, 3.0e-9]),
    (-12.5, 7, 2, 1, 7, 2, 0, 1e10, None, [1.0]),
])
def test_line_text_matches_reference_format(built_lib, args):
    import gainls
    import oracle
    nu, iF, jF, gF, iI, jI, gI, A, inten, amps = args
    a = gainls.format_line(nu, iF, jF, gF, iI, jI, gI, A, intensity=inten, amps=amps)
    b = oracle.line_text(nu, iF, jF, gF, iI, jI, gI, A, intens=inten, amps=amps)
    assert a == b


def test_manager_header_compiles_and_links(built_lib, tmp_path):
    """The C++ GpuManager mirror builds against the library: every method it defines, the
    block-pair entry points included, compiles and links (no GPU call is made)."""
    import shutil
    import subprocess
    from conftest import ROOT
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no g++")
    src = tmp_path / "use_manager.cpp"
    src.write_text(
        '#include "gain_gpu_manager.hpp"\n'
        "int main(int argc, char**) {\n"
        "    auto a = &gain::GpuManager::ExecuteBlockPair;\n"
        "    auto b = &gain::GpuManager::ExecuteBlockPairDegenerate;\n"
        "    auto c = &gain::GpuManager::ExecuteDotProduct;\n"
        "    return argc > 99 ? (int)(sizeof a + sizeof b + sizeof c) : 0;\n"
        "}\n")
    lib = os.path.join(ROOT, "gain-mpi_gb300", "lib")
    cuda = "/usr/local/cuda"
    out = tmp_path / "use_manager"
    subprocess.run([gxx, "-std=c++17", "-O0", "-I", os.path.join(ROOT, "include"), "-I", cuda + "/include", str(src),
                    "-o", str(out), "-L", lib, "-lgainls", "-L", cuda + "/lib64", "-lcudart",
                    "-Wl,-rpath," + lib], check=True)
    assert out.exists()


def test_struct_layouts_match_the_header(tmp_path):
    """Every ctypes mirror of a C ABI struct has the header struct's size and, member by member
    (same names), its offsets: a C program built from include/*.h prints them."""
    import shutil
    import subprocess
    import gainls
    from conftest import ROOT
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    pairs = [(gainls.PairJob, "gain_pair_job"), (gainls.SplitOpts, "gain_split_opts"), (gainls.Stats, "gain_stats"),
             (gainls.PlanStats, "gain_plan_stats"), (gainls.LineParams, "gain_line_params"),
             (gainls.State, "gain_state"), (gainls.Filters, "gain_filters"), (gainls.TroveState, "gain_trove_state")]
    lines = ['#include <stdio.h>', '#include "gain_trove.h"', "int main(void) {"]
    for cls, cname in pairs:
        lines.append(f'    printf("{cname} size %zu\\n", sizeof({cname}));')
        for f, _ in cls._fields_:
            lines.append(f'    printf("{cname} {f} %zu\\n", offsetof({cname}, {f}));')
    lines += ["    return 0;", "}"]
    src = tmp_path / "layouts.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layouts"
    subprocess.run([cc, "-std=c11", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = {}
    for line in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.splitlines():
        cname, what, val = line.split()
        got[(cname, what)] = int(val)
    for cls, cname in pairs:
        assert got[(cname, "size")] == ctypes.sizeof(cls), cname
        for f, _ in cls._fields_:
            assert got[(cname, f)] == getattr(cls, f).offset, (cname, f)
