"""Line-list text built on the device (gain_pair_lines_text, gain_format_values_device)
against the C library's printf and the oracle's restatement of Output::OutputLinestrength
(BaseClasses/Output.cpp:52-112): byte-identical text for the same doubles."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

JMAX = 11
_libc = ctypes.CDLL(None)


def c_printf(fmt: str, x: float) -> str:
    buf = ctypes.create_string_buffer(512)
    _libc.snprintf(buf, 512, fmt.encode(), ctypes.c_double(x))
    return buf.value.decode()


@pytest.mark.parametrize("conv,width,prec", [("E", 16, 9), ("f", 12, 6), ("E", 25, 17), ("f", 20, 9)])
def test_device_conversion_matches_printf(built_lib, conv, width, prec):
    import gainls
    from test_line_text_cpu import _random_values, _special_values
    vals = _special_values() + _random_values(20000, 77 + prec)
    got = gainls.format_values_device(vals, conv, width, prec)
    fmt = f"%{width}.{prec}{conv}"
    bad = [(x, a, b) for x, a, b in zip(vals, got, (c_printf(fmt, x) for x in vals)) if a != b]
    assert not bad, bad[:10]


@pytest.fixture(scope="module")
def pair_run(built_lib):
    import gainls
    import synth
    p = synth.make_problem(40, [2, 3], "c4", blocks=[(2, 0), (3, 1)])
    eng = gainls.Engine(JMAX, p.nsym, 1)
    gainls.upload_problem(eng, p)
    bI, bF = p.blocks[(0, 0)], p.blocks[(1, 1)]
    lo = list(range(0, bI.vecs.shape[0], 2))
    up = list(range(bF.vecs.shape[0]))
    eng.run_pair(0, 0, 1, 1, lo, up, gainls.PATH_SPLIT)
    eI = bI.energies[lo] + 0.0
    eF = bF.energies[up] + 0.0
    return p, eng, lo, up, eI, eF


@pytest.mark.parametrize("kw", [dict(), dict(intensity=False), dict(amplitudes=True),
                                dict(thresh=1e-3, freq=(50.0, 4000.0), zpe=120.0, temperature=1000.0,
                                     gnsF=3.0, q_part=7.5, amplitudes=True)])
def test_pair_text_matches_oracle(pair_run, kw):
    """The device text equals the oracle's sprintf/fprintf text of the same amplitudes, byte
    for byte, with and without the intensity column (lines whose printed intensity the
    device's exp could change take the host's value)."""
    import gainls
    import oracle
    p, eng, lo, up, eI, eF = pair_run
    amp = eng.fetch_amp().copy()
    args = dict(temperature=296.0, q_part=1.0, zpe=0.0, thresh=0.0, freq=(-1e9, 1e9), gnsF=1.0, intensity=True,
                amplitudes=False)
    args.update(kw)
    text, n = eng.lines_text(eI, eF, 2, 3, 0, 1, **args)
    assert n > 0 and len(text) > 0
    ref, nref = oracle.line_list(amp, eI, eF, lo, up, 2, 3, 0, 1, gnsF=args["gnsF"],
                                 temperature=args["temperature"], q_part=args["q_part"], zpe=args["zpe"],
                                 thresh=args["thresh"], freq=args["freq"], intensity=args["intensity"],
                                 amplitudes=args["amplitudes"])
    assert n == nref
    assert bytes(text) == ref


def test_text_device_pointer_and_small_buffer(pair_run):
    import gainls
    p, eng, lo, up, eI, eF = pair_run
    text, n = eng.lines_text(eI, eF, 2, 3, 0, 1)
    ptr, nb = ctypes.c_void_p(), ctypes.c_ulonglong()
    gainls.check(gainls.lib().gain_lines_text_device(eng.h, ctypes.byref(ptr), ctypes.byref(nb)))
    assert nb.value == len(text) and ptr.value
    small = np.empty(len(text) - 1, np.uint8)
    with pytest.raises(gainls.GainError):
        gainls.check(gainls.lib().gain_fetch_lines_text(eng.h, small.ctypes.data, small.size))


def test_text_into_host_buffer_part_by_part(pair_run):
    """gain_pair_lines_text_host gives the text gain_pair_lines_text builds; a buffer that is
    too small is refused with the size reported."""
    import gainls
    p, eng, lo, up, eI, eF = pair_run
    ref, n = eng.lines_text(eI, eF, 2, 3, 0, 1, amplitudes=True)
    out = np.zeros(len(ref) + 7, np.uint8)
    got, n2 = eng.lines_text_host(eI, eF, 2, 3, 0, 1, out, amplitudes=True)
    assert n2 == n and bytes(got) == bytes(ref)
    with pytest.raises(gainls.GainError, match="buffer"):
        eng.lines_text_host(eI, eF, 2, 3, 0, 1, np.zeros(len(ref) - 1, np.uint8), amplitudes=True)


def test_text_into_host_buffer_in_several_parts(built_lib):
    """A pair large enough for the copy to run in several parts (230 k lines)."""
    import gainls
    import synth
    p = synth.make_problem(120, [7, 8], "c4", blocks=[(7, 0), (8, 1)])
    eng = gainls.Engine(JMAX, p.nsym, 1)
    gainls.upload_problem(eng, p)
    bI, bF = p.blocks[(0, 0)], p.blocks[(1, 1)]
    lo, up = list(range(bI.vecs.shape[0])), list(range(bF.vecs.shape[0]))
    assert len(lo) * len(up) > 200_000
    eng.run_pair(0, 0, 1, 1, lo, up, gainls.PATH_SPLIT)
    ref, n = eng.lines_text(bI.energies, bF.energies, 7, 8, 0, 1)
    out = np.zeros(len(ref), np.uint8)
    got, n2 = eng.lines_text_host(bI.energies, bF.energies, 7, 8, 0, 1, out)
    assert n2 == n and bytes(got) == bytes(ref)
    # intensity column on, byte for byte against the oracle's sprintf of the same amplitudes
    # (some lines take the host's intensity: their printed digits depend on exp's last bit)
    import oracle
    want, n3 = oracle.line_list(eng.fetch_amp(), bI.energies, bF.energies, lo, up, 7, 8, 0, 1)
    assert n3 == n and bytes(ref) == want
    assert eng.intensity_host() > 0


def test_async_lines_equal_sync_and_overlap_the_next_run(pair_run):
    """gain_pair_lines_async gives gain_pair_lines' S, A and count once gain_lines_wait
    returns, also when the engine's next run was started before the wait."""
    import gainls
    import torch
    p, eng, lo, up, eI, eF = pair_run
    eng.run_pair(0, 0, 1, 1, lo, up, gainls.PATH_SPLIT)
    want = eng.lines(eI, eF, 2, 3, intensity=False, want=("S", "A"))
    n = len(lo) * len(up)
    S = torch.zeros(n, dtype=torch.float64).pin_memory().numpy()
    A = torch.zeros(n, dtype=torch.float64).pin_memory().numpy()
    eng.lines(eI, eF, 2, 3, intensity=False, want=("S", "A"), out_S=S, out_A=A, asynchronous=True)
    eng.run_pair(0, 0, 1, 1, lo[:2], up, gainls.PATH_PLAIN_FP64)   # the next run, before the wait
    nl = eng.lines_wait()
    assert nl == want["n_lines"]
    assert np.array_equal(S.reshape(want["S"].shape), want["S"])
    assert np.array_equal(A.reshape(want["A"].shape), want["A"])
    assert eng.lines_wait() == 0   # nothing pending
    # a synchronous call after an asynchronous one waits for it first
    eng.run_pair(0, 0, 1, 1, lo, up, gainls.PATH_SPLIT)
    eng.lines(eI, eF, 2, 3, intensity=False, want=("S", "A"), out_S=S, out_A=A, asynchronous=True)
    again = eng.lines(eI, eF, 2, 3, intensity=False, want=("S", "A"))
    assert np.array_equal(again["S"], want["S"])
    assert np.array_equal(S.reshape(want["S"].shape), want["S"])
