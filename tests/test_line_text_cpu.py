"""The line-list conversions (csrc/linefmt.h, the code the device text kernels run) compiled
for the host, against the C library's printf -- what Output::OutputLinestrength calls
(BaseClasses/Output.cpp:99-111) -- on random bit patterns over the whole double range, exact
rounding ties, powers of ten, subnormals, signed zeros, NaN and infinities."""
import ctypes
import struct
import types

import numpy as np
import pytest

_libc = ctypes.CDLL(None)


def c_printf(fmt: str, x: float) -> str:
    buf = ctypes.create_string_buffer(512)
    _libc.snprintf(buf, 512, fmt.encode(), ctypes.c_double(x))
    return buf.value.decode()


def _special_values():
    vals = [0.0, -0.0, float("nan"), -float("nan"), float("inf"), -float("inf"), 5e-324, -5e-324,
            2.2250738585072014e-308, 2.225073858507201e-308, 1.7976931348623157e308, -1.7976931348623157e308,
            1.0, -1.0, 0.1, 0.5, 1.5, 2.5, 9.5, 1e-6, 5e-7, 4.9999999999999996e-7, 0.0078125, 0.0234375,
            12345678905.0, 12345678915.0, 1234567890.5, 1234567891.5, 9.9999999995, 9.99999999949,
            999999.9999995, 99999.9999995, 99999.99999949999, 1e22, 1e23, 9.999999999e99, 9.9999999995e99,
            1e100, 1e-100, 1.0000000005e-100, 2.0 ** 63, 2.0 ** 64, 2.0 ** 64 + 4096.0, 18446744073709551615.0,
            123456789012345678901234567890.0, 6.02214076e23, 1.602176634e-19, 4503599627370495.5]
    vals += [k / 128.0 for k in range(1, 64, 2)]              # ties of %.6f
    vals += [10.0 ** e for e in range(-320, 309, 7)]
    vals += [-(10.0 ** e) * 0.99999999995 for e in range(-300, 300, 13)]
    return vals


def _random_values(n, seed):
    rng = np.random.default_rng(seed)
    bits = rng.integers(0, 2 ** 63, size=n, dtype=np.int64).astype(np.uint64)
    bits |= (rng.integers(0, 2, size=n).astype(np.uint64) << np.uint64(63))
    v = bits.view(np.float64)
    # and values in the ranges the line list prints (frequencies, A, intensities, amplitudes)
    w = np.concatenate([rng.uniform(0, 20000, n // 4), 10.0 ** rng.uniform(-60, 5, n // 4),
                        rng.standard_normal(n // 4) * 10.0 ** rng.uniform(-12, 2, n // 4)])
    return [float(x) for x in np.concatenate([v, w])]


@pytest.mark.parametrize("conv,width,prec", [("E", 16, 9), ("f", 12, 6), ("E", 0, 0), ("E", 25, 17),
                                             ("f", 0, 0), ("f", 20, 9), ("E", 12, 3)])
def test_conversion_matches_printf(built_lib, conv, width, prec):
    import gainls
    fmt = f"%{width}.{prec}{conv}" if width else f"%.{prec}{conv}"
    vals = _special_values() + _random_values(3000, 1000 + prec)
    bad = []
    for x in vals:
        a, b = gainls.format_value(x, conv, width, prec), c_printf(fmt, x)
        if a != b:
            bad.append((struct.pack("<d", x).hex(), a, b))
    assert not bad, bad[:10]


def test_line_text_native_matches_snprintf(built_lib):
    """Whole lines: the native conversions, the snprintf formatter and the oracle agree."""
    import gainls
    import oracle
    rng = np.random.default_rng(11)
    for i in range(400):
        nu = float(rng.uniform(1e-3, 25000.0)) if i % 7 else float(10.0 ** rng.uniform(-45, 6))
        iF, iI = int(rng.integers(0, 10 ** 8)), int(rng.integers(0, 10 ** 8))
        jF, jI = int(rng.integers(0, 200)), int(rng.integers(0, 200))
        gF, gI = int(rng.integers(0, 12)), int(rng.integers(0, 12))
        A = float(10.0 ** rng.uniform(-40, 6))
        inten = float(10.0 ** rng.uniform(-120, -15)) if i % 3 else None
        amps = list(rng.standard_normal(int(rng.integers(1, 4))) * 10.0 ** rng.uniform(-110, 1)) if i % 2 else None
        a = gainls.format_line_native(nu, iF, jF, gF, iI, jI, gI, A, intensity=inten, amps=amps)
        b = gainls.format_line(nu, iF, jF, gF, iI, jI, gI, A, intensity=inten, amps=amps)
        c = oracle.line_text(nu, iF, jF, gF, iI, jI, gI, A, intens=inten, amps=amps)
        assert a == b == c, (a, b, c)


def test_line_tail_is_fprintf_of_the_buffer(built_lib):
    """Output.cpp:111 appends " || \\n" to a buffer that already ends in a space."""
    import gainls
    s = gainls.format_line_native(1234.5, 9, 3, 1, 4, 2, 0, 1.25e-3, intensity=2.5e-21)
    assert s == " 1234.500000       10    3    2 <-        5    2    1  1.250000000E-03  2.500000000E-21  || \n"


def test_oracle_line_list_matches_per_line_text(built_lib):
    """The oracle's block-pair line list is the per-line text of the lines it keeps."""
    import oracle
    rng = np.random.default_rng(5)
    amp = rng.standard_normal((7, 9)) * 1e-2
    eI = np.sort(rng.uniform(0, 3000, 7))
    eF = np.sort(rng.uniform(0, 6000, 9))
    levI, levF = np.arange(7) * 3, np.arange(9) + 100
    text, n = oracle.line_list(amp, eI, eF, levI, levF, 4, 5, 1, 0, thresh=1e-9, freq=(10.0, 5000.0),
                               intensity=True, amplitudes=True)
    flt = types.SimpleNamespace(reduced=False, zpe=0.0, gns=[1.0], temperature=296.0, q_part=1.0, thresh=1e-9)
    lines, kept = [], 0
    for r in range(7):
        for c in range(9):
            nu = eF[c] - eI[r]
            if not (10.0 <= nu <= 5000.0):
                continue
            v = oracle.line([amp[r, c]], [1], 1, 1, 1, flt, eI[r], eF[c], 4, 5, 0)
            if v is None:
                continue
            kept += 1
            lines.append(oracle.line_text(nu, levF[c], 5, 0, levI[r], 4, 1, v[1], intens=v[2], amps=[amp[r, c]]))
    assert n == kept > 0
    assert text.decode() == "".join(lines)


def test_length_pass_equals_the_converted_length(built_lib):
    """The device's length pass (value ranges, conversion only outside them) gives the
    converted text's length for ordinary and extreme fields alike."""
    import gainls
    vals = _special_values() + _random_values(2000, 31)
    rng = np.random.default_rng(12)
    for i, x in enumerate(vals):
        y = vals[(7 * i + 3) % len(vals)]
        z = vals[(11 * i + 5) % len(vals)]
        idx = int(rng.integers(-5, 10 ** 9))
        for args in ((x, idx, 3, 1, 4, 2, 0, y), (abs(y), 9, -1, 7, idx, 1, 2, x)):
            for inten, amps in ((None, None), (z, None), (z, [x, y]), (None, [z])):
                n = gainls.line_length_native(*args, intensity=inten, amps=amps)
                t = gainls.format_line_native(*args, intensity=inten, amps=amps)
                assert n == len(t), (args, inten, amps, t)
