"""Pin the CPU oracle to the reference's own GPU kernels.

tests/golden/*.npz hold outputs of GAIN-MPI's unmodified GPU/dipole_GPU.cu run on a GB300
through oracle/ref_harness.cu (tests/golden/make_golden.py): per lower state the half line
strength after all K-block launches, and the cublasDdot amplitudes.  The oracle restates the
kernels' per-element operation sequence, so its half_ls must agree bit for bit; amplitudes
(summation order of cublasDdot unspecified) agree within the FP64 dot-product error bound.
"""
import glob
import os

import numpy as np
import pytest

from conftest import GOLDEN

FIXTURES = sorted(f for f in glob.glob(os.path.join(GOLDEN, "*.npz")) if not os.path.basename(f).startswith("rotsym_"))
ROT_FIXTURES = sorted(glob.glob(os.path.join(GOLDEN, "rotsym_*.npz")))


def _problem(d):
    import synth
    nv, jvals, rule = int(d["nv"]), [int(x) for x in d["jvals"]], str(d["rule"])
    bases = [synth.make_basis(J, nv) for J in jvals]
    infl = [synth.inflation_of(b, rule, synth.nsym_of(rule)) for b in bases]
    return jvals, bases, infl


def _components(d):
    """(idegI, idegF) of a fixture (0, 0 for the non-degenerate ones)."""
    return (int(d["idegI"]), int(d["idegF"])) if "idegI" in d.files else (0, 0)


def test_fixtures_present():
    names = {os.path.basename(f)[:-4] for f in FIXTURES}
    assert {"cfg1_small", "c4_dJp1", "c4_dJm1", "c4_dJ0", "c4_highJ", "full_blocked"} <= names
    assert {"c3e_EE_c00", "c3e_EE_c10", "c3e_EE_c01", "c3e_EE_c11_blocked", "c3e_A1A2"} <= names


@pytest.mark.parametrize("path", FIXTURES, ids=lambda p: os.path.basename(p)[:-4])
def test_fixture_inputs_are_reproducible(path):
    """The dipole regenerates from its seed (to rounding: the fixtures were made with libm's
    exp on another machine; every test below uses the stored copy); the 3j table the
    reference kernels consumed is the exact one, bit for bit."""
    import synth
    import threej
    d = np.load(path)
    np.testing.assert_allclose(d["dipole"], synth.make_dipole(int(d["nv"])), rtol=1e-10, atol=1e-300)
    assert np.array_equal(d["threej"], threej.threej_table(int(d["jmax"])))


@pytest.mark.parametrize("path", FIXTURES, ids=lambda p: os.path.basename(p)[:-4])
def test_oracle_half_ls_bit_exact(oracle_lib, path):
    import oracle
    d = np.load(path)
    jvals, bases, infl = _problem(d)
    jI, jF = jvals.index(int(d["JI"])), jvals.index(int(d["JF"]))
    gI = int(d["gI"])
    dI, _ = _components(d)
    s, e = (int(x) for x in d["block"])
    piece = np.ascontiguousarray(d["dipole"][:, :, s:e])
    nbad = 0
    for l in range(d["vec_lower"].shape[0]):
        prim = oracle.expand(infl[jI], gI, d["vec_lower"][l], ideg=dI)
        hls = np.zeros(bases[jF].dimen)
        for kF in range(bases[jF].J + 1):
            oracle.hls_kblock(int(bases[jF].kblock[kF]), bases[jI].dimen, bases[jI].J, bases[jF].J, kF,
                              bases[jI].tau, bases[jF].tau, bases[jI].vib, bases[jF].vib,
                              int(bases[jF].kstart[kF]), int(bases[jI].kstart[max(kF - 1, 0)]), s, e, e - s,
                              bases[jI].kblock, piece, int(d["nv"]), prim, d["threej"], int(d["jmax"]), hls)
        nbad += int(np.count_nonzero(hls.view(np.uint64) != d["ref_hls"][l].view(np.uint64)))
    assert nbad == 0


@pytest.mark.parametrize("path", FIXTURES, ids=lambda p: os.path.basename(p)[:-4])
def test_oracle_amplitudes_within_dot_bound(oracle_lib, path):
    import oracle
    d = np.load(path)
    jvals, bases, infl = _problem(d)
    jI, jF = jvals.index(int(d["JI"])), jvals.index(int(d["JF"]))
    gI, gF = int(d["gI"]), int(d["gF"])
    _, dF = _components(d)
    for l in range(d["vec_lower"].shape[0]):
        h = d["ref_hls"][l]
        for u in range(d["vec_upper"].shape[0]):
            prim = oracle.expand(infl[jF], gF, d["vec_upper"][u], ideg=dF)
            a = oracle.dot(prim, h, oracle.DD)
            bound = 2 * len(h) * 1.12e-16 * float(np.sum(np.abs(prim * h))) + 1e-300
            assert abs(a - d["ref_amp"][l, u]) <= bound


# ------------------------------------------------------------ rotational-symmetry (Euler) form

def _rot_inputs(d):
    import synth
    nv, JI, JF, md = int(d["nv"]), int(d["JI"]), int(d["JF"]), int(d["maxdeg"])
    bI, bF = synth.make_rotsym_basis(JI, nv, md), synth.make_rotsym_basis(JF, nv, md)
    s, e = (int(x) for x in d["block"])
    piece = np.ascontiguousarray(d["dipole"][:, :, s:e]).reshape(-1)
    return nv, md, bI, bF, s, e, piece


def test_rotsym_fixtures_present():
    names = {os.path.basename(f)[:-4] for f in ROT_FIXTURES}
    assert {"rotsym_dJp1", "rotsym_dJ0", "rotsym_dJm1_blocked"} <= names


@pytest.mark.parametrize("path", ROT_FIXTURES, ids=lambda p: os.path.basename(p)[:-4])
def test_rotsym_inputs_are_reproducible(path):
    """The Wigner table regenerates exactly from its seed, the dipole to rounding."""
    import synth
    d = np.load(path)
    assert np.array_equal(d["wigner"], synth.make_wigner(int(d["JI"]), int(d["JF"]), int(d["maxdeg"])))
    assert np.allclose(d["dipole"], synth.make_dipole(int(d["nv"])), rtol=1e-10, atol=0)


@pytest.mark.parametrize("path", ROT_FIXTURES, ids=lambda p: os.path.basename(p)[:-4])
def test_rotsym_oracle_bit_exact_vs_reference_kernel(path):
    """The oracle's restatement of the rotsym kernel (GPU/dipole_GPU.cu:641-723) equals the
    reference kernel's half_ls bit for bit, including the untouched entries outside the
    dipole block and degenerate levels (maxdeg 2)."""
    import oracle
    d = np.load(path)
    nv, md, bI, bF, s, e, piece = _rot_inputs(d)
    for v, ref in zip(d["vectors"], d["ref_hls"]):
        h = np.zeros(bF.dimen)
        oracle.hls_rotsym(bI, bF, int(d["nlevelI"]), int(d["nlevelF"]), md, piece, nv, (s, e, e - s), d["wigner"], v, h)
        assert np.array_equal(h, ref)


@pytest.mark.parametrize("path", ROT_FIXTURES, ids=lambda p: os.path.basename(p)[:-4])
def test_rotsym_reference_within_rounding_of_double_double(path):
    import oracle
    d = np.load(path)
    nv, md, bI, bF, s, e, piece = _rot_inputs(d)
    for v, ref in zip(d["vectors"], d["ref_hls"]):
        h = np.zeros(bF.dimen)
        oracle.hls_rotsym(bI, bF, int(d["nlevelI"]), int(d["nlevelF"]), md, piece, nv, (s, e, e - s), d["wigner"], v, h,
                          oracle.DD)
        assert np.max(np.abs(h - ref)) <= 64 * 2.0 ** -53 * bI.dimen * np.abs(ref).max()
