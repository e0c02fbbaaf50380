"""GPU parity of the engine's two block-pair paths against the CPU oracle.

plain FP64 path: the reference's method (half line strength per lower state, then dot
products with the upper vectors); must match the oracle to FP64 rounding (relative 1e-12
of the largest amplitude, far below the 1e-10 required on S).
split path: Ozaki-sliced BF16 tensor-core GEMMs with certified bounds and FP64 refinement;
line strengths S = amp^2 must match within 1e-8 relative for every line with
S > 1e-10 S_max (the tolerance of the headline metric).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

JMAX = 11
S_REL_TOL = 1e-8


def _oracle_amp(p, jI, gI, jF, gF, lo, up, mode, nthreads=8):
    import oracle
    import threej
    return oracle.run_pair(p, jI, gI, jF, gF, lo, up, threej.threej_table(JMAX), JMAX, mode, nthreads)


def _s_rel_err(amp, ref):
    S, Sr = amp ** 2, ref ** 2
    m = Sr > 1e-10 * Sr.max()
    return float(np.max(np.abs(S[m] - Sr[m]) / Sr[m]))


@pytest.fixture(scope="module")
def c4_small(built_lib):
    import gainls
    import synth
    p = synth.make_problem(16, [2, 3], "c4")
    eng = gainls.Engine(JMAX, p.nsym, 1)
    gainls.upload_problem(eng, p)
    return p, eng


PAIRS = [(0, 0, 1, 1), (1, 1, 0, 0), (1, 2, 1, 3), (0, 3, 1, 2)]


@pytest.mark.parametrize("pair", PAIRS)
def test_plain_fp64_matches_oracle(c4_small, pair):
    import gainls
    import oracle
    p, eng = c4_small
    jI, gI, jF, gF = pair
    lo = list(range(p.blocks[(jI, gI)].vecs.shape[0]))
    up = list(range(p.blocks[(jF, gF)].vecs.shape[0]))
    eng.run_pair(jI, gI, jF, gF, lo, up, gainls.PATH_PLAIN_FP64)
    amp = eng.fetch_amp()
    ref = _oracle_amp(p, jI, gI, jF, gF, lo, up, oracle.DD)
    assert np.max(np.abs(amp - ref)) <= 1e-12 * np.abs(ref).max()


@pytest.mark.parametrize("pair", PAIRS)
def test_split_matches_oracle(c4_small, pair):
    import gainls
    import oracle
    p, eng = c4_small
    jI, gI, jF, gF = pair
    lo = list(range(p.blocks[(jI, gI)].vecs.shape[0]))
    up = list(range(p.blocks[(jF, gF)].vecs.shape[0]))
    st = eng.run_pair(jI, gI, jF, gF, lo, up, gainls.PATH_SPLIT)
    amp = eng.fetch_amp()
    ref = _oracle_amp(p, jI, gI, jF, gF, lo, up, oracle.DD)
    assert st["status"] == gainls.OK
    assert _s_rel_err(amp, ref) <= S_REL_TOL
    assert np.max(np.abs(amp - ref)) <= 1e-11 * np.abs(ref).max()


def test_split_level_subsets_and_order(c4_small):
    """Arbitrary (unsorted, partial) level lists on both sides."""
    import gainls
    import oracle
    p, eng = c4_small
    rng = np.random.default_rng(5)
    nI = p.blocks[(0, 0)].vecs.shape[0]
    nF = p.blocks[(1, 1)].vecs.shape[0]
    lo = list(rng.permutation(nI)[: nI - 3])
    up = list(rng.permutation(nF)[: nF - 5])
    eng.run_pair(0, 0, 1, 1, lo, up, gainls.PATH_SPLIT)
    amp = eng.fetch_amp()
    ref = _oracle_amp(p, 0, 0, 1, 1, lo, up, oracle.DD)
    assert _s_rel_err(amp, ref) <= S_REL_TOL


@pytest.fixture(scope="module")
def c4_medium(built_lib):
    import gainls
    import synth
    p = synth.make_problem(120, [5, 6], "c4", blocks=[(5, 0), (6, 1)])
    eng = gainls.Engine(JMAX, p.nsym, 1)
    gainls.upload_problem(eng, p)
    return p, eng


@pytest.mark.parametrize("opts", [dict(), dict(beta=6), dict(kchunks=2), dict(beta=8, slices=6, kchunks=3)])
def test_split_matches_plain_medium(c4_medium, opts):
    """Several tiles per GEMM, digit widths 6-8 and 1-3 exact-accumulation chunks."""
    import gainls
    p, eng = c4_medium
    nI = p.blocks[(0, 0)].vecs.shape[0]
    nF = p.blocks[(1, 1)].vecs.shape[0]
    lo, up = list(range(nI)), list(range(nF))
    eng.run_pair(0, 0, 1, 1, lo, up, gainls.PATH_PLAIN_FP64)
    ref = eng.fetch_amp().copy()
    st = eng.run_pair(0, 0, 1, 1, lo, up, gainls.PATH_SPLIT, **opts)
    amp = eng.fetch_amp()
    assert st["status"] == gainls.OK, st
    assert _s_rel_err(amp, ref) <= S_REL_TOL
    if opts.get("kchunks"):
        assert st["chunks2"] == opts["kchunks"]


def test_plain_medium_matches_oracle_ref_order(c4_medium):
    import gainls
    import oracle
    p, eng = c4_medium
    lo = list(range(0, p.blocks[(0, 0)].vecs.shape[0], 37))
    up = list(range(p.blocks[(1, 1)].vecs.shape[0]))
    eng.run_pair(0, 0, 1, 1, lo, up, gainls.PATH_PLAIN_FP64)
    amp = eng.fetch_amp()
    ref = _oracle_amp(p, 0, 0, 1, 1, lo, up, oracle.REF)
    assert np.max(np.abs(amp - ref)) <= 1e-12 * np.abs(ref).max()


def test_full_rule_pair_and_dipole_block(built_lib):
    """One symmetry class (the whole basis) and a dipole piece covering part of the
    vibrational range: only upper functions whose vibrational index lies in the piece
    get contributions (BaseClasses/Dipole.h:9-15, GPU/dipole_GPU.cu:429)."""
    import gainls
    import oracle
    import synth
    p = synth.make_problem(16, [1, 2], "full")
    eng = gainls.Engine(JMAX, 1, 1)
    gainls.upload_problem(eng, p, dipole_block=(5, 11))
    lo = list(range(10))
    up = list(range(p.blocks[(1, 0)].vecs.shape[0]))
    ref = _oracle_amp_block(p, lo, up)
    for path in (gainls.PATH_PLAIN_FP64, gainls.PATH_SPLIT):
        eng.run_pair(0, 0, 1, 0, lo, up, path)
        amp = eng.fetch_amp()
        assert np.max(np.abs(amp - ref)) <= 1e-11 * np.abs(ref).max()


def _oracle_amp_block(p, lo, up):
    import oracle
    import threej
    return oracle.run_pair(p, 0, 0, 1, 0, lo, up, threej.threej_table(JMAX), JMAX, oracle.DD, 8,
                           dipole_block=(5, 11))


def test_async_eigvec_upload_orders_reads_after_the_copy(built_lib):
    """Queued uploads from page-locked memory give the synchronous upload's amplitudes on both
    paths, and a second queued upload (lower vectors doubled) is the one the next run reads."""
    import torch
    import gainls
    import synth
    p = synth.make_problem(120, [5, 6], "c4", blocks=[(5, 0), (6, 1)])
    eng = gainls.Engine(JMAX, p.nsym, 1)
    gainls.upload_problem(eng, p)
    vI, vF = p.blocks[(0, 0)].vecs, p.blocks[(1, 1)].vecs
    lo, up = list(range(vI.shape[0])), list(range(vF.shape[0]))
    ref = {}
    for path in (gainls.PATH_SPLIT, gainls.PATH_PLAIN_FP64):
        eng.run_pair(0, 0, 1, 1, lo, up, path)
        ref[path] = eng.fetch_amp().copy()

    def pinned(a):
        t = torch.empty(a.shape, dtype=torch.float64, pin_memory=True)
        t.numpy()[...] = a
        return t

    hI, hF = pinned(vI), pinned(vF)
    for path in (gainls.PATH_SPLIT, gainls.PATH_PLAIN_FP64):
        eng.upload_eigvecs_async(0, 0, hI.numpy())
        eng.upload_eigvecs_async(1, 1, hF.numpy())
        eng.run_pair(0, 0, 1, 1, lo, up, path)
        assert np.array_equal(eng.fetch_amp(), ref[path])
    hI2 = pinned(2.0 * vI)   # exact scaling: amplitudes double exactly
    eng.upload_eigvecs_async(0, 0, hI2.numpy())
    eng.run_pair(0, 0, 1, 1, lo, up, gainls.PATH_SPLIT)
    assert np.array_equal(eng.fetch_amp(), 2.0 * ref[gainls.PATH_SPLIT])
    del eng


def test_bounded_wait_gives_up_and_the_engine_stays_usable(built_lib):
    """Failure detection without a GPU fault: a bounded mbarrier wait on a barrier nothing
    arrives on gives up after its limit and reports GAIN_ERR_TIMEOUT; the same engine then
    computes a block pair as usual."""
    import time
    import gainls
    import synth
    p = synth.make_problem(16, [2, 3], "c4", blocks=[(2, 0), (3, 1)])
    eng = gainls.Engine(11, p.nsym, 1)
    gainls.upload_problem(eng, p)
    t0 = time.perf_counter()
    with pytest.raises(gainls.GainError) as ex:
        gainls.check(gainls.lib().gain_selftest_bounded_wait(eng.h, 20.0))
    assert ex.value.status == gainls.ERR_TIMEOUT
    assert "gave up" in str(ex.value)
    assert time.perf_counter() - t0 < 5.0
    lo = list(range(p.blocks[(0, 0)].vecs.shape[0]))
    up = list(range(p.blocks[(1, 1)].vecs.shape[0]))
    st = eng.run_pair(0, 0, 1, 1, lo, up, gainls.PATH_SPLIT)
    assert st["status"] == gainls.OK


def test_upper_side_in_two_halves_matches_one_phase(built_lib, monkeypatch):
    """While the upper vectors arrive in two parts (asynchronous upload of at least 512
    levels), the upper digits and the amplitude GEMM run in two halves; the amplitudes are
    the same bits as in one phase (GAINLS_UPPER_HALVES=force takes the two-phase route even
    when the copy has already landed)."""
    import torch
    import gainls
    import synth
    p = synth.make_problem(160, [7, 8], "c4", blocks=[(7, 0), (8, 1)])
    eng = gainls.Engine(11, p.nsym, 1)
    gainls.upload_problem(eng, p)
    vl, vu = p.blocks[(0, 0)].vecs, p.blocks[(1, 1)].vecs
    assert vu.shape[0] >= 512
    lo, up = list(range(vl.shape[0])), list(range(vu.shape[0]))
    eng.run_pair(0, 0, 1, 1, lo, up, gainls.PATH_SPLIT)
    one = eng.fetch_amp().copy()
    pin = torch.empty(vu.shape, dtype=torch.float64, pin_memory=True).numpy()
    pin[...] = vu
    monkeypatch.setenv("GAINLS_UPPER_HALVES", "force")
    eng.upload_eigvecs_async(1, 1, pin)
    st = eng.run_pair(0, 0, 1, 1, lo, up, gainls.PATH_SPLIT)
    assert st["kernel_launches"] >= 9   # two upper slicings and two amplitude GEMM launches
    np.testing.assert_array_equal(eng.fetch_amp(), one)


def test_fused_first_gemm_products_are_exact(c4_medium, monkeypatch):
    """Short band tiles add the digit products of one weight into one accumulator before the
    drain.  The sums are exact integers; only the truncation of weights below 2^-50 of the
    fixed-point recombination moves (once per group instead of once per product), so the
    amplitudes agree with the unfused run's to that level and both certify."""
    import gainls
    p, eng = c4_medium
    nI = p.blocks[(0, 0)].vecs.shape[0]
    nF = p.blocks[(1, 1)].vecs.shape[0]
    lo, up = list(range(nI)), list(range(nF))
    st = eng.run_pair(0, 0, 1, 1, lo, up, gainls.PATH_SPLIT)
    fused = eng.fetch_amp().copy()
    monkeypatch.setenv("GAINLS_FUSE1", "0")
    st0 = eng.run_pair(0, 0, 1, 1, lo, up, gainls.PATH_SPLIT)
    assert st["inexact"] == 0 and st0["inexact"] == 0
    unfused = eng.fetch_amp()
    assert np.max(np.abs(unfused - fused)) <= 1e-13 * np.abs(unfused).max()
