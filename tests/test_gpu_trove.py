"""A block pair run from ingested TROVE checkpoint files (gain_trove_basis_upload, the
dipole pieces of j0_extfield.chk, eigenvector records) gives the amplitudes of the same
problem uploaded directly; with the dipole split into pieces, the amplitudes summed over
the pieces (one run per piece, MultiGpuManager::ExecuteHalfLs's block loop) agree too."""
import os

import numpy as np
import pytest

import trove_files

pytestmark = pytest.mark.gpu

JMAX = 11


def test_pair_from_trove_files_matches_direct_upload(tmp_path, built_lib):
    import gainls
    import synth
    p = synth.make_problem(20, [2, 3], "c4", blocks=[(2, 0), (3, 1)])
    trove_files.write_problem(str(tmp_path), p)
    d = str(tmp_path)
    direct = gainls.Engine(JMAX, p.nsym, 1)
    gainls.upload_problem(direct, p)
    eng = gainls.Engine(JMAX, p.nsym, 1)
    for jind, J in enumerate(p.jvals):
        gainls.trove_upload_basis(eng, jind, d, J, p.nsym, p.sym_degen)
    n, pieces = gainls.trove_dipole(os.path.join(d, "j0_extfield.chk"))
    (s, e, c, piece), = pieces
    eng.upload_dipole(piece, n, s, e, c)
    f = gainls.make_filters([1.0] * 4, p.isym_pairs, p.igamma_pair, p.sym_degen, (0.0, 1e9), (0.0, 1e9))
    for jind, J, g in ((0, 2, 0), (1, 3, 1)):
        st, dim = gainls.trove_states(d, J, g, f)
        vecs = gainls.trove_vectors(os.path.join(d, f"j0eigen_vectors{J}_{g + 1}.chk"), dim, st["irec"])
        eng.upload_eigvecs(jind, g, vecs)
    lo = list(range(p.blocks[(0, 0)].vecs.shape[0]))
    up = list(range(p.blocks[(1, 1)].vecs.shape[0]))
    for path in (gainls.PATH_PLAIN_FP64, gainls.PATH_SPLIT):
        direct.run_pair(0, 0, 1, 1, lo, up, path)
        eng.run_pair(0, 0, 1, 1, lo, up, path)
        np.testing.assert_array_equal(eng.fetch_amp(), direct.fetch_amp())


def test_dipole_pieces_sum_to_the_whole(tmp_path, built_lib):
    import gainls
    import synth
    p = synth.make_problem(20, [2, 3], "c4", blocks=[(2, 0), (3, 1)])
    trove_files.write_problem(str(tmp_path), p)
    eng = gainls.Engine(JMAX, p.nsym, 1)
    gainls.upload_problem(eng, p)
    lo = list(range(p.blocks[(0, 0)].vecs.shape[0]))
    up = list(range(p.blocks[(1, 1)].vecs.shape[0]))
    eng.run_pair(0, 0, 1, 1, lo, up, gainls.PATH_PLAIN_FP64)
    whole = eng.fetch_amp().copy()
    n, pieces = gainls.trove_dipole(os.path.join(str(tmp_path), "j0_extfield.chk"), 3 * 20 * 20 * 8 // 3)
    assert len(pieces) == 4
    total = np.zeros_like(whole)
    for s, e, c, piece in pieces:
        eng.upload_dipole(piece, n, s, e, c)
        eng.run_pair(0, 0, 1, 1, lo, up, gainls.PATH_PLAIN_FP64)
        total += eng.fetch_amp()
    assert np.max(np.abs(total - whole)) <= 1e-13 * np.abs(whole).max()


@pytest.mark.parametrize("rule", ["c4", "c4r"])
def test_engine_loops_over_dipole_pieces(tmp_path, built_lib, rule):
    """gain_upload_dipole_pieces: the split path accumulates the first GEMM of every piece
    and the plain path sums per-piece amplitudes; both reproduce the one-piece run."""
    import gainls
    import synth
    p = synth.make_problem(24, [3, 4], rule, blocks=[(3, 0), (4, 1)])
    nv = p.dipole.shape[-1]
    eng = gainls.Engine(JMAX, p.nsym, 1)
    gainls.upload_problem(eng, p)
    lo = list(range(p.blocks[(0, 0)].vecs.shape[0]))
    up = list(range(p.blocks[(1, 1)].vecs.shape[0]))
    ref = {}
    for path in (gainls.PATH_PLAIN_FP64, gainls.PATH_SPLIT):
        eng.run_pair(0, 0, 1, 1, lo, up, path)
        ref[path] = eng.fetch_amp().copy()
    bounds = [0, 5, 11, 17, nv]
    pieces = [(s, e, np.ascontiguousarray(p.dipole[:, :, s:e]).reshape(-1)) for s, e in zip(bounds, bounds[1:])]
    eng.upload_dipole_pieces(pieces, nv)
    eng.run_pair(0, 0, 1, 1, lo, up, gainls.PATH_PLAIN_FP64)
    plain = eng.fetch_amp()
    scale = np.abs(ref[gainls.PATH_PLAIN_FP64]).max()
    assert np.max(np.abs(plain - ref[gainls.PATH_PLAIN_FP64])) <= 1e-13 * scale
    st = eng.run_pair(0, 0, 1, 1, lo, up, gainls.PATH_SPLIT)
    assert st["status"] == gainls.OK
    split = eng.fetch_amp()
    assert np.max(np.abs(split - ref[gainls.PATH_PLAIN_FP64])) <= 1e-11 * scale
    S, Sr = split ** 2, ref[gainls.PATH_PLAIN_FP64] ** 2
    m = Sr > 1e-10 * Sr.max()
    assert np.max(np.abs(S[m] - Sr[m]) / Sr[m]) <= 1e-8
    with pytest.raises(gainls.GainError):
        eng.adjoint(0, 0, 1, 1, lo, up, np.ones((len(lo), len(up))), np.zeros(p.dipole.size))


def test_refinement_overflow_in_an_earlier_piece_fails_the_run(built_lib, monkeypatch):
    """With dipole pieces the first GEMM's refinement list restarts per piece: a list that
    overflows in an earlier piece (entries left unrefined) must fail the run with
    TOL_NOT_MET and leave no amplitudes to fetch, even when the last piece's list fits."""
    import gainls
    import synth
    p = synth.make_problem(24, [3, 4], "c4", blocks=[(3, 0), (4, 1)])
    nv = p.dipole.shape[-1]
    eng = gainls.Engine(JMAX, p.nsym, 1)
    gainls.upload_problem(eng, p)
    lo = list(range(p.blocks[(0, 0)].vecs.shape[0]))
    up = list(range(p.blocks[(1, 1)].vecs.shape[0]))

    def piece(s, e):
        return (s, e, np.ascontiguousarray(p.dipole[:, :, s:e]).reshape(-1))

    # 40-bit first-GEMM digits: no H entry certifies FP64-grade, every non-zero one is flagged
    monkeypatch.setenv("GAINLS_GEMM1_BITS", "40")
    counts = []
    # the last piece holds the last two vibrational indices (class 1 of rule c4 has only the
    # even ones, so it must reach vib nv - 2)
    for rng in ((0, nv - 2), (nv - 2, nv)):
        eng.upload_dipole_pieces([piece(*rng)], nv)
        st = eng.run_pair(0, 0, 1, 1, lo, up, gainls.PATH_SPLIT)
        assert st["status"] == gainls.OK
        counts.append(st["inexact"])
    first, last = counts
    assert first > last + 1 > 1, counts
    eng.upload_dipole_pieces([piece(0, nv - 2), piece(nv - 2, nv)], nv)
    st = eng.run_pair(0, 0, 1, 1, lo, up, gainls.PATH_SPLIT)
    assert st["status"] == gainls.OK and st["inexact"] == first + last
    monkeypatch.setenv("GAINLS_MAX_FLAGS", str((first + last) // 2))   # holds the last piece's only
    st = eng.run_pair(0, 0, 1, 1, lo, up, gainls.PATH_SPLIT, raise_on_error=False)
    assert st["status"] == gainls.ERR_TOL_NOT_MET, st
    with pytest.raises(gainls.GainError) as ei:
        eng.fetch_amp()
    assert ei.value.status == gainls.ERR_NOT_READY
    eng.close()
