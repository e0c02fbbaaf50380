"""TROVE checkpoint ingestion (include/gain_trove.h) on files written in the formats the
reference reads: the basis, J=0 correlation and symmetry tables of j0eigen_quanta<J>.chk
(TroveClasses/TroveBasisSet.cpp), the flipped and blocked dipole of j0_extfield.chk
(TroveClasses/TroveDipole.cpp), the states of j0eigen_descr<J>_<G>.chk
(TroveClasses/TroveStates.cpp) and the vector records (BaseClasses/EigenVector.cpp) must
reproduce the synthetic problem the files were written from."""
import os

import numpy as np
import pytest

import trove_files


@pytest.fixture(scope="module")
def trove_dir(tmp_path_factory, built_lib):
    import synth
    d = tmp_path_factory.mktemp("trove")
    p = synth.make_problem(12, [0, 1, 2], "c4")
    trove_files.write_problem(str(d), p)
    return str(d), p


@pytest.mark.parametrize("jind", [0, 1, 2])
def test_basis_matches_the_written_problem(trove_dir, jind):
    import gainls
    d, p = trove_dir
    b = gainls.trove_basis(d, p.jvals[jind], p.nsym, p.sym_degen)
    ref, inf = p.bases[jind], p.infl[jind]
    assert b["dimen"] == ref.dimen and b["maxcoeff"] == inf.maxcoeff and b["matsize"] == 1
    np.testing.assert_array_equal(b["K"], ref.K)
    np.testing.assert_array_equal(b["tau"], ref.tau)
    np.testing.assert_array_equal(b["vib"], ref.vib)
    np.testing.assert_array_equal(b["kblock"], ref.kblock)
    np.testing.assert_array_equal(b["kstart"], ref.kstart)
    np.testing.assert_array_equal(b["icontr"], inf.icontr)
    np.testing.assert_array_equal(b["ijterms"], inf.ijterms)
    np.testing.assert_array_equal(b["Ntot"], inf.Ntot)
    for g in range(p.nsym):
        np.testing.assert_array_equal(b["N"][g], inf.N[g])
        np.testing.assert_array_equal(b["repres"][g], inf.repres[g])


def test_rotsym_form_keeps_level_and_degeneracy(trove_dir):
    """ROTSYM EULER: K holds the degeneracy index, tau the rotational level (:478-483)."""
    import gainls
    d, p = trove_dir
    b = gainls.trove_basis(d, 2, p.nsym, p.sym_degen, rotsym=True)
    ref = p.bases[2]
    lev = np.where(ref.K == 0, 0, 2 * ref.K - 1 + ref.tau)
    np.testing.assert_array_equal(b["tau"], lev)
    np.testing.assert_array_equal(b["K"], np.zeros_like(ref.K))
    assert b["kblock"][0] == ref.dimen


def test_vibrational_correlation_uses_the_j0_file(tmp_path, built_lib):
    """The vibrational index comes from the J=0 contracted index of the matching quanta,
    not from the position in the J file: permute the J=0 cases and the indices follow."""
    import gainls
    import synth
    nv = 6
    b0, b1 = synth.make_basis(0, nv), synth.make_basis(1, nv)
    perm = np.array([3, 0, 5, 1, 4, 2])
    b0p = synth.Basis(0, nv, b0.K, b0.tau, b0.vib[perm], b0.kstart, b0.kblock)   # case i holds quanta perm[i]
    for b, name in ((b0p, "j0eigen_quanta0.chk"), (b1, "j0eigen_quanta1.chk")):
        trove_files.write_quanta(str(tmp_path / name), b, synth.make_inflation(b, synth.classes_of(b, "full"), 1), 1)
    got = gainls.trove_basis(str(tmp_path), 1, 1, [1])
    inv = np.argsort(perm)
    np.testing.assert_array_equal(got["vib"], inv[b1.vib])


@pytest.mark.parametrize("max_bytes", [1 << 40, 3 * 12 * 12 * 8 // 3, 1000])
def test_dipole_is_flipped_and_blocked_like_the_reference(trove_dir, max_bytes):
    import gainls
    d, p = trove_dir
    n, pieces = gainls.trove_dipole(os.path.join(d, "j0_extfield.chk"), max_bytes)
    nv = p.dipole.shape[-1]
    assert n == nv
    nblocks = 3 * nv * nv * 8 // max_bytes + 1
    per = int(np.ceil(np.float32(nv) / np.float32(nblocks)))
    assert len(pieces) == nblocks
    for b, (s, e, c, piece) in enumerate(pieces):
        assert (s, e) == (b * per, min((b + 1) * per, nv)) and c == e - s
        np.testing.assert_array_equal(piece, np.ascontiguousarray(p.dipole[:, :, s:e]).reshape(-1))


def test_states_filter_and_rotational_labels(trove_dir):
    import gainls
    d, p = trove_dir
    blk = p.blocks[(2, 1)]
    f = gainls.make_filters([1.0, 1.0, 1.0, 1.0], p.isym_pairs, p.igamma_pair, p.sym_degen, (0.0, 1500.0),
                            (6000.0, 7000.0))
    st, dim = gainls.trove_states(d, 2, 1, f)
    e = blk.energies
    keep = ((e >= 0.0) & (e <= 1500.0)) | ((e >= 6000.0) & (e <= 7000.0))
    assert dim == blk.vecs.shape[1]
    np.testing.assert_array_equal(st["ilevel"], np.nonzero(keep)[0])
    np.testing.assert_array_equal(st["energy"], e[keep])
    np.testing.assert_array_equal(st["irec"], st["ilevel"])
    assert (st["rec_len"] == dim).all()
    f0 = gainls.make_filters([1.0, 0.0, 1.0, 1.0], p.isym_pairs, p.igamma_pair, p.sym_degen, (0.0, 1e9), (0.0, 1e9))
    st0, _ = gainls.trove_states(d, 2, 1, f0)   # isym_do false for this symmetry
    assert len(st0) == 0


def test_vector_records(trove_dir):
    import gainls
    d, p = trove_dir
    blk = p.blocks[(1, 3)]
    recs = [4, 0, len(blk.energies) - 1]
    v = gainls.trove_vectors(os.path.join(d, "j0eigen_vectors1_4.chk"), blk.vecs.shape[1], recs)
    np.testing.assert_array_equal(v, blk.vecs[recs])


def test_malformed_files_are_reported(tmp_path, trove_dir):
    import gainls
    d, p = trove_dir
    with pytest.raises(gainls.GainError, match="not found"):
        gainls.trove_dipole(str(tmp_path / "missing.chk"))
    bad = tmp_path / "j0_extfield.chk"
    raw = open(os.path.join(d, "j0_extfield.chk"), "rb").read()
    bad.write_bytes(raw.replace(b"Start external field", b"Start external fielX"))
    with pytest.raises(gainls.GainError, match="bogus header"):
        gainls.trove_dipole(str(bad))
    for name in ("j0eigen_quanta0.chk", "j0eigen_quanta1.chk"):
        text = open(os.path.join(d, name)).read()
        (tmp_path / name).write_text(text.replace("End irreducible transformation", "End"))
    with pytest.raises(gainls.GainError, match="irrep-footer"):
        gainls.trove_basis(str(tmp_path), 1, p.nsym, p.sym_degen)
    with pytest.raises(gainls.GainError):
        gainls.trove_vectors(os.path.join(d, "j0eigen_vectors1_4.chk"), 10 ** 6, [3])
