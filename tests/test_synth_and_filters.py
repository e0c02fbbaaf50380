"""The synthetic stand-in for TROVE inputs and the state-selection rules.

Basis sets must satisfy the reference's K-block assumptions (TroveClasses/TroveBasisSet.cpp:
659-681), expansion tables must be the selection the reference's expansion kernel
reproduces, and the transition set is the one main.cpp:238-296 visits."""
import numpy as np
import pytest


def test_basis_k_blocks():
    import synth
    for J, nv in [(0, 5), (1, 3), (4, 7), (11, 2)]:
        b = synth.make_basis(J, nv)
        assert b.dimen == nv * (2 * J + 1)
        assert np.all(np.diff(b.K) >= 0)
        for k in range(J + 1):
            blk = slice(b.kstart[k], b.kstart[k] + b.kblock[k])
            assert np.all(b.K[blk] == k)
            assert b.kblock[k] == (nv if k == 0 else 2 * nv)
            if k == 0:
                assert np.all(b.tau[blk] == J % 2)
        assert b.kstart[J] + b.kblock[J] == b.dimen


def test_classes_partition_and_pairing():
    import synth
    b = synth.make_basis(6, 8)
    c = synth.classes_of(b, "c4")
    assert set(np.unique(c)) <= {0, 1, 2, 3}
    inf = synth.make_inflation(b, c, 4)
    assert int(inf.Ntot.sum()) == b.dimen
    pair = synth.igamma_pair_of(synth.selection_of("c4"))
    assert list(pair) == [1, 0, 3, 2]
    assert list(synth.igamma_pair_of(synth.selection_of("full"))) == [0]


def test_expansion_is_selection(oracle_lib):
    import oracle
    import synth
    b = synth.make_basis(3, 6)
    c = synth.classes_of(b, "c4")
    inf = synth.make_inflation(b, c, 4)
    for g in range(4):
        v = np.arange(1, inf.Ntot[g] + 1, dtype=np.float64)
        prim = oracle.expand(inf, g, v)
        assert np.array_equal(prim[inf.members[g]], v)
        mask = np.ones(b.dimen, bool)
        mask[inf.members[g]] = False
        assert np.all(prim[mask] == 0)


def test_dipole_and_eigvecs():
    import synth
    d = synth.make_dipole(30)
    assert d.shape == (3, 30, 30)
    assert np.array_equal(d, np.transpose(d, (0, 2, 1)))
    assert np.array_equal(d, synth.make_dipole(30))
    q = synth.make_eigvecs(40, 2, 1)
    assert np.allclose(q @ q.T, np.eye(40), atol=1e-13)
    e = synth.make_energies(40, 2, 1)
    assert np.all(np.diff(e) >= 0) and e.min() >= 0 and e.max() <= 8000


def _filters(p, **kw):
    import oracle
    args = dict(jvals=p.jvals, gns=[1.0] * p.nsym, isym_pairs=p.isym_pairs, igamma_pair=p.igamma_pair,
                sym_degen=p.sym_degen, erange_lower=(0, 3000), erange_upper=(0, 8000))
    args.update(kw)
    return oracle.Filters(**args)


def test_transition_selection_rules():
    import synth
    import oracle
    p = synth.make_problem(4, [0, 1, 2], "c4", max_levels=6)
    f = _filters(p)
    tr = oracle.transitions(p, f)
    assert tr
    maxJ = 2
    for I, F in tr:
        jI, jF = p.st_J[I], p.st_J[F]
        assert abs(jI - jF) <= 1 and jI + jF >= 1 and not (jI == maxJ and jF == maxJ)
        assert p.igamma_pair[p.st_gamma[I]] == p.st_gamma[F]
        assert p.st_energy[I] <= 3000
    # GNS = 0 disables a symmetry on both sides (TroveInput.cpp:296-306)
    f0 = _filters(p, gns=[0.0, 1.0, 1.0, 1.0])
    assert all(p.st_gamma[I] != 0 and p.st_gamma[F] != 0 for I, F in oracle.transitions(p, f0))
    # frequency window applies to nu = E_F - E_I
    fw = _filters(p, freq_window=(0.0, 1e9))
    assert all(p.st_energy[F] >= p.st_energy[I] for I, F in oracle.transitions(p, fw))


def test_degeneracy_filter_types():
    import oracle
    f = oracle.Filters([0, 1], [1.0] * 6, [1, 1, 2, 3, 3, 2], [1, 0, 5, 4, 3, 2], [1, 1, 2, 1, 1, 2],
                       (0, 1), (0, 1), reduced=True, symmetry_type=2)
    assert f.degeneracy_filter(0, 1, 0, 0)           # a non-degenerate side passes everything
    assert f.degeneracy_filter(2, 5, 1, 0)
    assert not f.degeneracy_filter(2, 5, 0, 0)
    f.reduced = False
    assert f.degeneracy_filter(2, 5, 0, 1)


def test_line_strength_formula(oracle_lib):
    """S, A, I of one line against the formulas of Output.cpp:78-102 evaluated by hand."""
    import oracle
    f = oracle.Filters([0, 1], [1.0], [1], [0], [1], (0, 1e4), (0, 1e4), temperature=296.0, q_part=2.5)
    amp = np.array([0.37])
    S, A, I = oracle.line(amp, [1], 1, 1, 1, f, 100.0, 1100.0, 0, 1, 0)
    assert S == 0.37 * 0.37
    assert A == 3.13618923e-7 * 1 * S * 1000.0 ** 3
    beta = 6.62606896e-27 * 2.99792458e+10 / (1.380658e-16 * 296.0)
    assert I == pytest.approx(1.327209365e-12 * A * 1.0 * 3.0 * np.exp(-beta * 100.0) *
                              (1 - np.exp(-beta * 1000.0)) / (1000.0 ** 2 * 2.5), rel=1e-14)
    assert oracle.line(amp, [1], 1, 1, 1, f, 100.0, 100.0, 0, 1, 0) is None   # nu < 1e-40 skipped


def test_mixed_expansion_is_orthonormal(oracle_lib):
    """Rule c4m: every symmetric function is a combination of the components of its case;
    the expansion T (the reference's expand kernel on unit vectors) has orthonormal columns,
    partitions the primitives over the four classes, and is not a selection."""
    import oracle
    import synth
    b = synth.make_basis(3, 6)
    inf = synth.make_mixed_inflation(b, 4)
    assert inf.matsize == 2 and int(inf.Ntot.sum()) == b.dimen
    cols = []
    for g in range(4):
        for s in range(int(inf.Ntot[g])):
            e = np.zeros(inf.Ntot[g])
            e[s] = 1.0
            cols.append(oracle.expand(inf, g, e))
    T = np.array(cols).T
    assert np.allclose(T.T @ T, np.eye(b.dimen), atol=1e-15)
    assert (np.count_nonzero(T, axis=0) == 2).sum() > 0   # mixed columns exist


def test_degenerate_expansion_is_orthonormal(oracle_lib):
    """Rule c3e: A1, A2 and both components of E together form an orthonormal expansion of
    the primitives (the reference's expand kernel on unit vectors, with ideg), and the E
    components are distinct functions."""
    import oracle
    import synth
    b = synth.make_basis(4, 6)
    inf = synth.make_degenerate_inflation(b)
    assert list(inf.sdeg) == [1, 1, 2] and inf.matsize == 2
    assert int(inf.Ntot[0] + inf.Ntot[1] + 2 * inf.Ntot[2]) == b.dimen
    cols = []
    for g in range(3):
        for ideg in range(int(inf.sdeg[g])):
            for s in range(int(inf.Ntot[g])):
                e = np.zeros(inf.Ntot[g])
                e[s] = 1.0
                cols.append(oracle.expand(inf, g, e, ideg=ideg))
    T = np.array(cols).T
    assert np.allclose(T.T @ T, np.eye(b.dimen), atol=1e-15)
    p = synth.make_problem(6, [1, 2], "c3e", blocks=[(1, 2), (2, 2)])
    assert list(p.sym_degen) == [1, 1, 2] and list(p.igamma_pair) == [1, 0, 2]
    assert set(p.st_ndeg.tolist()) == {2}


def test_oracle_pair_components_follow_the_expansion(oracle_lib):
    """oracle.run_pair with components (idegI, idegF) equals the dense restatement: both
    vectors expanded with their component (numpy over the tables), the half line strength of
    the lower primitive vector, its dot with the upper primitive vector."""
    import oracle
    import synth
    import threej
    jmax = 4
    p = synth.make_problem(8, [2, 3], "c3e", blocks=[(2, 2), (3, 2)])
    lo = [0, 3, 5]
    up = list(range(0, p.blocks[(1, 2)].vecs.shape[0], 4))
    tj = threej.threej_table(jmax)

    def dense_T(jind, ideg):
        inf, d = p.infl[jind], p.bases[jind].dimen
        nt, sd = int(inf.Ntot[2]), int(inf.sdeg[2])
        T = np.zeros((d, nt))
        for r in range(d):
            irow, ib = inf.icontr[r], inf.icontr[r + d]
            it = inf.ijterms[irow + 2 * inf.maxcoeff]
            for i in range(inf.N[2][irow]):
                T[r, it + i] = inf.repres[2][it + i + ideg * nt + ib * sd * nt]
        return T

    for comps in ((0, 0), (1, 0), (0, 1), (1, 1)):
        amp = oracle.run_pair(p, 0, 2, 1, 2, lo, up, tj, jmax, components=comps)
        TI, TF = dense_T(0, comps[0]), dense_T(1, comps[1])
        for a, l in enumerate(lo):
            h = oracle.half_ls(p.bases[0], p.bases[1], TI @ p.blocks[(0, 2)].vecs[l], p.dipole, tj, jmax)
            want = (TF @ p.blocks[(1, 2)].vecs[up].T).T @ h
            assert np.allclose(amp[a], want, rtol=0, atol=1e-12 * np.abs(want).max())
