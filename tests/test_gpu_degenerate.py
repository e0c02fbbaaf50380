"""Degenerate symmetries in the batched engine (rule c3e: A1, A2 and a doubly degenerate E).

Each component pair (idegI, idegF) of a block pair is computed with the vectors expanded by
transform_vector_primitive's ideg (GPU/dipole_GPU.cu:859-889) and checked against the
oracle's double-double restatement of the reference loop; the line assembly combines the
component slots as Output::OutputLinestrength does (BaseClasses/Output.cpp:78-91): the sum of
amp^2 over the pairs passing DegeneracyFilter, idegF outer, divided by ndegI, times ndegI
when SYMMETRY REDUCED and both states are degenerate.  S is compared bit for bit with the
oracle's orc_line on the engine's own component amplitudes, and the text with the oracle's
sprintf of the same doubles."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

JMAX = 11
E = 2   # the degenerate symmetry of rule c3e


def _oracle(p, jI, gI, jF, gF, lo, up, comps):
    import oracle
    import threej
    return oracle.run_pair(p, jI, gI, jF, gF, lo, up, threej.threej_table(JMAX), JMAX, oracle.DD, 4,
                           components=comps)


def _filters(p, reduced=False, symmetry_type=1):
    import gainls
    return gainls.make_filters([1.0] * p.nsym, p.isym_pairs, p.igamma_pair, p.sym_degen, (-1e9, 1e9), (-1e9, 1e9),
                               reduced=reduced, symmetry_type=symmetry_type)


@pytest.fixture(scope="module")
def ee_problem(built_lib):
    import synth
    return synth.make_problem(40, [3, 4], "c3e", blocks=[(3, E), (4, E), (3, 0), (4, 1)])


@pytest.mark.parametrize("path", ["plain", "split"])
def test_component_pairs_match_oracle(ee_problem, path):
    import gainls
    p = ee_problem
    eng = gainls.Engine(JMAX, p.nsym, 2)
    gainls.upload_problem(eng, p)
    lo = list(range(0, p.blocks[(0, E)].vecs.shape[0], 3))
    up = list(range(p.blocks[(1, E)].vecs.shape[0]))
    pth = gainls.PATH_PLAIN_FP64 if path == "plain" else gainls.PATH_SPLIT
    for comps in ((0, 0), (1, 0), (0, 1), (1, 1)):
        ref = _oracle(p, 0, E, 1, E, lo, up, comps)
        st = eng.run_pair(0, E, 1, E, lo, up, pth, components=comps)
        assert st["status"] == gainls.OK, st
        amp = eng.fetch_amp()
        scale = np.abs(ref).max()
        assert scale > 0
        assert np.max(np.abs(amp - ref)) <= (1e-13 if path == "plain" else 1e-11) * scale, comps
    # the components differ from one another (the expansion's ideg is really used)
    eng.run_pair(0, E, 1, E, lo, up, pth, components=(0, 0))
    a00 = eng.fetch_amp().copy()
    eng.run_pair(0, E, 1, E, lo, up, pth, components=(1, 1))
    assert not np.allclose(a00, eng.fetch_amp())


@pytest.mark.parametrize("reduced,symmetry_type", [(False, 1), (True, 2)])
def test_degenerate_lines_match_oracle(ee_problem, reduced, symmetry_type):
    import gainls
    import oracle
    p = ee_problem
    eng = gainls.Engine(JMAX, p.nsym, 2)
    gainls.upload_problem(eng, p)
    lo = list(range(0, p.blocks[(0, E)].vecs.shape[0], 2))
    up = list(range(p.blocks[(1, E)].vecs.shape[0]))
    f = _filters(p, reduced, symmetry_type)
    st = eng.run_pair(0, E, 1, E, lo, up, gainls.PATH_SPLIT, filters=f)
    assert st["status"] == gainls.OK, st
    # the component amplitudes the lines combine, fetched one by one
    passing = [(dI, dF) for dF in range(2) for dI in range(2) if gainls.degeneracy_filter(f, E, E, dI, dF)]
    assert passing == ([(0, 0), (1, 0), (0, 1), (1, 1)] if symmetry_type == 1 else [(1, 0)])
    slots = np.zeros((len(lo), len(up), 4))
    for dI, dF in passing:
        eng.run_pair(0, E, 1, E, lo, up, gainls.PATH_SPLIT, components=(dI, dF))
        slots[:, :, dI + 2 * dF] = eng.fetch_amp()
    eI = p.blocks[(0, E)].energies[lo]
    eF = p.blocks[(1, E)].energies[up]
    kw = dict(temperature=500.0, q_part=3.0, zpe=10.0, thresh=0.0, freq=(-1e9, 1e9), gnsF=2.0)
    out = eng.lines(eI, eF, 3, 4, ndeg=(2, 2), reduced=reduced, **kw)
    flt = oracle.Filters([3, 4], [2.0] * 3, p.isym_pairs, p.igamma_pair, p.sym_degen, (-1e9, 1e9), (-1e9, 1e9),
                         reduced=reduced, symmetry_type=symmetry_type, temperature=500.0, q_part=3.0, zpe=10.0,
                         thresh=0.0)
    mask = np.zeros(4, np.uint8)
    for dI, dF in passing:
        mask[dI + 2 * dF] = 1
    bad = 0
    for r in range(len(lo)):
        for c in range(len(up)):
            res = oracle.line(slots[r, c], mask, 2, 2, 2, flt, eI[r], eF[c], 3, 4, E)
            if res is not None:
                S, A, I = res
                bad += S != out["S"][r, c] or A != out["A"][r, c]
                bad += abs(I - out["I"][r, c]) > 2e-15 * abs(I)   # device and host exp may differ by 1 ulp
            assert (res is not None) == bool(out["keep"][r, c])
    assert bad == 0
    # the text: line by line what the oracle's sprintf writes for the same doubles
    text, n = eng.lines_text(eI, eF, 3, 4, E, E, intensity=False, amplitudes=True, ndeg=(2, 2), reduced=reduced, **kw)
    want = []
    for r in range(len(lo)):
        for c in range(len(up)):
            nu = eF[c] - eI[r]
            if not out["keep"][r, c]:
                continue
            amps = [slots[r, c, dI + 2 * dF] for dI, dF in passing]
            want.append(oracle.line_text(nu, up[c], 4, E, lo[r], 3, E, out["A"][r, c], amps=amps))
    assert n == len(want)
    assert bytes(text).decode() == "".join(want)


def test_nondegenerate_pair_in_a_degenerate_engine(ee_problem):
    """A1 -> A2 in an engine built for maxdeg 2: gain_run_pair and the ndeg 1 lines as before."""
    import gainls
    p = ee_problem
    eng = gainls.Engine(JMAX, p.nsym, 2)
    gainls.upload_problem(eng, p)
    lo = list(range(p.blocks[(0, 0)].vecs.shape[0]))
    up = list(range(p.blocks[(1, 1)].vecs.shape[0]))
    ref = _oracle(p, 0, 0, 1, 1, lo, up, (0, 0))
    st = eng.run_pair(0, 0, 1, 1, lo, up, gainls.PATH_SPLIT)
    assert st["status"] == gainls.OK
    amp = eng.fetch_amp()
    assert np.max(np.abs(amp - ref)) <= 1e-11 * np.abs(ref).max()
    out = eng.lines(p.blocks[(0, 0)].energies, p.blocks[(1, 1)].energies, 3, 4)
    assert np.array_equal(out["S"], amp * amp)


def test_degenerate_argument_errors(ee_problem):
    import gainls
    p = ee_problem
    eng = gainls.Engine(JMAX, p.nsym, 2)
    gainls.upload_problem(eng, p)
    lo, up = [0, 1, 2], [0, 1, 2, 3]
    eI = p.blocks[(0, E)].energies[lo]
    eF = p.blocks[(1, E)].energies[up]
    with pytest.raises(gainls.GainError):   # component outside the degeneracy of A1
        eng.run_pair(0, 0, 1, 1, lo, up, gainls.PATH_PLAIN_FP64, components=(1, 0))
    eng.run_pair(0, E, 1, E, lo, up, gainls.PATH_PLAIN_FP64)   # no component slot
    with pytest.raises(gainls.GainError, match="component"):
        eng.lines(eI, eF, 3, 4, ndeg=(2, 2))
    with pytest.raises(gainls.GainError):   # ndeg above the engine's maxdeg
        eng.lines(eI, eF, 3, 4, ndeg=(3, 1))
    # slots of another job do not serve this one
    eng.run_pair(0, E, 1, E, lo, up, gainls.PATH_PLAIN_FP64, components=(0, 0))
    eng.run_pair(0, E, 1, E, lo, up[:3], gainls.PATH_PLAIN_FP64)
    with pytest.raises(gainls.GainError, match="component"):
        eng.lines(eI, eF[:3], 3, 4, ndeg=(2, 2))
    # an engine whose maxdeg is below the tables' degeneracy refuses them
    eng1 = gainls.Engine(JMAX, p.nsym, 1)
    b = p.bases[0]
    eng1.upload_basis(0, b.J, b.K, b.tau, b.vib, b.kblock, b.kstart)
    inf = p.infl[0]
    with pytest.raises(gainls.GainError, match="maxdeg"):
        eng1.upload_inflation(0, inf.icontr, inf.ijterms, b.dimen, inf.maxcoeff, inf.matsize, inf.N, inf.repres,
                              inf.Ntot, inf.sdeg)


@pytest.mark.parametrize("reduced,symmetry_type,precision,tol", [(False, 1, "f64", 1e-11), (True, 2, "f64", 1e-11),
                                                                (False, 1, "f32", 2e-5)])
def test_degenerate_adjoint_exact_directions(ee_problem, reduced, symmetry_type, precision, tol):
    """gain_adjoint_pair_degenerate: for Phi = sum w S with S combined over the passing component
    pairs as the line assembly forms it, dPhi/dmu . d = sum w r sum_c 2 amp_c(mu) amp_c(d)
    exactly (amp_c is linear in mu; r = 1/ndegI, or 1 when reduced with both states
    degenerate), amp_c(d) the plain FP64 forward of component pair c for the dipole d."""
    import gainls
    p = ee_problem
    nv = p.dipole.shape[-1]
    eng = gainls.Engine(JMAX, p.nsym, 2)
    gainls.upload_problem(eng, p)
    lo = list(range(0, p.blocks[(0, E)].vecs.shape[0], 2))
    up = list(range(p.blocks[(1, E)].vecs.shape[0]))
    f = _filters(p, reduced, symmetry_type)
    passing = [(dI, dF) for dF in range(2) for dI in range(2) if gainls.degeneracy_filter(f, E, E, dI, dF)]
    r = 1.0 if (reduced and True) else 0.5
    rng = np.random.default_rng(17)
    w = rng.standard_normal((len(lo), len(up)))
    # the lines' S equals r sum_c amp_c^2 (so w is a gradient over exactly those S)
    eng.run_pair(0, E, 1, E, lo, up, gainls.PATH_PLAIN_FP64, filters=f)
    S = eng.lines(p.blocks[(0, E)].energies[lo], p.blocks[(1, E)].energies[up], 3, 4, ndeg=(2, 2),
                  reduced=reduced, want=("S",))["S"]
    amp0 = {}
    for c in passing:
        eng.run_pair(0, E, 1, E, lo, up, gainls.PATH_PLAIN_FP64, components=c)
        amp0[c] = eng.fetch_amp().copy()
    assert np.allclose(S, r * sum(a * a for a in amp0.values()), rtol=1e-14, atol=0)
    grad = eng.adjoint(0, E, 1, E, lo, up, w, np.zeros(p.dipole.size), precision=precision, filters=f)
    grad = grad.reshape(p.dipole.shape)
    assert np.abs(grad).max() > 0
    for _ in range(2):
        d = rng.standard_normal(p.dipole.shape)
        eng.upload_dipole(np.ascontiguousarray(d).reshape(-1), nv, 0, nv, nv)
        terms = np.zeros_like(w)
        for c in passing:
            eng.run_pair(0, E, 1, E, lo, up, gainls.PATH_PLAIN_FP64, components=c)
            terms += w * r * 2.0 * amp0[c] * eng.fetch_amp()
        eng.upload_dipole(np.ascontiguousarray(p.dipole).reshape(-1), nv, 0, nv, nv)
        assert abs(np.sum(grad * d) - terms.sum()) <= tol * np.abs(terms).sum()


def test_plain_adjoint_refuses_degenerate_pairs(ee_problem):
    import gainls
    p = ee_problem
    eng = gainls.Engine(JMAX, p.nsym, 2)
    gainls.upload_problem(eng, p)
    with pytest.raises(gainls.GainError, match="degenerate"):
        eng.adjoint(0, E, 1, E, [0, 1], [0, 1, 2], np.ones((2, 3)), np.zeros(p.dipole.size))
