"""The split path with an expansion that mixes primitives (rule c4m: every symmetric function
of a K >= 1 case is (p0 +- p1)/sqrt(2), as TROVE's symmetry-adapted functions combine the
components of a case), in both of its forms: the band formed over symmetric functions, and
GEMM1 over primitives (lower vectors expanded before it, H contracted with the upper
expansion after it).  Amplitudes are checked against the oracle's double-double restatement
of the reference loop (expand -> half_ls -> expand -> dot), single CTAs and CTA pairs, with a
dipole block and with dipole pieces."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

JMAX = 11


def _oracle(p, jI, gI, jF, gF, lo, up, block=None):
    import oracle
    import threej
    return oracle.run_pair(p, jI, gI, jF, gF, lo, up, threej.threej_table(JMAX), JMAX, oracle.DD, 4,
                           dipole_block=block)


def _s_rel(amp, ref):
    S, Sr = amp ** 2, ref ** 2
    m = Sr > 1e-10 * Sr.max()
    return float(np.max(np.abs(S[m] - Sr[m]) / Sr[m]))


@pytest.fixture(params=["symband", "primitive"])
def split_form(request, monkeypatch):
    """Both forms of the split path for mixing expansions: the band over symmetric functions
    (every function here combines primitives of one K) and GEMM1 over primitives with the
    contraction after it (GAINLS_SPLIT_FORM=primitive)."""
    if request.param == "primitive":
        monkeypatch.setenv("GAINLS_SPLIT_FORM", "primitive")
    else:
        monkeypatch.delenv("GAINLS_SPLIT_FORM", raising=False)
    return request.param


@pytest.mark.parametrize("nv,jv", [(16, (2, 3)), (80, (3, 4))])
def test_mixed_expansion_split_and_plain_match_oracle(built_lib, split_form, nv, jv):
    import gainls
    import synth
    p = synth.make_problem(nv, list(jv), "c4m", blocks=[(jv[0], 0), (jv[1], 1)])
    eng = gainls.Engine(JMAX, p.nsym, 1)
    gainls.upload_problem(eng, p)
    lo = list(range(p.blocks[(0, 0)].vecs.shape[0]))
    up = list(range(p.blocks[(1, 1)].vecs.shape[0]))
    ref = _oracle(p, 0, 0, 1, 1, lo, up)
    scale = np.abs(ref).max()
    eng.run_pair(0, 0, 1, 1, lo, up, gainls.PATH_PLAIN_FP64)
    assert np.max(np.abs(eng.fetch_amp() - ref)) <= 1e-13 * scale
    st = eng.run_pair(0, 0, 1, 1, lo, up, gainls.PATH_SPLIT)
    assert st["status"] == gainls.OK, st
    amp = eng.fetch_amp()
    assert np.max(np.abs(amp - ref)) <= 1e-11 * scale
    assert _s_rel(amp, ref) <= 1e-8
    if split_form == "primitive":
        assert st["kernel_launches"] >= 9   # expansion and contraction run too


def test_mixed_expansion_with_dipole_block_and_pieces(built_lib, split_form):
    import gainls
    import synth
    p = synth.make_problem(24, [2, 3], "c4m", blocks=[(2, 1), (3, 0)])
    nv = p.dipole.shape[-1]
    eng = gainls.Engine(JMAX, p.nsym, 1)
    gainls.upload_problem(eng, p, dipole_block=(5, 19))
    lo = list(range(p.blocks[(0, 1)].vecs.shape[0]))
    up = list(range(p.blocks[(1, 0)].vecs.shape[0]))
    ref = _oracle(p, 0, 1, 1, 0, lo, up, block=(5, 19))
    st = eng.run_pair(0, 1, 1, 0, lo, up, gainls.PATH_SPLIT)
    assert st["status"] == gainls.OK
    assert np.max(np.abs(eng.fetch_amp() - ref)) <= 1e-11 * np.abs(ref).max()
    bounds = [0, 7, 15, nv]
    eng.upload_dipole_pieces([(s, e, np.ascontiguousarray(p.dipole[:, :, s:e]).reshape(-1))
                              for s, e in zip(bounds, bounds[1:])], nv)
    ref = _oracle(p, 0, 1, 1, 0, lo, up)
    st = eng.run_pair(0, 1, 1, 0, lo, up, gainls.PATH_SPLIT)
    assert st["status"] == gainls.OK
    assert np.max(np.abs(eng.fetch_amp() - ref)) <= 1e-11 * np.abs(ref).max()
