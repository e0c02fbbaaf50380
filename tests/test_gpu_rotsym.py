"""The engine's rotational-symmetry (Euler) form: block pairs whose Wigner table is uploaded
run with the dense-in-K matrix of the reference's rotsym kernel (GPU/dipole_GPU.cu:641-723).
Both paths are checked against amplitudes built from the oracle's double-double restatement
of that kernel (expansion -> rotsym half_ls -> dot products, the loop of
GpuManager::ExecuteRotSymHalfLs and ExecuteDotProduct)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

JMAX = 11
S_REL_TOL = 1e-8


def _oracle_amp(p, jI, gI, jF, gF, lo, up, block=None):
    import oracle
    import synth
    bI, bF = p.bases[jI], p.bases[jF]
    iI, iF = p.infl[jI], p.infl[jF]
    nv = p.dipole.shape[-1]
    s, e = block if block is not None else (0, nv)
    piece = np.ascontiguousarray(p.dipole[:, :, s:e]).reshape(-1)
    wig = synth.make_wigner(bI.J, bF.J, 1)
    nI, nF = synth.rotsym_levels(bI.J), synth.rotsym_levels(bF.J)
    up_prim = [oracle.expand(iF, gF, p.blocks[(jF, gF)].vecs[u], mode=oracle.DD) for u in up]
    amp = np.zeros((len(lo), len(up)))
    for a, l in enumerate(lo):
        prim = oracle.expand(iI, gI, p.blocks[(jI, gI)].vecs[l], mode=oracle.DD)
        h = np.zeros(bF.dimen)
        oracle.hls_rotsym(bI, bF, nI, nF, 1, piece, nv, (s, e, e - s), wig, prim, h, oracle.DD)
        for b, pu in enumerate(up_prim):
            amp[a, b] = oracle.dot(pu, h, oracle.DD)
    return amp


def _s_rel_err(amp, ref):
    S, Sr = amp ** 2, ref ** 2
    m = Sr > 1e-10 * Sr.max()
    return float(np.max(np.abs(S[m] - Sr[m]) / Sr[m]))


@pytest.fixture(scope="module")
def rot_problem(built_lib):
    import gainls
    import synth
    p = synth.make_problem(24, [3, 4], "c4r", blocks=[(3, 0), (4, 1), (4, 0), (3, 1)])
    eng = gainls.Engine(JMAX, p.nsym, 1)
    gainls.upload_problem(eng, p)
    return p, eng


@pytest.mark.parametrize("pair", [(0, 0, 1, 1), (1, 1, 0, 0), (1, 0, 1, 1)])
def test_plain_path_rotsym_matches_oracle(rot_problem, pair):
    import gainls
    p, eng = rot_problem
    jI, gI, jF, gF = pair
    lo = list(range(p.blocks[(jI, gI)].vecs.shape[0]))
    up = list(range(p.blocks[(jF, gF)].vecs.shape[0]))
    eng.run_pair(jI, gI, jF, gF, lo, up, gainls.PATH_PLAIN_FP64)
    amp = eng.fetch_amp()
    ref = _oracle_amp(p, jI, gI, jF, gF, lo, up)
    assert np.max(np.abs(amp - ref)) <= 1e-12 * np.abs(ref).max()


@pytest.mark.parametrize("pair", [(0, 0, 1, 1), (1, 1, 0, 0), (1, 0, 1, 1)])
def test_split_path_rotsym_matches_oracle(rot_problem, pair):
    """The split path with the dense band: the first GEMM then splits its inner dimension
    into chunks (8-bit digits), like the amplitude GEMM."""
    import gainls
    p, eng = rot_problem
    jI, gI, jF, gF = pair
    lo = list(range(p.blocks[(jI, gI)].vecs.shape[0]))
    up = list(range(p.blocks[(jF, gF)].vecs.shape[0]))
    st = eng.run_pair(jI, gI, jF, gF, lo, up, gainls.PATH_SPLIT)
    assert st["status"] == gainls.OK, st
    assert st["beta1"] == 8
    amp = eng.fetch_amp()
    ref = _oracle_amp(p, jI, gI, jF, gF, lo, up)
    assert _s_rel_err(amp, ref) <= S_REL_TOL
    assert np.max(np.abs(amp - ref)) <= 1e-11 * np.abs(ref).max()


def test_rotsym_and_kblock_pairs_coexist_in_one_engine(built_lib):
    """A Wigner table switches only its own (J'', J') pair to the rotsym form; with a dipole
    block only the listed upper vibrational range contributes."""
    import gainls
    import synth
    p = synth.make_problem(16, [2, 3], "c4r", blocks=[(2, 0), (3, 1)])
    eng = gainls.Engine(JMAX, p.nsym, 1)
    gainls.upload_problem(eng, p, dipole_block=(4, 12))
    lo = list(range(p.blocks[(0, 0)].vecs.shape[0]))
    up = list(range(p.blocks[(1, 1)].vecs.shape[0]))
    ref = _oracle_amp(p, 0, 0, 1, 1, lo, up, block=(4, 12))
    for path in (gainls.PATH_PLAIN_FP64, gainls.PATH_SPLIT):
        eng.run_pair(0, 0, 1, 1, lo, up, path)
        amp = eng.fetch_amp()
        assert np.max(np.abs(amp - ref)) <= 1e-11 * np.abs(ref).max()
