"""gain_adjoint_pair: dL/dmu of a loss over one block pair's line strengths.

S = amp^2 is quadratic in the dipole, so for Phi(mu) = sum w S(mu) a central difference is
exact up to rounding: the adjoint must reproduce it along random directions and for single
entries, in the K-block and the rotational-symmetry forms, with and without a dipole block."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

JMAX = 11


def _phi(eng, p, piece, block, lo, up, w):
    import gainls
    nv = p.dipole.shape[-1]
    s, e = block
    eng.upload_dipole(np.ascontiguousarray(piece).reshape(-1), nv, s, e, e - s)
    eng.run_pair(0, 0, 1, 1, lo, up, gainls.PATH_PLAIN_FP64)
    return float(np.sum(w * eng.fetch_amp() ** 2))


@pytest.mark.parametrize("rule,block", [("c4", None), ("c4", (3, 13)), ("c4r", None)])
def test_adjoint_matches_central_differences(built_lib, rule, block):
    import gainls
    import synth
    p = synth.make_problem(16, [2, 3], rule, blocks=[(2, 0), (3, 1)])
    nv = p.dipole.shape[-1]
    blk = block or (0, nv)
    eng = gainls.Engine(JMAX, p.nsym, 1)
    gainls.upload_problem(eng, p, dipole_block=blk)
    lo = list(range(p.blocks[(0, 0)].vecs.shape[0]))
    up = list(range(p.blocks[(1, 1)].vecs.shape[0]))
    rng = np.random.default_rng(78)
    w = rng.standard_normal((len(lo), len(up)))
    piece0 = np.ascontiguousarray(p.dipole[:, :, blk[0]:blk[1]])
    grad = np.zeros(piece0.size)
    eng.adjoint(0, 0, 1, 1, lo, up, w, grad)
    grad = grad.reshape(piece0.shape)
    assert np.abs(grad).max() > 0
    scale = np.abs(grad).max()
    h = 1e-3
    for _ in range(3):   # random directions
        d = rng.standard_normal(piece0.shape)
        fd = (_phi(eng, p, piece0 + h * d, blk, lo, up, w) - _phi(eng, p, piece0 - h * d, blk, lo, up, w)) / (2 * h)
        assert abs(fd - np.sum(grad * d)) <= 1e-9 * scale * np.abs(d).sum()
    flat = np.flatnonzero(np.abs(grad.reshape(-1)) > 0)
    for k in rng.choice(flat, size=min(12, flat.size), replace=False):   # single entries
        d = np.zeros(piece0.size)
        d[k] = 1.0
        d = d.reshape(piece0.shape)
        fd = (_phi(eng, p, piece0 + h * d, blk, lo, up, w) - _phi(eng, p, piece0 - h * d, blk, lo, up, w)) / (2 * h)
        assert abs(fd - grad.reshape(-1)[k]) <= 1e-8 * scale


def test_adjoint_reuses_the_last_run_of_the_same_job(built_lib):
    """After a run of the same pair (either path) the adjoint takes its amplitudes; after an
    upload it runs its own FP64 forward.  The split path's amplitudes move the gradient by
    their certified error only."""
    import gainls
    import synth
    p = synth.make_problem(16, [2, 3], "c4", blocks=[(2, 0), (3, 1)])
    eng = gainls.Engine(JMAX, p.nsym, 1)
    gainls.upload_problem(eng, p)
    lo = list(range(p.blocks[(0, 0)].vecs.shape[0]))
    up = list(range(p.blocks[(1, 1)].vecs.shape[0]))
    w = np.random.default_rng(3).standard_normal((len(lo), len(up)))
    g_plain = eng.adjoint(0, 0, 1, 1, lo, up, w, np.zeros(p.dipole.size))
    eng.run_pair(0, 0, 1, 1, lo, up, gainls.PATH_SPLIT)
    g_split = eng.adjoint(0, 0, 1, 1, lo, up, w, np.zeros(p.dipole.size))
    assert np.max(np.abs(g_split - g_plain)) <= 1e-8 * np.abs(g_plain).max()
    # a different dipole: the stored amplitudes no longer apply
    eng.run_pair(0, 0, 1, 1, lo, up, gainls.PATH_PLAIN_FP64)
    nv = p.dipole.shape[-1]
    eng.upload_dipole((2.0 * p.dipole).reshape(-1), nv, 0, nv, nv)
    g2 = eng.adjoint(0, 0, 1, 1, lo, up, w, np.zeros(p.dipole.size))
    assert np.max(np.abs(g2 - 2.0 * g_plain)) <= 1e-12 * np.abs(g2).max()   # S = amp^2: dS/dmu doubles
