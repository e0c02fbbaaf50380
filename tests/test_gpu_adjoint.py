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


@pytest.mark.parametrize("rule", ["c4", "c4r"])
@pytest.mark.parametrize("precision,tol", [("f64", 1e-11), ("f32", 2e-5)])
def test_adjoint_exact_directions_several_tiles(built_lib, rule, precision, tol):
    """Blocks of several 64-function tiles per side, so the (F, I) tile list skips the tiles
    outside |K_I - K_F| <= 1 (K-block form) and keeps all of them (rotational-symmetry form).
    amp is linear in mu, so dPhi/dmu . d = sum w 2 amp(mu) amp(d) exactly, amp(d) being the
    FP64 forward of the dipole d.  FP32: the chain's products and sums round to FP32 (unit
    2^-24) over sums of a few hundred terms; tol is relative to sum |w 2 amp amp(d)|."""
    import gainls
    import synth
    p = synth.make_problem(64, [4, 5], rule, blocks=[(4, 0), (5, 1)])
    nv = p.dipole.shape[-1]
    eng = gainls.Engine(JMAX, p.nsym, 1)
    gainls.upload_problem(eng, p)
    lo = list(range(p.blocks[(0, 0)].vecs.shape[0]))
    up = list(range(p.blocks[(1, 1)].vecs.shape[0]))
    assert min(len(lo), len(up)) > 128
    rng = np.random.default_rng(91)
    w = rng.standard_normal((len(lo), len(up)))
    grad = eng.adjoint(0, 0, 1, 1, lo, up, w, np.zeros(p.dipole.size), precision=precision).reshape(p.dipole.shape)
    eng.run_pair(0, 0, 1, 1, lo, up, gainls.PATH_PLAIN_FP64)
    amp0 = eng.fetch_amp().copy()
    for _ in range(3):
        d = rng.standard_normal(p.dipole.shape)
        eng.upload_dipole(np.ascontiguousarray(d).reshape(-1), nv, 0, nv, nv)
        eng.run_pair(0, 0, 1, 1, lo, up, gainls.PATH_PLAIN_FP64)
        terms = w * 2.0 * amp0 * eng.fetch_amp()
        assert abs(np.sum(grad * d) - terms.sum()) <= tol * np.abs(terms).sum()
    # FP32 against FP64 entry by entry
    if precision == "f32":
        eng.upload_dipole(np.ascontiguousarray(p.dipole).reshape(-1), nv, 0, nv, nv)
        g64 = eng.adjoint(0, 0, 1, 1, lo, up, w, np.zeros(p.dipole.size)).reshape(p.dipole.shape)
        assert np.max(np.abs(grad - g64)) <= tol * np.abs(g64).max()
        assert np.array_equal(grad == 0, g64 == 0)


def test_adjoint_rejects_unknown_precision(built_lib):
    import ctypes
    import gainls
    import synth
    p = synth.make_problem(16, [2, 3], "c4", blocks=[(2, 0), (3, 1)])
    eng = gainls.Engine(JMAX, p.nsym, 1)
    gainls.upload_problem(eng, p)
    lo, up = np.arange(4, dtype=np.int32), np.arange(4, dtype=np.int32)
    job = gainls.PairJob(0, 0, 1, 1, 4, lo.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), 4,
                         up.ctypes.data_as(ctypes.POINTER(ctypes.c_int)))
    g, out = np.zeros(16), np.zeros(p.dipole.size)
    st = gainls.Stats()
    rc = gainls.lib().gain_adjoint_pair_prec(eng.h, ctypes.byref(job), g.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                             out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), 7, ctypes.byref(st))
    assert rc == gainls.ERR_INVALID_ARG


@pytest.mark.parametrize("rule,block", [("c4", None), ("c4", (3, 13)), ("c4r", None), ("c4m", None)])
def test_tensor_core_adjoint_matches_fp64(built_lib, rule, block):
    """GAIN_ADJOINT_SPLIT (both products as digit GEMMs on the tensor cores, 48-bit digits)
    against the FP64 chain: the same gradient to 1e-9 of its largest component; it also runs
    its own split forward when the job's amplitudes are not resident."""
    import gainls
    import synth
    p = synth.make_problem(40, [3, 4], rule, blocks=[(3, 0), (4, 1)])
    nv = p.dipole.shape[-1]
    blk = block or (0, nv)
    eng = gainls.Engine(JMAX, p.nsym, 1)
    gainls.upload_problem(eng, p, dipole_block=blk)
    lo = list(range(p.blocks[(0, 0)].vecs.shape[0]))
    up = list(range(p.blocks[(1, 1)].vecs.shape[0]))
    w = np.random.default_rng(11).standard_normal((len(lo), len(up)))
    size = 3 * nv * (blk[1] - blk[0])
    g64 = eng.adjoint(0, 0, 1, 1, lo, up, w, np.zeros(size), precision="f64")
    scale = np.abs(g64).max()
    assert scale > 0
    gtc = eng.adjoint(0, 0, 1, 1, lo, up, w, np.zeros(size), precision="split")   # reuses the FP64 forward
    assert np.max(np.abs(gtc - g64)) <= 1e-9 * scale
    assert eng.last_adjoint_stats.tensor_flops > 0
    nvb = blk[1] - blk[0]
    eng.upload_dipole(np.ascontiguousarray(p.dipole[:, :, blk[0]:blk[1]]).reshape(-1), nv, blk[0], blk[1], nvb)
    gtc2 = eng.adjoint(0, 0, 1, 1, lo, up, w, np.zeros(size), precision="split")   # its own split forward
    assert np.max(np.abs(gtc2 - g64)) <= 1e-9 * scale
    eng.close()


def test_tensor_core_adjoint_degenerate(built_lib):
    import gainls
    import synth
    p = synth.make_problem(30, [3, 4], "c3e", blocks=[(3, 2), (4, 2)])
    eng = gainls.Engine(JMAX, p.nsym, 2)
    gainls.upload_problem(eng, p)
    lo = list(range(p.blocks[(0, 2)].vecs.shape[0]))
    up = list(range(p.blocks[(1, 2)].vecs.shape[0]))
    f = gainls.make_filters([1.0] * p.nsym, p.isym_pairs, p.igamma_pair, p.sym_degen, (-1e9, 1e9), (-1e9, 1e9))
    w = np.random.default_rng(12).standard_normal((len(lo), len(up)))
    g64 = eng.adjoint(0, 2, 1, 2, lo, up, w, np.zeros(p.dipole.size), precision="f64", filters=f)
    gtc = eng.adjoint(0, 2, 1, 2, lo, up, w, np.zeros(p.dipole.size), precision="split", filters=f)
    assert np.max(np.abs(gtc - g64)) <= 1e-9 * np.abs(g64).max()
    eng.close()
