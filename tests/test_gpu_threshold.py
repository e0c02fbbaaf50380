"""Line-list membership under THRESH_LINE (BaseClasses/Output.cpp:95-96: a line is written
only when A >= THRESH_LINE) on the split path.

A split-path amplitude carries a certified error bound; a line whose A lies within that bound
of the threshold could fall on either side, so the line assembly recomputes it with the
plain FP64 path before deciding.  The threshold is set within 1e-14 (relative) of one line's
A -- well inside the split path's bound and well outside FP64 rounding -- on each side, and
the kept lines and the line text (no intensity column) must equal the oracle's, computed
from double-double amplitudes; the non-degenerate form and the degenerate component slots
(rule c3e, E -> E) are both covered."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

JMAX = 11
E = 2


def _dd(p, jI, gI, jF, gF, lo, up, comps=(0, 0)):
    import oracle
    import threej
    return oracle.run_pair(p, jI, gI, jF, gF, lo, up, threej.threej_table(JMAX), JMAX, oracle.DD, 4,
                           components=comps)


@pytest.mark.parametrize("side", [+1, -1])
def test_threshold_membership_matches_oracle(built_lib, side):
    import gainls
    import oracle
    import synth
    p = synth.make_problem(60, [4, 5], "c4", blocks=[(4, 0), (5, 1)])
    eng = gainls.Engine(JMAX, p.nsym, 1)
    gainls.upload_problem(eng, p)
    bI, bF = p.blocks[(0, 0)], p.blocks[(1, 1)]
    lo, up = list(range(bI.vecs.shape[0])), list(range(bF.vecs.shape[0]))
    eI, eF = bI.energies, bF.energies
    # the threshold: next to the line of median A (the plain FP64 path's A), on one side
    eng.run_pair(0, 0, 1, 1, lo, up, gainls.PATH_PLAIN_FP64)
    A = eng.lines(eI, eF, 4, 5, intensity=False, want=("A", "keep"))
    kept = A["A"][A["keep"].astype(bool)]
    a_med = float(np.sort(kept)[kept.size // 2])
    thresh = a_med * (1.0 + side * 1e-14)
    assert eng.threshold_refined() == 0
    # split path: the line near the threshold is recomputed in FP64
    st = eng.run_pair(0, 0, 1, 1, lo, up, gainls.PATH_SPLIT)
    assert st["status"] == gainls.OK
    text, n = eng.lines_text(eI, eF, 4, 5, 0, 1, intensity=False, thresh=thresh)
    assert eng.threshold_refined() >= 1
    # the text is the oracle's sprintf of the amplitudes the line assembly used (the split
    # ones, with the near-threshold line recomputed in FP64) ...
    used = eng.fetch_amp().copy()
    want, n_want = oracle.line_list(used, eI, eF, lo, up, 4, 5, 0, 1, thresh=thresh, intensity=False)
    assert (n, bytes(text)) == (n_want, want)
    # ... and its lines are those the double-double amplitudes keep (nu and the state labels
    # of every line; A's tenth digit may differ with the amplitudes' last bits)
    amp_dd = _dd(p, 0, 0, 1, 1, lo, up)
    ref, n_ref = oracle.line_list(amp_dd, eI, eF, lo, up, 4, 5, 0, 1, thresh=thresh, intensity=False)
    assert n == n_ref
    assert [l[:53] for l in bytes(text).decode().splitlines()] == [l[:53] for l in ref.decode().splitlines()]
    # keep from the line assembly as well (after a fresh split run, so the check runs again)
    eng.run_pair(0, 0, 1, 1, lo, up, gainls.PATH_SPLIT)
    out = eng.lines(eI, eF, 4, 5, intensity=False, thresh=thresh, want=("A", "keep"))
    assert eng.threshold_refined() >= 1
    keep_dd = np.zeros_like(out["keep"])
    for r in range(len(lo)):
        for c in range(len(up)):
            S = amp_dd[r, c] ** 2
            nu = eF[c] - eI[r]
            Add = 3.13618923e-7 * 9 * S * abs(nu) ** 3
            keep_dd[r, c] = nu >= 1e-40 and Add >= thresh
    np.testing.assert_array_equal(out["keep"], keep_dd)


def test_degenerate_slots_threshold_membership(built_lib):
    import gainls
    import synth
    p = synth.make_problem(40, [3, 4], "c3e", blocks=[(3, E), (4, E)])
    eng = gainls.Engine(JMAX, p.nsym, 2)
    gainls.upload_problem(eng, p)
    bI, bF = p.blocks[(0, E)], p.blocks[(1, E)]
    lo = list(range(0, bI.vecs.shape[0], 2))
    up = list(range(bF.vecs.shape[0]))
    eI, eF = bI.energies[lo], bF.energies[up]
    f = gainls.make_filters([1.0] * p.nsym, p.isym_pairs, p.igamma_pair, p.sym_degen, (-1e9, 1e9), (-1e9, 1e9))
    comps = [(0, 0), (1, 0), (0, 1), (1, 1)]
    dd = {c: _dd(p, 0, E, 1, E, lo, up, c) for c in comps}
    S_dd = sum(dd[c] ** 2 for c in comps) / 2.0
    nu = eF[None, :] - eI[:, None]
    A_dd = 3.13618923e-7 * 7 * S_dd * np.abs(nu) ** 3
    ok = nu >= 1e-40
    a_med = float(np.sort(A_dd[ok])[A_dd[ok].size // 2])
    for side in (+1, -1):
        thresh = a_med * (1.0 + side * 1e-14)
        st = eng.run_pair(0, E, 1, E, lo, up, gainls.PATH_SPLIT, filters=f)
        assert st["status"] == gainls.OK
        out = eng.lines(eI, eF, 3, 4, ndeg=(2, 2), intensity=False, thresh=thresh, want=("A", "keep"))
        assert eng.threshold_refined() >= 1
        np.testing.assert_array_equal(out["keep"].astype(bool), ok & (A_dd >= thresh))
