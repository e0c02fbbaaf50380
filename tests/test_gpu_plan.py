"""gain_run_plan: a plan of block pairs over several engines of one device (one host thread
and one stream each, largest jobs first).  Every job's amplitudes, read in its completion
callback, equal those of the same job run alone on one engine; a failing job stops the plan
with its status and names the job."""
import threading

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

JMAX = 11


@pytest.fixture(scope="module")
def plan_problem(built_lib):
    import gainls
    import synth
    p = synth.make_problem(24, [1, 2, 3, 4], "c4")
    filt = gainls.make_filters([1.0] * p.nsym, p.isym_pairs, p.igamma_pair, p.sym_degen, (0.0, 6000.0),
                               (-1e9, 1e9), (-1e9, 1e9), 0.0, 4)
    table = gainls.state_table(p.st_energy, p.st_J, p.st_jind, p.st_gamma, p.st_ndeg, p.st_ilevel)
    pairs = gainls.plan_pairs(filt, table)
    assert len(pairs) >= 8
    return p, pairs


def _engines(p, n):
    import gainls
    out = []
    for _ in range(n):
        e = gainls.Engine(JMAX, p.nsym, 1)
        gainls.upload_problem(e, p)
        out.append(e)
    return out


@pytest.mark.parametrize("path_name,n_engines", [("split", 3), ("plain", 2), ("split", 1)])
def test_plan_matches_single_engine_runs(plan_problem, path_name, n_engines):
    import gainls
    p, pairs = plan_problem
    path = gainls.PATH_SPLIT if path_name == "split" else gainls.PATH_PLAIN_FP64
    ref_eng = _engines(p, 1)[0]
    want = []
    for jI, gI, jF, gF, lo, up in pairs:
        ref_eng.run_pair(jI, gI, jF, gF, lo, up, path)
        want.append(ref_eng.fetch_amp().copy())
    engines = _engines(p, n_engines)
    got = [None] * len(pairs)
    threads = set()

    def done(job, eng, status):
        assert status == gainls.OK
        got[job] = eng.fetch_amp().copy()
        threads.add(threading.get_ident())

    stats = gainls.run_plan(engines, pairs, path, on_done=done)
    assert len(stats) == len(pairs) and all(s["rows"] == len(pr[4]) for s, pr in zip(stats, pairs))
    for j in range(len(pairs)):
        assert got[j] is not None, j
        assert np.array_equal(got[j], want[j]), j
    assert len(threads) <= n_engines


def test_plan_failure_names_the_job(plan_problem):
    import gainls
    p, pairs = plan_problem
    engines = _engines(p, 2)
    bad = list(pairs)
    jI, gI, jF, gF, lo, up = bad[3]
    bad[3] = (jI, gI, jF, gF, list(lo), list(up) + [10 ** 6])   # an upper level out of range
    seen = []
    with pytest.raises(gainls.GainError, match="job 3"):
        gainls.run_plan(engines, bad, gainls.PATH_SPLIT, on_done=lambda j, e, s: seen.append((j, s)))
    assert (3, gainls.ERR_INVALID_ARG) in seen
    # the engines stay usable
    jI, gI, jF, gF, lo, up = pairs[0]
    engines[1].run_pair(jI, gI, jF, gF, lo, up, gainls.PATH_SPLIT)


def test_plan_rejects_repeated_engines(plan_problem):
    import gainls
    p, pairs = plan_problem
    e = _engines(p, 1)[0]
    with pytest.raises(gainls.GainError, match="repeated"):
        gainls.run_plan([e, e], pairs[:2], gainls.PATH_SPLIT)
