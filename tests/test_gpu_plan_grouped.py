"""gain_plan_*: many block pairs as one unit -- per-job digit slicing, ONE grouped tensor-core
launch of the first GEMM over every job's tiles, per-job refinement and slicing of H, ONE
grouped launch of the second GEMM, per-job refinement -- captured in a CUDA graph.

The digit arithmetic is exact and the recombination order-independent, so with the same digit
configuration every job's amplitudes equal the single-pair run's bit for bit, whatever the
tile shape, the schedule or which job's digits of a shared lower or upper block it reads.  Replays reuse the graph; new eigenvectors of the same sizes are
picked up without a new capture; the autotuner's choice keeps S within 1e-8 of the plain FP64
path; lines and text read through gain_plan_select equal the single-pair run's."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

JMAX = 11


def _jobs(p, frac=0.5):
    import gainls
    filt = gainls.make_filters([1.0] * p.nsym, p.isym_pairs, p.igamma_pair, p.sym_degen, (0.0, 4000.0),
                               (-1e9, 1e9), (-1e9, 1e9), 0.0, 4)
    table = gainls.state_table(p.st_energy, p.st_J, p.st_jind, p.st_gamma, p.st_ndeg, p.st_ilevel)
    return gainls.plan_pairs(filt, table)


def _problem(rule, nv=24, jvals=(1, 2, 3, 4)):
    import gainls
    import synth
    p = synth.make_problem(nv, list(jvals), rule)
    eng = gainls.Engine(JMAX, p.nsym, 1)
    gainls.upload_problem(eng, p)
    return p, eng


@pytest.mark.parametrize("rule", ["c4", "c4m", "c4r"])
def test_plan_equals_single_pair_runs(built_lib, rule):
    import gainls
    p, eng = _problem(rule)
    jobs = _jobs(p)
    assert len(jobs) >= 8
    want = []
    for jI, gI, jF, gF, lo, up in jobs:
        eng.run_pair(jI, gI, jF, gF, lo, up, gainls.PATH_SPLIT)
        want.append(eng.fetch_amp().copy())
    plan = gainls.Plan(eng, jobs)
    ps, js, st = plan.run()
    assert st == gainls.OK and ps["failed_jobs"] == 0
    assert ps["jobs"] == len(jobs) and ps["captures"] == 1
    # jobs of one upper block read its first job's upper digits, and (without mixing
    # expansions) jobs of one lower block its first job's lower digits
    assert ps["shared_upper"] > 0
    if rule != "c4m":
        assert ps["shared_lower"] > 0
    assert ps["transitions"] == sum(len(j[4]) * len(j[5]) for j in jobs)
    for q in range(len(jobs)):
        np.testing.assert_array_equal(plan.amp(q), want[q])
    # a replay reuses the graph and gives the same amplitudes
    ps2, _, _ = plan.run()
    assert ps2["captures"] == 1
    for q in range(len(jobs)):
        np.testing.assert_array_equal(plan.amp(q), want[q])
    plan.close()


def test_plan_single_cta_tiles_equal_pairs(built_lib, monkeypatch):
    """128 x 128 tiles (GAINLS_GEMM_PAIR=0) and 256 x 128 CTA-pair tiles give the same bits."""
    import gainls
    p, eng = _problem("c4", nv=120, jvals=(4, 5, 6))
    jobs = _jobs(p)
    assert max(len(j[4]) for j in jobs) > 128   # some job has CTA-pair tiles
    a = gainls.Plan(eng, jobs)
    sa, _, _ = a.run()
    amps = [a.amp(q) for q in range(len(jobs))]
    a.close()
    monkeypatch.setenv("GAINLS_GEMM_PAIR", "0")
    b = gainls.Plan(eng, jobs)
    sb, _, _ = b.run()
    assert (sa["pair"], sb["pair"]) == (1, 0)
    for q in range(len(jobs)):
        np.testing.assert_array_equal(b.amp(q), amps[q])
    b.close()


def test_new_eigenvectors_without_a_new_capture(built_lib):
    import gainls
    p, eng = _problem("c4")
    jobs = _jobs(p)
    plan = gainls.Plan(eng, jobs)
    plan.run()
    # scaled eigenvectors of the same sizes: same device buffers, the graph stays valid
    for (jind, g), blk in p.blocks.items():
        eng.upload_eigvecs(jind, g, 0.5 * blk.vecs)
    ps, _, _ = plan.run()
    assert ps["captures"] == 1
    for q, (jI, gI, jF, gF, lo, up) in enumerate(jobs):
        eng.run_pair(jI, gI, jF, gF, lo, up, gainls.PATH_SPLIT)
        np.testing.assert_array_equal(plan.amp(q), eng.fetch_amp())
    # a new dipole: the next run prepares and captures again
    nv = p.dipole.shape[-1]
    eng.upload_dipole((2.0 * p.dipole).reshape(-1), nv, 0, nv, nv)
    ps, _, _ = plan.run()
    assert ps["captures"] == 2
    jI, gI, jF, gF, lo, up = jobs[0]
    eng.run_pair(jI, gI, jF, gF, lo, up, gainls.PATH_SPLIT)
    np.testing.assert_array_equal(plan.amp(0), eng.fetch_amp())
    plan.close()


def test_autotuned_plan_accuracy_and_lines(built_lib):
    import gainls
    p, eng = _problem("c4", nv=60, jvals=(3, 4, 5))
    jobs = _jobs(p)
    plan = gainls.Plan(eng, jobs, autotune=True)
    ps, js, st = plan.run()
    assert st == gainls.OK and ps["tuned"] == 1 and ps["tune_ms"] > 0
    for q, (jI, gI, jF, gF, lo, up) in enumerate(jobs):
        got = plan.amp(q)
        eng.run_pair(jI, gI, jF, gF, lo, up, gainls.PATH_PLAIN_FP64)
        ref = eng.fetch_amp()
        S, Sr = got ** 2, ref ** 2
        m = Sr > 1e-10 * Sr.max()
        assert np.max(np.abs(S[m] - Sr[m]) / Sr[m]) <= 1e-8, q
    # a second plan of the same shape takes the cached choice without tuning again
    plan2 = gainls.Plan(eng, jobs, autotune=True)
    ps2, _, _ = plan2.run()
    assert ps2["tuned"] == 1 and ps2["tune_ms"] == 0.0
    assert (ps2["pair"], ps2["beta2"], ps2["slices2"]) == (ps["pair"], ps["beta2"], ps["slices2"])
    # the line text of a job through gain_plan_select equals the single-pair run's
    jI, gI, jF, gF, lo, up = jobs[-1]
    eI = p.blocks[(jI, gI)].energies[lo]
    eF = p.blocks[(jF, gF)].energies[up]
    JI, JF = p.jvals[jI], p.jvals[jF]
    plan2.select(len(jobs) - 1)
    text_plan, n_plan = eng.lines_text(eI, eF, JI, JF, gI, gF)
    if ps2["beta2"] == [0, 0, 0, 0] or all(b in (0, 8) for b in ps2["beta2"]):
        eng.run_pair(jI, gI, jF, gF, lo, up, gainls.PATH_SPLIT)
        text_pair, n_pair = eng.lines_text(eI, eF, JI, JF, gI, gF)
        assert (n_plan, bytes(text_plan)) == (n_pair, bytes(text_pair))
    plan.close()
    plan2.close()
