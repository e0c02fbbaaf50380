"""Handle-level thread safety (the reference gives each OpenMP thread its own stream, cuBLAS
handle and buffers, main.cpp:292-334): engines on distinct handles run block pairs from
concurrent host threads (ctypes releases the GIL during each call) and give the amplitudes
and line text they give one at a time."""
import threading

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

JMAX = 11


def test_concurrent_engines_match_sequential(built_lib):
    import gainls
    import synth
    p = synth.make_problem(40, [3, 4], "c4", blocks=[(3, 0), (4, 1), (4, 0), (3, 1)])
    jobs = [(0, 0, 1, 1), (1, 1, 0, 0), (1, 0, 1, 1), (0, 1, 1, 0)]
    engines = []
    for _ in jobs:
        eng = gainls.Engine(JMAX, p.nsym, 1)
        gainls.upload_problem(eng, p)
        engines.append(eng)

    def levels(j):
        jI, gI, jF, gF = j
        return list(range(p.blocks[(jI, gI)].vecs.shape[0])), list(range(p.blocks[(jF, gF)].vecs.shape[0]))

    def run(eng, j, out, k):
        lo, up = levels(j)
        for path in (gainls.PATH_SPLIT, gainls.PATH_PLAIN_FP64):
            for _ in range(3):
                eng.run_pair(*j, lo, up, path)
            out[(k, path)] = eng.fetch_amp().copy()
        eI = p.blocks[(j[0], j[1])].energies
        eF = p.blocks[(j[2], j[3])].energies
        out[(k, "text")] = bytes(eng.lines_text(eI, eF, p.jvals[j[0]], p.jvals[j[2]], j[1], j[3])[0])

    seq = {}
    for k, (eng, j) in enumerate(zip(engines, jobs)):
        run(eng, j, seq, k)
    par, errors = {}, []

    def guarded(*a):
        try:
            run(*a)
        except Exception as exc:   # reported after the join
            errors.append(exc)

    threads = [threading.Thread(target=guarded, args=(eng, j, par, k)) for k, (eng, j) in enumerate(zip(engines, jobs))]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors, errors
    for key, v in seq.items():
        if key[1] == "text":
            assert par[key] == v
        else:
            np.testing.assert_array_equal(par[key], v)
