"""The product's state selection (gain_filter_intensity, gain_degeneracy_filter,
gain_transition_details, gain_plan_pairs) against the oracle's restatement of
BaseClasses/States.cpp, on synthetic state tables with varied windows and weights."""
import itertools

import numpy as np
import pytest


def _tables(p, **kw):
    import gainls
    import oracle
    args = dict(gns=[1.0] * p.nsym, isym_pairs=p.isym_pairs, igamma_pair=p.igamma_pair, sym_degen=p.sym_degen,
                erange_lower=(0.0, 3000.0), erange_upper=(0.0, 8000.0), freq_window=(-1e9, 1e9), zpe=0.0)
    args.update(kw)
    of = oracle.Filters(p.jvals, args["gns"], args["isym_pairs"], args["igamma_pair"], args["sym_degen"],
                        args["erange_lower"], args["erange_upper"], args["freq_window"], args["zpe"])
    gf = gainls.make_filters(args["gns"], args["isym_pairs"], args["igamma_pair"], args["sym_degen"],
                             args["erange_lower"], args["erange_upper"], args["freq_window"], args["zpe"],
                             max(p.jvals))
    table = gainls.state_table(p.st_energy, p.st_J, p.st_jind, p.st_gamma, p.st_ndeg, p.st_ilevel)
    return of, gf, table


CASES = [dict(), dict(freq_window=(0.0, 1e9)), dict(freq_window=(500.0, 2500.0)),
         dict(gns=[0.0, 1.0, 3.0, 3.0]), dict(erange_lower=(1000.0, 2000.0), erange_upper=(1500.0, 6000.0)),
         dict(zpe=400.0)]


@pytest.mark.parametrize("kw", CASES)
def test_transitions_match_oracle(built_lib, kw):
    import gainls
    import oracle
    import synth
    p = synth.make_problem(3, [0, 1, 2], "c4", max_levels=5)
    of, gf, table = _tables(p, **kw)
    ref = set(oracle.transitions(p, of))
    n = len(table)
    got = {(i, j) for i in range(n) for j in range(n) if i != j and gainls.filter_intensity(gf, table[i], table[j])}
    assert got == ref
    ninit, ntrans, mx = gainls.transition_details(gf, table)
    assert ntrans == len(ref)
    assert ninit == sum(1 for i in range(n) if of.filter_lower(p.st_energy[i], p.st_gamma[i]))


@pytest.mark.parametrize("kw", CASES)
def test_plan_covers_exactly_the_transitions(built_lib, kw):
    """Every transition lies in exactly one planned block pair (the frequency window is the
    only per-line condition left to the line assembly)."""
    import gainls
    import oracle
    import synth
    p = synth.make_problem(3, [0, 1, 2], "c4", max_levels=5)
    of, gf, table = _tables(p, **kw)
    ref = set(oracle.transitions(p, of))
    index = {(int(p.st_jind[i]), int(p.st_gamma[i]), int(p.st_ilevel[i])): i for i in range(len(table))}
    covered = set()
    for jI, gI, jF, gF, lo, up in gainls.plan_pairs(gf, table):
        for l, u in itertools.product(lo, up):
            I, F = index[(jI, gI, l)], index[(jF, gF, u)]
            nu = p.st_energy[F] - p.st_energy[I]
            if of.freq_window[0] <= nu <= of.freq_window[1] and I != F:
                assert (I, F) not in covered
                covered.add((I, F))
    assert covered == ref


def test_degeneracy_filter_matches_oracle(built_lib):
    import gainls
    import oracle
    degen = [1, 1, 2, 3, 3, 2]
    for red, st in itertools.product([False, True], [1, 2, 3]):
        of = oracle.Filters([0, 1], [1.0] * 6, [1] * 6, [0] * 6, degen, (0, 1), (0, 1), reduced=red,
                            symmetry_type=st)
        gf = gainls.make_filters([1.0] * 6, [1] * 6, [0] * 6, degen, (0, 1), (0, 1), reduced=red,
                                 symmetry_type=st)
        for gI, gF, dI, dF in itertools.product(range(6), range(6), range(3), range(3)):
            assert gainls.degeneracy_filter(gf, gI, gF, dI, dF) == of.degeneracy_filter(gI, gF, dI, dF)


def test_selection_rejects_bad_tables(built_lib):
    import gainls
    gf = gainls.make_filters([1.0], [1], [0], [1], (0, 1), (0, 1))
    bad = gainls.state_table([1.0], [0], [0], [5], [1], [0])
    with pytest.raises(gainls.GainError):
        gainls.transition_details(gf, bad)
