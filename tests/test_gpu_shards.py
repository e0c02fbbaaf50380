"""Lower-state sharding through the engine (MultiGpuManager's split of the lower states over
devices and ranks, BaseClasses/MultiGpuManager.cpp:101-150,233-291, main.cpp:292-293): runs of
one block pair over disjoint lower-state ranges give line-list shards whose concatenation in
range order is the whole run's list, byte for byte, on both paths.  On one GPU the ranks run
one after another on separate engines, as independent ranks would (no data exchange)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

JMAX = 11


@pytest.mark.parametrize("path_name", ["split", "plain"])
def test_shards_concatenate_to_the_whole_list(built_lib, path_name):
    import gainls
    import synth
    path = {"split": gainls.PATH_SPLIT, "plain": gainls.PATH_PLAIN_FP64}[path_name]
    p = synth.make_problem(60, [4, 5], "c4", blocks=[(4, 0), (5, 1)])
    bI, bF = p.blocks[(0, 0)], p.blocks[(1, 1)]
    nI, nF = bI.vecs.shape[0], bF.vecs.shape[0]
    up = list(range(nF))
    whole_eng = gainls.Engine(JMAX, p.nsym, 1)
    gainls.upload_problem(whole_eng, p)
    whole_eng.run_pair(0, 0, 1, 1, list(range(nI)), up, path)
    whole, n_whole = whole_eng.lines_text(bI.energies, bF.energies, 4, 5, 0, 1, intensity=False)
    amp_whole = whole_eng.fetch_amp().copy()
    whole_eng.close()
    world = 3
    bounds = [nI * r // world for r in range(world + 1)]
    parts, n_parts = [], 0
    for r in range(world):
        eng = gainls.Engine(JMAX, p.nsym, 1)
        gainls.upload_problem(eng, p)
        lo = list(range(bounds[r], bounds[r + 1]))
        eng.run_pair(0, 0, 1, 1, lo, up, path)
        # a rank's levels are printed from its own level list: the global lower index
        text, n = eng.lines_text(bI.energies[lo], bF.energies, 4, 5, 0, 1, intensity=False)
        parts.append(bytes(text))
        n_parts += n
        if path == gainls.PATH_PLAIN_FP64:
            # the plain path's amplitudes do not depend on the batch
            np.testing.assert_array_equal(eng.fetch_amp(), amp_whole[lo])
        eng.close()
    assert n_parts == n_whole
    if path == gainls.PATH_PLAIN_FP64:
        assert b"".join(parts) == bytes(whole)
    else:
        # the split path's digit scaling is per row, so a row's amplitudes do not depend on
        # the other rows of its batch either
        assert b"".join(parts) == bytes(whole)
