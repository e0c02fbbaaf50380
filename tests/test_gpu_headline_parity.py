"""Parity at the headline workload's full size: N_v = 2000, J''=10 Gamma 0 (11000 functions)
-> J'=11 Gamma 1 (12000 functions), the 2000 lowest lower states x all 12000 upper states.

The split tensor-core path and the plain FP64 path run over the whole block pair on the GPU;
eight sampled lower states are checked against the double-double oracle (the accurate value
of the reference's formula, GPU/dipole_GPU.cu:392-515 then the dot of
BaseClasses/GpuManager.cpp:741) over every upper state.  Bars:
  split path:  max relative error of S = amp^2 <= 1e-8 over lines with S > 1e-10 S_max,
               no uncertified line in that domain;
  plain path:  max relative error of S <= 1e-10 over the same lines (the FP64 bar),
               amplitudes within 1e-12 of the largest.
At full size, on every transition: the split path's S agrees with the plain path's within
the same 1e-8 bar, and the per-lower-state sums of S over all upper states agree too.
"""
import os
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


@pytest.fixture(scope="module")
def headline(built_lib):
    import torch
    import bench
    import gainls
    torch.cuda.set_device(0)
    inp = bench.make_inputs(False, 0, "cuda")
    eng = bench.setup_engine(inp, 0)
    B, NU = inp["vl"].shape[0], inp["vu"].shape[0]
    assert (B, NU) == (2000, 12000)
    lo, up = list(range(B)), list(range(NU))
    st = eng.run_pair(0, bench.GI, 1, bench.GF, lo, up, gainls.PATH_SPLIT)
    split = eng.fetch_amp().copy()
    eng.run_pair(0, bench.GI, 1, bench.GF, lo, up, gainls.PATH_PLAIN_FP64)
    plain = eng.fetch_amp().copy()
    sample = list(range(0, B, B // 8))[:8]
    dd = bench.oracle_sample(inp, sample)
    yield dict(inp=inp, st=st, split=split, plain=plain, sample=sample, dd=dd)
    eng.close()


def test_split_path_against_the_oracle(headline):
    h = headline
    mx, p99, n = __import__("bench").s_rel_err(h["split"][h["sample"]] ** 2, h["dd"] ** 2)
    assert n > 0.9 * h["dd"].size
    assert mx <= 1e-8, (mx, p99)
    assert h["st"]["status"] == 0 and h["st"]["uncertified"] == 0


def test_plain_path_against_the_oracle(headline):
    h = headline
    mx, _, _ = __import__("bench").s_rel_err(h["plain"][h["sample"]] ** 2, h["dd"] ** 2)
    assert mx <= 1e-10
    err = np.max(np.abs(h["plain"][h["sample"]] - h["dd"]))
    assert err <= 1e-12 * np.abs(h["dd"]).max()


def test_split_against_plain_on_every_transition(headline):
    h = headline
    mx, _, n = __import__("bench").s_rel_err(h["split"] ** 2, h["plain"] ** 2)
    assert n > 0.9 * h["plain"].size
    assert mx <= 1e-8


def test_row_sums_of_line_strengths(headline):
    """sum_u amp[l,u]^2 (= |h_l|^2 for the orthonormal upper block) of the two paths."""
    h = headline
    rs = np.sum(h["split"] ** 2, axis=1)
    rp = np.sum(h["plain"] ** 2, axis=1)
    assert np.max(np.abs(rs - rp) / rp) <= 1e-8
