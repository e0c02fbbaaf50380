"""GPU parity of the kernel-level drop-ins (gain_hls_kblock, gain_expand, gain_dot)
against the CPU oracle, called through the C ABI with device pointers."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

JMAX = 11


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.mark.parametrize("case", [("full", 16, 2, 3), ("full", 12, 3, 2), ("full", 10, 4, 4),
                                  ("c4", 16, 10, 11)])
def test_hls_kblock_bit_exact_vs_oracle(built_lib, case):
    """Every K block of the drop-in equals the oracle's restatement of
    device_compute_1st_half_ls_flipped_dipole_shared_block_nontrove bit for bit."""
    import torch
    import gainls
    import oracle
    import synth
    import threej
    rule, nv, JI, JF = case
    bI, bF = synth.make_basis(JI, nv), synth.make_basis(JF, nv)
    rng = np.random.default_rng(JI * 100 + JF)
    vec = rng.standard_normal(bI.dimen)
    vec[rng.random(bI.dimen) < 0.3] = 0.0           # zero entries are skipped like the reference
    dip = synth.make_dipole(nv)
    tj = threej.threej_table(JMAX)
    for (s, e) in [(0, nv), (3, nv - 2)]:
        piece = np.ascontiguousarray(dip[:, :, s:e]).reshape(-1)
        ref = np.full(bF.dimen, -7.0)
        d_tI, d_tF, d_vI, d_vF = map(_dev, (bI.tau, bF.tau, bI.vib, bF.vib))
        d_kb, d_dip, d_vec, d_tj = _dev(bI.kblock), _dev(piece), _dev(vec), _dev(tj)
        d_out = torch.full((bF.dimen,), -7.0, dtype=torch.float64, device="cuda")
        for kF in range(JF + 1):
            args = (int(bF.kblock[kF]), bI.dimen, JI, JF, kF)
            startF, startI = int(bF.kstart[kF]), int(bI.kstart[max(kF - 1, 0)])
            oracle.hls_kblock(*args, bI.tau, bF.tau, bI.vib, bF.vib, startF, startI, s, e, e - s,
                              bI.kblock, piece, nv, vec, tj, JMAX, ref, oracle.REF)
            gainls.hls_kblock(*args, d_tI.data_ptr(), d_tF.data_ptr(), d_vI.data_ptr(), d_vF.data_ptr(),
                              startF, startI, s, e, e - s, int(bF.kblock[kF]), d_kb.data_ptr(),
                              d_dip.data_ptr(), d_vec.data_ptr(), d_tj.data_ptr(), d_out.data_ptr(), JMAX, nv)
        torch.cuda.synchronize()
        out = d_out.cpu().numpy()
        assert np.array_equal(out.view(np.uint64), ref.view(np.uint64))


def test_expand_matches_oracle(built_lib):
    import torch
    import gainls
    import oracle
    import synth
    b = synth.make_basis(3, 10)
    cls = synth.classes_of(b, "c4")
    inf = synth.make_inflation(b, cls, 4)
    for g in range(4):
        v = np.random.default_rng(g).standard_normal(int(inf.Ntot[g]))
        ref = oracle.expand(inf, g, v)
        d = {k: _dev(x) for k, x in dict(ij=inf.ijterms, ic=inf.icontr, N=inf.N[g], rp=inf.repres[g], v=v).items()}
        out = torch.zeros(b.dimen, dtype=torch.float64, device="cuda")
        gainls.expand(b.dimen, g, inf.maxcoeff, 0, 1, int(inf.Ntot[g]), d["ij"].data_ptr(), d["ic"].data_ptr(),
                      d["N"].data_ptr(), d["rp"].data_ptr(), d["v"].data_ptr(), out.data_ptr())
        torch.cuda.synchronize()
        assert np.array_equal(out.cpu().numpy(), ref)


def test_dot_matches_oracle(built_lib):
    import torch
    import gainls
    import oracle
    rng = np.random.default_rng(9)
    for n in (1, 31, 1000, 12345):
        x, y = rng.standard_normal(n), rng.standard_normal(n)
        res = torch.zeros(1, dtype=torch.float64, device="cuda")
        dx, dy = _dev(x), _dev(y)          # keep both alive while the kernel reads them
        gainls.dot(n, dx.data_ptr(), dy.data_ptr(), res.data_ptr())
        torch.cuda.synchronize()
        ref = oracle.dot(x, y, oracle.DD)
        assert abs(res.item() - ref) <= 4 * n * 1.2e-16 * np.sum(np.abs(x * y))


def test_invalid_arguments_rejected_before_launch(built_lib):
    import gainls
    with pytest.raises(gainls.GainError) as e:
        gainls.hls_kblock(10, 10, 1, 3, 0, 1, 1, 1, 1, 0, 0, 0, 5, 5, 10, 1, 1, 1, 1, 1, JMAX, 5)
    assert e.value.status == gainls.ERR_INVALID_ARG
