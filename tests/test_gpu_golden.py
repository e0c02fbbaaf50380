"""The product on the GPU against the reference's own kernels (tests/golden fixtures):
the drop-in K-block kernel bit for bit, both engine paths within tolerance."""
import glob
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu
FIXTURES = sorted(f for f in glob.glob(os.path.join(GOLDEN, "*.npz")) if not os.path.basename(f).startswith("rotsym_"))
ROT_FIXTURES = sorted(glob.glob(os.path.join(GOLDEN, "rotsym_*.npz")))


def _problem(d):
    import synth
    nv, jvals, rule = int(d["nv"]), [int(x) for x in d["jvals"]], str(d["rule"])
    bases = [synth.make_basis(J, nv) for J in jvals]
    infl = [synth.inflation_of(b, rule, synth.nsym_of(rule)) for b in bases]
    return nv, jvals, rule, bases, infl


@pytest.mark.parametrize("path", FIXTURES, ids=lambda p: os.path.basename(p)[:-4])
def test_dropin_hls_bit_exact_vs_reference_kernel(built_lib, path):
    import torch
    import gainls
    import oracle
    d = np.load(path)
    nv, jvals, rule, bases, infl = _problem(d)
    jI, jF = jvals.index(int(d["JI"])), jvals.index(int(d["JF"]))
    bI, bF = bases[jI], bases[jF]
    gI = int(d["gI"])
    dI = int(d["idegI"]) if "idegI" in d.files else 0
    s, e = (int(x) for x in d["block"])
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
    keep = [dev(x) for x in (bI.tau, bF.tau, bI.vib, bF.vib, bI.kblock,
                             np.ascontiguousarray(d["dipole"][:, :, s:e]).reshape(-1), d["threej"])]
    for l in range(d["vec_lower"].shape[0]):
        prim = dev(oracle.expand(infl[jI], gI, d["vec_lower"][l], ideg=dI))
        out = torch.zeros(bF.dimen, dtype=torch.float64, device="cuda")
        for kF in range(bF.J + 1):
            gainls.hls_kblock(int(bF.kblock[kF]), bI.dimen, bI.J, bF.J, kF, *[k.data_ptr() for k in keep[:4]],
                              int(bF.kstart[kF]), int(bI.kstart[max(kF - 1, 0)]), s, e, e - s,
                              int(bF.kblock[kF]), keep[4].data_ptr(), keep[5].data_ptr(), prim.data_ptr(),
                              keep[6].data_ptr(), out.data_ptr(), int(d["jmax"]), nv)
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        assert np.array_equal(got.view(np.uint64), d["ref_hls"][l].view(np.uint64))


def _engine_for(d):
    import gainls
    nv, jvals, rule, bases, infl = _problem(d)
    jI, jF = jvals.index(int(d["JI"])), jvals.index(int(d["JF"]))
    gI, gF = int(d["gI"]), int(d["gF"])
    eng = gainls.Engine(int(d["jmax"]), len(infl[0].N), int(max(int(x) for x in infl[0].sdeg)))
    for jind, b in enumerate(bases):
        eng.upload_basis(jind, b.J, b.K, b.tau, b.vib, b.kblock, b.kstart)
        inf = infl[jind]
        eng.upload_inflation(jind, inf.icontr, inf.ijterms, b.dimen, inf.maxcoeff, inf.matsize, inf.N, inf.repres,
                             inf.Ntot, inf.sdeg)
    s, e = (int(x) for x in d["block"])
    eng.upload_dipole(np.ascontiguousarray(d["dipole"][:, :, s:e]).reshape(-1), nv, s, e, e - s)
    eng.upload_eigvecs(jI, gI, d["vec_lower"])
    eng.upload_eigvecs(jF, gF, d["vec_upper"])
    return eng, (jI, gI, jF, gF)


@pytest.mark.parametrize("path", FIXTURES, ids=lambda p: os.path.basename(p)[:-4])
def test_engine_paths_vs_reference_amplitudes(built_lib, path):
    import gainls
    d = np.load(path)
    eng, (jI, gI, jF, gF) = _engine_for(d)
    ref = d["ref_amp"]
    comps = (int(d["idegI"]), int(d["idegF"])) if "idegI" in d.files else None
    lo, up = list(range(ref.shape[0])), list(range(ref.shape[1]))
    eng.run_pair(jI, gI, jF, gF, lo, up, gainls.PATH_PLAIN_FP64, components=comps)
    plain = eng.fetch_amp().copy()
    assert np.max(np.abs(plain - ref)) <= 1e-13 * np.abs(ref).max()
    st = eng.run_pair(jI, gI, jF, gF, lo, up, gainls.PATH_SPLIT, components=comps)
    split = eng.fetch_amp()
    assert st["uncertified"] == 0
    S, Sr = split ** 2, ref ** 2
    m = Sr > 1e-10 * Sr.max()
    assert np.max(np.abs(S[m] - Sr[m]) / Sr[m]) <= 1e-8
    assert np.max(np.abs(split - ref)) <= 1e-11 * np.abs(ref).max()
    eng.close()


@pytest.mark.parametrize("path", ROT_FIXTURES, ids=lambda p: os.path.basename(p)[:-4])
def test_dropin_rotsym_bit_exact_vs_reference_kernel(built_lib, path):
    """gain_hls_rotsym equals the reference's rotsym kernel bit for bit, and leaves the
    entries outside the dipole block untouched."""
    import torch
    import gainls
    import synth
    d = np.load(path)
    nv, JI, JF, md = int(d["nv"]), int(d["JI"]), int(d["JF"]), int(d["maxdeg"])
    bI, bF = synth.make_rotsym_basis(JI, nv, md), synth.make_rotsym_basis(JF, nv, md)
    s, e = (int(x) for x in d["block"])
    piece = np.ascontiguousarray(d["dipole"][:, :, s:e]).reshape(-1)

    def dev(a, dt):
        return torch.from_numpy(np.ascontiguousarray(a, dt)).cuda()

    keep = [dev(bI.K, np.int32), dev(bF.K, np.int32), dev(bI.tau, np.int32), dev(bF.tau, np.int32),
            dev(bI.vib, np.int32), dev(bF.vib, np.int32), dev(piece, np.float64), dev(d["wigner"], np.float64)]
    for v, ref in zip(d["vectors"], d["ref_hls"]):
        dv = dev(v, np.float64)
        out = torch.full((bF.dimen,), 7.0, dtype=torch.float64, device="cuda")
        gainls.hls_rotsym(bF.dimen, bI.dimen, int(d["nlevelI"]), int(d["nlevelF"]), md, *[t.data_ptr() for t in keep[:6]],
                          s, e, e - s, keep[6].data_ptr(), keep[7].data_ptr(), dv.data_ptr(), out.data_ptr(), nv)
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        inside = (bF.vib >= s) & (bF.vib < e)
        assert np.array_equal(got[inside], ref[inside])
        assert np.all(got[~inside] == 7.0)
