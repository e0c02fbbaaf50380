"""Generate the golden fixtures of the line-strength path by running the reference's own
kernels on a GPU.

The reference (GAIN-MPI) ships no tests, sample inputs or expected outputs.  These fixtures
are outputs of its unmodified GPU/dipole_GPU.cu (compiled for sm_103a into
oracle/_ref/dipole_GPU.cubin by oracle/build_ref.sh), driven by oracle/ref_harness.cu the
way BaseClasses/GpuManager.cpp drives it: per lower state the expansion kernel and one
K-block launch per K', then per upper state the expansion kernel and cublasDdot.

Each fixture stores the exact inputs that are not pure integer tables (eigenvectors,
dipole piece, 3j table) next to the reference outputs (half_ls per lower state and the
amplitudes), so the CPU tests can replay them anywhere.

    python tests/golden/make_golden.py OUTDIR [rotsym|mixed|degenerate]   # needs a GPU and the reference cubin
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, os.path.join(ROOT, "gain-mpi_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import synth  # noqa: E402
import threej  # noqa: E402
import ref_harness  # noqa: E402

# name: nv, J values, symmetry rule, (J'', Gamma''), (J', Gamma'), lower levels, upper levels, dipole block
CASES = {
    "cfg1_small": (200, [0, 1], "full", (0, 0), (1, 0), list(range(8)), list(range(64)), None),
    "c4_dJp1": (16, [2, 3], "c4", (2, 0), (3, 1), None, None, None),
    "c4_dJm1": (16, [2, 3], "c4", (3, 1), (2, 0), None, None, None),
    "c4_dJ0": (16, [2, 3], "c4", (3, 2), (3, 3), None, None, None),
    "c4_highJ": (6, [10, 11], "c4", (10, 0), (11, 1), list(range(12)), list(range(20)), None),
    "full_blocked": (16, [2, 3], "full", (2, 0), (3, 0), list(range(6)), list(range(30)), (5, 11)),
    # expansions that mix primitives (synth rule c4m)
    "c4m_dJp1": (16, [2, 3], "c4m", (2, 0), (3, 1), None, None, None),
    "c4m_dJ0_blocked": (16, [2, 3], "c4m", (3, 2), (3, 3), None, None, (3, 12)),
}
MIXED = ("c4m_dJp1", "c4m_dJ0_blocked")
# degenerate symmetries (synth rule c3e: A1, A2, E): every component pair (idegI, idegF) of an
# E -> E pair, and an A1 -> A2 pair of the same tables; name -> case, components
DEGENERATE = {
    "c3e_EE_c00": ((12, [2, 3], "c3e", (2, 2), (3, 2), None, None, None), (0, 0)),
    "c3e_EE_c10": ((12, [2, 3], "c3e", (2, 2), (3, 2), None, None, None), (1, 0)),
    "c3e_EE_c01": ((12, [2, 3], "c3e", (2, 2), (3, 2), None, None, None), (0, 1)),
    "c3e_EE_c11_blocked": ((12, [2, 3], "c3e", (2, 2), (3, 2), None, None, (2, 9)), (1, 1)),
    "c3e_A1A2": ((12, [2, 3], "c3e", (3, 0), (2, 1), None, None, None), (0, 0)),
}


def make_case(name, jmax=11):
    comps = (0, 0)
    if name in DEGENERATE:
        case, comps = DEGENERATE[name]
    else:
        case = CASES[name]
    nv, jvals, rule, (JI, gI), (JF, gF), lo, up, blk = case
    p = synth.make_problem(nv, jvals, rule, blocks=[(JI, gI), (JF, gF)])
    jI, jF = jvals.index(JI), jvals.index(JF)
    nI = p.blocks[(jI, gI)].vecs.shape[0]
    nF = p.blocks[(jF, gF)].vecs.shape[0]
    lo = list(range(nI)) if lo is None else lo
    up = list(range(nF)) if up is None else up
    tj = threej.threej_table(jmax)
    vl = p.blocks[(jI, gI)].vecs[lo]
    vu = p.blocks[(jF, gF)].vecs[up]
    amp, hls, _ = ref_harness.run_pair(p, jI, gI, jF, gF, lo, up, tj, jmax, dipole_block=blk,
                                       vec_lower=vl, vec_upper=vu, components=comps)
    return dict(nv=nv, jvals=np.array(jvals), rule=rule, JI=JI, gI=gI, JF=JF, gF=gF,
                idegI=comps[0], idegF=comps[1],
                lower=np.array(lo), upper=np.array(up), block=np.array(blk if blk else (0, nv)),
                jmax=jmax, threej=tj, dipole=p.dipole, vec_lower=vl, vec_upper=vu,
                ref_hls=hls, ref_amp=amp)


# rotational-symmetry (Euler) half line strength: nv, J'', J', degeneracy, lower vectors, dipole block
ROTSYM_CASES = {
    "rotsym_dJp1": (12, 2, 3, 2, 6, None),
    "rotsym_dJ0": (12, 3, 3, 1, 6, None),
    "rotsym_dJm1_blocked": (12, 3, 2, 2, 4, (3, 9)),
}


def make_rotsym_case(name):
    """The reference's rotsym kernel (device_compute_1st_half_ls_flipped_dipole_shared_rotsym_
    nontrove) on seeded primitive lower vectors of the synthetic rotsym basis."""
    nv, JI, JF, maxdeg, nvec, blk = ROTSYM_CASES[name]
    bI, bF = synth.make_rotsym_basis(JI, nv, maxdeg), synth.make_rotsym_basis(JF, nv, maxdeg)
    nI, nF = synth.rotsym_levels(JI), synth.rotsym_levels(JF)
    wig = synth.make_wigner(JI, JF, maxdeg)
    dip = synth.make_dipole(nv)
    rng = np.random.default_rng(4242 + 10 * JI + JF)
    vecs = rng.standard_normal((nvec, bI.dimen)) / np.sqrt(bI.dimen)
    block = blk if blk else (0, nv)
    hls = np.stack([ref_harness.hls_rotsym(bI, bF, nI, nF, maxdeg, dip, block, wig, v) for v in vecs])
    return dict(nv=nv, JI=JI, JF=JF, maxdeg=maxdeg, block=np.array(block), nlevelI=nI, nlevelF=nF,
                wigner=wig, dipole=dip, vectors=vecs, ref_hls=hls)


def main(outdir):
    os.makedirs(outdir, exist_ok=True)
    for name in CASES:
        d = make_case(name)
        np.savez_compressed(os.path.join(outdir, name + ".npz"), **d)
        print(name, d["ref_hls"].shape, d["ref_amp"].shape, float(np.abs(d["ref_amp"]).max()))
    for name in ROTSYM_CASES:
        d = make_rotsym_case(name)
        np.savez_compressed(os.path.join(outdir, name + ".npz"), **d)
        print(name, d["ref_hls"].shape, float(np.abs(d["ref_hls"]).max()))


if __name__ == "__main__":
    out = sys.argv[1] if len(sys.argv) > 1 else os.path.dirname(os.path.abspath(__file__))
    if len(sys.argv) > 2 and sys.argv[2] == "mixed":    # only the mixing-expansion fixtures
        os.makedirs(out, exist_ok=True)
        for name in MIXED:
            d = make_case(name)
            np.savez_compressed(os.path.join(out, name + ".npz"), **d)
            print(name, d["ref_hls"].shape, d["ref_amp"].shape, float(np.abs(d["ref_amp"]).max()))
    elif len(sys.argv) > 2 and sys.argv[2] == "degenerate":   # only the degenerate fixtures
        os.makedirs(out, exist_ok=True)
        for name in DEGENERATE:
            d = make_case(name)
            np.savez_compressed(os.path.join(out, name + ".npz"), **d)
            print(name, d["ref_hls"].shape, d["ref_amp"].shape, float(np.abs(d["ref_amp"]).max()))
    elif len(sys.argv) > 2 and sys.argv[2] == "rotsym":   # only the rotsym fixtures
        os.makedirs(out, exist_ok=True)
        for name in ROTSYM_CASES:
            d = make_rotsym_case(name)
            np.savez_compressed(os.path.join(out, name + ".npz"), **d)
            print(name, d["ref_hls"].shape, float(np.abs(d["ref_hls"]).max()))
    else:
        main(out)
