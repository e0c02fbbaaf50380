"""Writers of TROVE checkpoint files in the formats the reference reads (test
infrastructure): a synth.Problem becomes j0eigen_quanta<J>.chk, j0eigen_descr<J>_<G>.chk,
j0eigen_vectors<J>_<G>.chk and j0_extfield.chk.

Mapping of the synthetic basis onto TROVE's contracted basis: every primitive function is
one case with one degenerate component; its vibrational class holds the J=0 contracted
index (so the J=0 correlation of TroveBasisSet::Correlate returns it), and its rotational
level is the index of (K, tau) in the order (0, J mod 2), (1, 0), (1, 1), (2, 0), ...
(TroveStates.cpp:34-50); rot_index(level, 1) = (J, K, tau)."""
import struct

import numpy as np


def rot_level(J, K, tau):
    return 0 if K == 0 else 2 * K - 1 + tau


def write_quanta(path, basis, infl, nsym):
    J, d = basis.J, basis.dimen
    lines = ["Start Primitive basis set", f"{d} 1 {d} 1"]
    for i in range(d):
        lines.append(f"1 {rot_level(J, int(basis.K[i]), int(basis.tau[i])) + 1} {int(basis.vib[i]) + 1}")
        lines.append(f"{i + 1} 1 1")
    lines.append(f"{2 * J + 1} 1")
    levels = [(0, J % 2)] + [(k, t) for k in range(1, J + 1) for t in (0, 1)]
    for lev, (k, t) in enumerate(levels):
        lines.append(f"{lev + 1} 1 {J} {k} {t}")
    lines += ["End Primitive basis set", "Start irreducible transformation", "1",
              " ".join(str(int(x)) for x in infl.Ntot)]
    for g in range(nsym):
        lines += [str(int(x)) for x in infl.N[g]]
        lines += [repr(float(x)) for x in infl.repres[g]]
    lines.append("End irreducible transformation")
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def write_states(path, J, gamma, energies, rec_len, k_ind=None):
    lines = ["header line of the descr file", "Start Quantum numbers and energies", "column titles", "units",
             f"{len(energies)} {rec_len}"]
    for lev, e in enumerate(energies):
        k = 0 if k_ind is None else int(k_ind[lev])
        lines.append(f"{lev + 1} {gamma + 1} {lev + 1} 1 {float(e)!r} {k} 0 0 0")
    lines.append("End Quantum numbers and energies")
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def fortran_record(payload: bytes) -> bytes:
    n = struct.pack("<i", len(payload))
    return n + payload + n


def write_dipole(path, dipole):
    """dipole[k][i][f] (the flipped piece layout) -> j0_extfield.chk, component k stored as
    the Fortran array (i, f) the reader flips back (TroveDipole.cpp:107-110)."""
    n = dipole.shape[-1]
    out = fortran_record(b"Start external field") + fortran_record(struct.pack("<i", n))
    for k in range(3):
        out += fortran_record(struct.pack("<i", k + 1))
        out += fortran_record(np.ascontiguousarray(dipole[k].T).astype("<f8").tobytes())
    out += fortran_record(b"End external field  ")
    with open(path, "wb") as f:
        f.write(out)


def write_problem(dirpath, p):
    """Every checkpoint file of a synth.Problem (blocks: energies, vectors)."""
    import os
    for jind, J in enumerate(p.jvals):
        write_quanta(os.path.join(dirpath, f"j0eigen_quanta{J}.chk"), p.bases[jind], p.infl[jind], p.nsym)
    if 0 not in p.jvals:
        import synth
        b0 = synth.make_basis(0, p.nv)
        write_quanta(os.path.join(dirpath, "j0eigen_quanta0.chk"), b0,
                     synth.make_inflation(b0, synth.classes_of(b0, p.rule), p.nsym), p.nsym)
    for (jind, g), blk in p.blocks.items():
        J = p.jvals[jind]
        write_states(os.path.join(dirpath, f"j0eigen_descr{J}_{g + 1}.chk"), J, g, blk.energies, blk.vecs.shape[1])
        blk.vecs.astype("<f8").tofile(os.path.join(dirpath, f"j0eigen_vectors{J}_{g + 1}.chk"))
    write_dipole(os.path.join(dirpath, "j0_extfield.chk"), p.dipole)
