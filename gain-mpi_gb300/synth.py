"""Seeded synthetic stand-in for the TROVE checkpoint inputs of the line-strength path.

No TROVE checkpoint files (j0_extfield.chk, j0eigen_*.chk) exist for this work, so every
input the reference reads from them is generated here with fixed seeds:

* primitive rotational-vibrational basis per J, in the K-sorted order the reference's
  K-block kernel assumes (TroveClasses/TroveBasisSet.cpp:659-681): K ascending; K = 0 holds
  one tau (= J mod 2), K >= 1 hold tau = 0 then tau = 1; inside each (K, tau) the
  vibrational index v = 0 .. N_v-1.  K-block sizes are therefore N_v (K = 0) and 2 N_v.
* symmetry classes: either one class holding the whole basis ("full"), or four classes
  Gamma = 2 (v mod 2) + ((K + tau) mod 2) ("c4").  The pairing Gamma <-> Gamma xor 1 is
  what the reference derives from SELECTION 1 1 2 2 (TroveClasses/TroveInput.cpp:202-236).
  The symmetry-adapted basis of a class is the set of its primitive functions in primitive
  order, so the expansion tables (ijterms, icontr, N, repres) describe a selection with
  coefficient 1.0 (the reference's general expansion, GPU/dipole_GPU.cu:859-889, still runs
  on them unchanged).
* vibrational dipole: three N_v x N_v components, entries N(0,1) 0.5 exp(-|i-j|/20),
  symmetrised, seed 1234, stored in the reference's flipped layout
  piece[f + i N + d N N] (TroveClasses/TroveDipole.cpp:107-110).
* eigenvectors of each (J, Gamma) block: Q of a QR factorisation of a seeded N(0,1) square
  matrix (seed 1000 + 100 J + Gamma); state k has coefficient vector Q[:, k].
* energies of each (J, Gamma) block: sorted U[0, 8000] cm^-1 (seed 5000 + 100 J + Gamma);
  state k of the block has the k-th energy.
"""
from __future__ import annotations

import dataclasses
import numpy as np

DIPOLE_SEED = 1234


def vec_seed(J: int, gamma: int) -> int:
    return 1000 + 100 * J + gamma


def energy_seed(J: int, gamma: int) -> int:
    return 5000 + 100 * J + gamma


@dataclasses.dataclass
class Basis:
    """Primitive basis of one J: per-function K, tau, vibrational index and K-blocks."""
    J: int
    nv: int
    K: np.ndarray        # int32 [dimen]
    tau: np.ndarray      # int32 [dimen], 0/1
    vib: np.ndarray      # int32 [dimen], J=0 contracted (vibrational) index
    kstart: np.ndarray   # int32 [J+1]
    kblock: np.ndarray   # int32 [J+1]

    @property
    def dimen(self) -> int:
        return int(self.K.shape[0])


def make_basis(J: int, nv: int) -> Basis:
    K, tau, vib = [], [], []
    kstart = np.zeros(J + 1, np.int32)
    kblock = np.zeros(J + 1, np.int32)
    pos = 0
    for k in range(J + 1):
        taus = [J % 2] if k == 0 else [0, 1]
        kstart[k] = pos
        for t in taus:
            K.append(np.full(nv, k, np.int32))
            tau.append(np.full(nv, t, np.int32))
            vib.append(np.arange(nv, dtype=np.int32))
            pos += nv
        kblock[k] = pos - kstart[k]
    return Basis(J, nv, np.concatenate(K), np.concatenate(tau), np.concatenate(vib),
                 kstart, kblock)


def make_rotsym_basis(J: int, nv: int, maxdeg: int = 1) -> Basis:
    """Primitive basis of the rotational-symmetry (Euler) form: each function is a symmetrised
    rotational level (2J+1 levels, each with maxdeg degenerate components) times a vibrational
    function.  The fields follow the reference's rotsym use of the basis arrays
    (TroveClasses/TroveBasisSet.cpp:480-483): K holds the degeneracy index, tau the level
    index.  Order: vibrational index slowest, so the functions are not K-sorted."""
    nlev = 2 * J + 1
    v, lev, deg = np.meshgrid(np.arange(nv), np.arange(nlev), np.arange(maxdeg), indexing="ij")
    K = deg.reshape(-1).astype(np.int32)
    tau = lev.reshape(-1).astype(np.int32)
    vib = v.reshape(-1).astype(np.int32)
    kblock = np.zeros(J + 1, np.int32)
    kstart = np.zeros(J + 1, np.int32)
    if maxdeg == 1:   # every K (degeneracy index) is 0: one K-block holding all functions
        kblock[0] = K.shape[0]
        kstart[1:] = K.shape[0]
    return Basis(J, nv, K, tau, vib, kstart, kblock)


def rotsym_levels(J: int) -> int:
    return 2 * J + 1


def make_wigner(JI: int, JF: int, maxdeg: int = 1) -> np.ndarray:
    """Rotational matrix elements of the three dipole components between the symmetrised
    levels of J'' and J' (synthetic, seeded): rot[d + 3 (lI + nI (lF + nF (dI + maxdeg dF)))],
    the layout of GpuManager::TransferWigner (BaseClasses/GpuManager.cpp:457) and of the
    rotsym kernel's index (GPU/dipole_GPU.cu:692)."""
    nI, nF = rotsym_levels(JI), rotsym_levels(JF)
    rng = np.random.default_rng(7000 + 100 * JI + JF)
    return (0.5 * rng.uniform(-1.0, 1.0, 3 * nI * nF * maxdeg * maxdeg)).astype(np.float64)


def classes_of(basis: Basis, rule: str) -> np.ndarray:
    if rule == "full":
        return np.zeros(basis.dimen, np.int32)
    if rule == "c4":
        return (2 * (basis.vib % 2) + ((basis.K + basis.tau) % 2)).astype(np.int32)
    if rule == "c4r":   # rotsym basis: level index in place of K + tau
        return (2 * (basis.vib % 2) + (basis.tau % 2)).astype(np.int32)
    if rule in ("c4m", "c3e"):   # classes belong to mixed functions, not primitives
        return np.full(basis.dimen, -1, np.int32)
    raise ValueError(f"unknown symmetry rule {rule!r}")


def nsym_of(rule: str) -> int:
    return {"full": 1, "c4": 4, "c4r": 4, "c4m": 4, "c3e": 3}[rule]


def degen_of(rule: str) -> np.ndarray:
    """Degeneracy of each symmetry: rule "c3e" has a doubly degenerate E (A1, A2, E)."""
    if rule == "c3e":
        return np.array([1, 1, 2], np.int32)
    return np.ones(nsym_of(rule), np.int32)


def selection_of(rule: str) -> np.ndarray:
    """isym_pairs: classes with equal entries pair up (SELECTION keyword)."""
    return {"full": np.array([1], np.int32), "c4": np.array([1, 1, 2, 2], np.int32),
            "c4r": np.array([1, 1, 2, 2], np.int32), "c4m": np.array([1, 1, 2, 2], np.int32),
            "c3e": np.array([1, 1, 2], np.int32)}[rule]


def igamma_pair_of(isym_pairs: np.ndarray) -> np.ndarray:
    """Gamma -> paired Gamma, the rule of TroveInput::ComputeIGammaPair (TroveInput.cpp:202-236)."""
    n = len(isym_pairs)
    pair = np.arange(n, dtype=np.int32)
    for gi in range(n):
        found = 0
        for gf in range(n):
            if gi != gf and isym_pairs[gi] == isym_pairs[gf]:
                pair[gi] = gf
                found += 1
                if found > 1:
                    raise ValueError("selection rules do not come in pairs")
    return pair


@dataclasses.dataclass
class Inflation:
    """Symmetry-adapted -> primitive expansion tables of one J (GpuManager::TransferInflation)."""
    maxcoeff: int
    icontr: np.ndarray          # int32 [2*dimen]: irow, then ib
    ijterms: np.ndarray         # int32 [maxcoeff*nsym]
    N: list                     # per Gamma int32 [maxcoeff]
    repres: list                # per Gamma float64 [Ntot*sdeg*matsize]
    Ntot: np.ndarray            # int32 [nsym]
    sdeg: np.ndarray            # int32 [nsym]
    members: list               # per Gamma: primitive indices of the class, ascending (selections)
    matsize: int = 1            # components per case (the repres matrices' last dimension)


def make_inflation(basis: Basis, cls: np.ndarray, nsym: int) -> Inflation:
    d = basis.dimen
    icontr = np.concatenate([np.arange(d, dtype=np.int32), np.zeros(d, np.int32)])
    ijterms = np.zeros(d * nsym, np.int32)
    Ns, repres, members = [], [], []
    Ntot = np.zeros(nsym, np.int32)
    for g in range(nsym):
        n_g = (cls == g).astype(np.int32)
        ijterms[g * d:(g + 1) * d] = np.concatenate([[0], np.cumsum(n_g)[:-1]]).astype(np.int32)
        Ns.append(n_g)
        Ntot[g] = int(n_g.sum())
        repres.append(np.ones(int(Ntot[g]), np.float64))
        members.append(np.nonzero(cls == g)[0].astype(np.int32))
    return Inflation(d, icontr, ijterms, Ns, repres, Ntot, np.ones(nsym, np.int32), members)


def inflation_of(basis: Basis, rule: str, nsym: int) -> "Inflation":
    """The expansion tables of a basis under a symmetry rule."""
    if rule == "c4m":
        return make_mixed_inflation(basis, nsym)
    if rule == "c3e":
        return make_degenerate_inflation(basis)
    return make_inflation(basis, classes_of(basis, rule), nsym)


MIX_COEF = 0.7071067811865476   # the double nearest 1/sqrt(2)


def make_mixed_inflation(basis: Basis, nsym: int = 4) -> Inflation:
    """Expansion tables of rule "c4m", a symmetrisation that mixes primitives the way TROVE's
    symmetry-adapted functions do (a case holds several primitive components and each
    symmetric function of the case is a linear combination of them):

    * case (K = 0, v): one component, the primitive (0, J mod 2, v); one function of class
      2 (v mod 2) + (J mod 2);
    * case (K >= 1, v): components ib = 0, 1 = the primitives (K, 0, v), (K, 1, v); functions
      (p0 + p1) / sqrt(2) of class 2 (v mod 2) + (K mod 2) and (p0 - p1) / sqrt(2) of class
      2 (v mod 2) + ((K + 1) mod 2).

    repres has mat_size = 2 (the component index); cases are numbered in primitive order."""
    d = basis.dimen
    J = basis.J
    icontr = np.zeros(2 * d, np.int32)
    case_of, cases = {}, []          # (K, v) -> case index; per case: list of (ib, primitive)
    for r in range(d):
        key = (int(basis.K[r]), int(basis.vib[r]))
        if key not in case_of:
            case_of[key] = len(cases)
            cases.append([])
        ib = 0 if basis.K[r] == 0 else int(basis.tau[r])
        cases[case_of[key]].append((ib, r))
        icontr[r] = case_of[key]
        icontr[r + d] = ib
    ncase = len(cases)
    funcs = [[] for _ in range(nsym)]   # per class: (case, coefficients of components 0, 1)
    for c, comps in enumerate(cases):
        K = int(basis.K[comps[0][1]])
        v = int(basis.vib[comps[0][1]])
        if K == 0:
            funcs[2 * (v % 2) + (J % 2)].append((c, (1.0, 0.0)))
        else:
            funcs[2 * (v % 2) + (K % 2)].append((c, (MIX_COEF, MIX_COEF)))
            funcs[2 * (v % 2) + ((K + 1) % 2)].append((c, (MIX_COEF, -MIX_COEF)))
    ijterms = np.zeros(ncase * nsym, np.int32)
    Ns, repres = [], []
    Ntot = np.zeros(nsym, np.int32)
    for g in range(nsym):
        n_g = np.zeros(ncase, np.int32)
        for c, _ in funcs[g]:
            n_g[c] += 1
        ijterms[g * ncase:(g + 1) * ncase] = np.concatenate([[0], np.cumsum(n_g)[:-1]]).astype(np.int32)
        Ns.append(n_g)
        Ntot[g] = len(funcs[g])
        rep = np.zeros(2 * int(Ntot[g]), np.float64)   # [s + ib Ntot], sdeg = 1, mat_size = 2
        for s_idx, (c, co) in enumerate(funcs[g]):     # funcs[g] is in case order
            rep[s_idx] = co[0]
            rep[s_idx + int(Ntot[g])] = co[1]
        repres.append(rep)
    return Inflation(ncase, icontr, ijterms, Ns, repres, Ntot, np.ones(nsym, np.int32), [None] * nsym, matsize=2)


E_PAIRS = ((0.6, 0.8), (MIX_COEF, MIX_COEF))   # (a, b) of the E components, exact in binary64 terms


def make_degenerate_inflation(basis: Basis) -> Inflation:
    """Expansion tables of rule "c3e": symmetries A1, A2 and a doubly degenerate E, built the
    way a C3v symmetric top's are (K = 3n mixes into A1/A2, other K form E pairs):

    * case (K = 0, v): one component, the primitive; one function of A1 for even v + J, else A2;
    * case (K >= 1, v), components ib = 0, 1 = the primitives (K, 0, v), (K, 1, v):
      - K mod 3 == 0: (p0 + p1) / sqrt(2) and (p0 - p1) / sqrt(2) in A1 and A2 (the other way
        round for odd v);
      - otherwise one E function whose component 0 is a p0 + b p1 and component 1 is
        b p0 - a p1, (a, b) = E_PAIRS[(K + v) mod 2].

    repres[s + ideg Ntot + ib sdeg Ntot] (transform_vector_primitive's index,
    GPU/dipole_GPU.cu:882), sdeg = (1, 1, 2), mat_size = 2; cases in primitive order."""
    d = basis.dimen
    J = basis.J
    icontr = np.zeros(2 * d, np.int32)
    case_of, cases = {}, []
    for r in range(d):
        key = (int(basis.K[r]), int(basis.vib[r]))
        if key not in case_of:
            case_of[key] = len(cases)
            cases.append([])
        ib = 0 if basis.K[r] == 0 else int(basis.tau[r])
        cases[case_of[key]].append((ib, r))
        icontr[r] = case_of[key]
        icontr[r + d] = ib
    ncase = len(cases)
    nsym = 3
    sdeg = np.array([1, 1, 2], np.int32)
    funcs = [[] for _ in range(nsym)]   # per class: (case, [per component: coefficients of ib 0, 1])
    for c, comps in enumerate(cases):
        K = int(basis.K[comps[0][1]])
        v = int(basis.vib[comps[0][1]])
        if K == 0:
            funcs[(v + J) % 2].append((c, [(1.0, 0.0)]))
        elif K % 3 == 0:
            funcs[v % 2].append((c, [(MIX_COEF, MIX_COEF)]))
            funcs[1 - v % 2].append((c, [(MIX_COEF, -MIX_COEF)]))
        else:
            a, b = E_PAIRS[(K + v) % 2]
            funcs[2].append((c, [(a, b), (b, -a)]))
    ijterms = np.zeros(ncase * nsym, np.int32)
    Ns, repres = [], []
    Ntot = np.zeros(nsym, np.int32)
    for g in range(nsym):
        n_g = np.zeros(ncase, np.int32)
        for c, _ in funcs[g]:
            n_g[c] += 1
        ijterms[g * ncase:(g + 1) * ncase] = np.concatenate([[0], np.cumsum(n_g)[:-1]]).astype(np.int32)
        Ns.append(n_g)
        Ntot[g] = len(funcs[g])
        nt, sd = int(Ntot[g]), int(sdeg[g])
        rep = np.zeros(nt * sd * 2, np.float64)
        for s_idx, (c, co) in enumerate(funcs[g]):
            for ideg in range(sd):
                for ib in range(2):
                    rep[s_idx + ideg * nt + ib * sd * nt] = co[ideg][ib]
        repres.append(rep)
    return Inflation(ncase, icontr, ijterms, Ns, repres, Ntot, sdeg, [None] * nsym, matsize=2)


def make_dipole(nv: int, seed: int = DIPOLE_SEED) -> np.ndarray:
    """[3, N, N] array whose flat order is the flipped piece layout f + i N + d N N."""
    rng = np.random.default_rng(seed)
    idx = np.arange(nv)
    # exp(-k/20) as successive powers of the double nearest e^{-1/20}: IEEE products give the
    # same bits on every machine, unlike libm's exp
    pw = np.empty(max(nv, 1))
    pw[0] = 1.0
    for k in range(1, nv):
        pw[k] = pw[k - 1] * 0.951229424500714
    decay = 0.5 * pw[np.abs(idx[:, None] - idx[None, :])]
    out = np.empty((3, nv, nv), np.float64)
    for d in range(3):
        a = rng.standard_normal((nv, nv)) * decay
        out[d] = 0.5 * (a + a.T)
    return out


def make_energies(n: int, J: int, gamma: int) -> np.ndarray:
    rng = np.random.default_rng(energy_seed(J, gamma))
    return np.sort(rng.uniform(0.0, 8000.0, n))


def make_eigvecs(n: int, J: int, gamma: int, device: str | None = None,
                 nstates: int | None = None) -> np.ndarray:
    """Rows are state coefficient vectors (Q[:, k] of QR of a seeded Gaussian matrix).

    nstates < n keeps the first nstates states only; the first k columns of Q depend only
    on the first k columns of the Gaussian matrix, so they equal the full factorisation's.
    device=None uses numpy's QR; device="cuda" runs the same factorisation through torch on
    the GPU (used only to make large inputs quickly, never on a timed path).
    """
    rng = np.random.default_rng(vec_seed(J, gamma))
    g = rng.standard_normal((n, n))
    if nstates is not None and nstates < n:
        g = np.ascontiguousarray(g[:, :nstates])
    if device is None:
        q, r = np.linalg.qr(g)
        s = np.sign(np.diag(r))
        s[s == 0] = 1.0
        q = q * s[None, :]
        return np.ascontiguousarray(q.T)
    import torch
    t = torch.from_numpy(g).to(device)
    q, r = torch.linalg.qr(t)
    s = torch.sign(torch.diagonal(r))
    s[s == 0] = 1.0
    q = q * s[None, :]
    return np.ascontiguousarray(q.T.cpu().numpy())


def make_eigvecs_kron(n: int, J: int, gamma: int, device: str = "cuda"):
    """A dense orthonormal n x n matrix made quickly on the device (for block sizes whose QR
    factorisation would take minutes).  With n1 = floor(sqrt(n)), n2 = n // n1, m = n1 n2 and
    r = n - m: Y = (Q3 (x) Q4) P (Q1 (x) Q2) on the first m coordinates (a row permutation P
    between two Kronecker products of Q factors of seeded N(0,1) matrices, the second product
    applied as two small contractions, so every entry sums n1 n2 products and the rows are
    dense rather than spiky), Q5 (r x r) on the rest, then seeded permutations of rows and
    columns.  Kronecker products and permutations of orthogonal matrices are orthogonal, so the
    result is orthonormal to rounding.  Returns a torch tensor [n, n] (rows = states)."""
    import torch
    rng = np.random.default_rng(vec_seed(J, gamma))
    n1 = max(1, int(np.floor(np.sqrt(n))))
    n2 = n // n1
    m = n1 * n2
    r = n - m

    def q(k):
        g = torch.from_numpy(rng.standard_normal((k, k))).to(device)
        qq, rr = torch.linalg.qr(g)
        sgn = torch.sign(torch.diagonal(rr))
        sgn[sgn == 0] = 1.0
        return qq * sgn[None, :]

    Q1, Q2, Q3, Q4 = q(n1), q(n2), q(n1), q(n2)
    Y = torch.kron(Q1, Q2)
    Y = Y[torch.from_numpy(rng.permutation(m)).to(device)]
    # (Q3 (x) Q4) Y: rows indexed (a, b), a < n1, b < n2
    Y = Y.view(n1, n2, m)
    Y = torch.einsum("bc,acj->abj", Q4, Y)
    Y = torch.einsum("ac,cbj->abj", Q3, Y).reshape(m, m)
    U = torch.zeros((n, n), dtype=torch.float64, device=device)
    U[:m, :m] = Y
    del Y
    if r > 0:
        U[m:, m:] = q(r)
    pr = torch.from_numpy(rng.permutation(n)).to(device)
    pc = torch.from_numpy(rng.permutation(n)).to(device)
    return U[pr][:, pc].contiguous()


@dataclasses.dataclass
class Block:
    J: int
    jind: int
    gamma: int
    vecs: np.ndarray      # [nlevels, Ntot]
    energies: np.ndarray  # [nlevels]


@dataclasses.dataclass
class Problem:
    nv: int
    jvals: list
    rule: str
    nsym: int
    sym_degen: np.ndarray
    isym_pairs: np.ndarray
    igamma_pair: np.ndarray
    bases: list
    infl: list
    classes: list
    dipole: np.ndarray
    blocks: dict          # (jind, gamma) -> Block
    # state table in global energy order (TroveStates::ReadStates sorts by energy)
    st_J: np.ndarray = None
    st_jind: np.ndarray = None
    st_gamma: np.ndarray = None
    st_ndeg: np.ndarray = None
    st_ilevel: np.ndarray = None
    st_energy: np.ndarray = None

    def block_states(self, jind: int, gamma: int) -> np.ndarray:
        """Global state indices of a block, in the block's level order."""
        sel = np.nonzero((self.st_jind == jind) & (self.st_gamma == gamma))[0]
        return sel[np.argsort(self.st_ilevel[sel], kind="stable")]


def make_problem(nv: int, jvals, rule: str = "c4", blocks=None, qr_device=None,
                 max_levels=None) -> Problem:
    """Build bases, expansion tables, dipole and the (J, Gamma) blocks.

    blocks: iterable of (J, Gamma) to materialise (default: every class of every J).
    max_levels: optional cap on how many (lowest) levels of a block are kept.
    """
    nsym = nsym_of(rule)
    isym_pairs = selection_of(rule)
    bases, infl, classes = [], [], []
    for J in jvals:
        b = make_rotsym_basis(J, nv) if rule == "c4r" else make_basis(J, nv)
        c = classes_of(b, rule)
        bases.append(b)
        classes.append(c)
        infl.append(inflation_of(b, rule, nsym))
    if blocks is None:
        blocks = [(J, g) for J in jvals for g in range(nsym)]
    blk = {}
    for (J, g) in blocks:
        jind = list(jvals).index(J)
        n = int(infl[jind].Ntot[g])
        if n == 0:
            continue
        vecs = make_eigvecs(n, J, g, qr_device)
        en = make_energies(n, J, g)
        if max_levels is not None and max_levels < n:
            vecs, en = vecs[:max_levels], en[:max_levels]
        blk[(jind, g)] = Block(J, jind, g, np.ascontiguousarray(vecs), en)
    p = Problem(nv, list(jvals), rule, nsym, degen_of(rule), isym_pairs,
                igamma_pair_of(isym_pairs), bases, infl, classes, make_dipole(nv), blk)
    J_, jind_, g_, lev_, e_ = [], [], [], [], []
    for (jind, g), b in sorted(blk.items()):
        n = b.energies.shape[0]
        J_ += [b.J] * n
        jind_ += [jind] * n
        g_ += [g] * n
        lev_ += list(range(n))
        e_.append(b.energies)
    e = np.concatenate(e_) if e_ else np.zeros(0)
    order = np.argsort(e, kind="stable")
    p.st_J = np.asarray(J_, np.int32)[order]
    p.st_jind = np.asarray(jind_, np.int32)[order]
    p.st_gamma = np.asarray(g_, np.int32)[order]
    p.st_ndeg = p.sym_degen[p.st_gamma].astype(np.int32)
    p.st_ilevel = np.asarray(lev_, np.int32)[order]
    p.st_energy = e[order]
    return p


# Named workloads (sizes of the reference's headline configurations).
CONFIGS = {
    # J''=0 -> J'=1, whole basis, 50 lowest J=0 states against every J=1 state.
    "cfg1": dict(nv=200, jvals=[0, 1], rule="full", lower=(0, 0), upper=(1, 0), n_lower=50,
                 e_lower=(0.0, 8000.0), e_upper=(0.0, 8000.0)),
    # J''=10 class 0 (11000 functions) -> J'=11 class 1 (12000 functions); the 2000 lowest
    # lower states (all below 5000 cm^-1) against every upper state below 10000 cm^-1.
    "cfg2": dict(nv=2000, jvals=[10, 11], rule="c4", lower=(10, 0), upper=(11, 1), n_lower=2000,
                 e_lower=(0.0, 5000.0), e_upper=(0.0, 10000.0)),
}
