"""Benchmark of the line-strength hot path (one JSON line on rank 0).

Workload (the headline configuration): N_v = 2000, J''=10 symmetry class 0 (11000 basis
functions) -> J'=11 class 1 (12000 functions); the 2000 lowest lower states (all below
5000 cm^-1) against all 12000 upper states (all below 10000 cm^-1): 2.4e7 line strengths
per step.  Synthetic, seeded inputs stand in for the TROVE checkpoints.

One step = the split-precision tensor-core path over the whole block pair starting from
FP64 inputs resident in HBM: digit slicing of both eigenvector sets, the rotational-dipole
band GEMM, the amplitude GEMM, FP64 refinement of uncertified lines.  `e2e` runs the same
step through the C ABI from pinned host buffers: upload of both eigenvector sets, the run,
and the device-to-host read of S and A.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "gain-mpi_gb300"))
# the CPU oracle's OpenMP threads sleep when idle instead of spinning on the host cores that
# drive the GPU (they would otherwise keep spinning for a while after each parallel loop)
os.environ.setdefault("OMP_WAIT_POLICY", "PASSIVE")

METRIC = "transitions/s: split-prec TC vs FP64 plain @ S rel-err≤1e-8; % of roofline"
UNIT = "transitions/s"
NV, JI, JF, GI, GF = 2000, 10, 11, 0, 1
N_LOWER = 2000
WORKLOAD = ("N_v=2000, J''=10 Gamma 0 (11000 functions) -> J'=11 Gamma 1 (12000 functions), "
            "2000 lowest lower states x 12000 upper states")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-plain", action="store_true", help="skip the plain FP64 comparison run")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--small", action="store_true", help="reduced sizes (development only)")
    ap.add_argument("--lower", type=int, default=0,
                    help="number of lower states (profiling captures; default: the workload's 2000)")
    ap.add_argument("--precision-sweep", action="store_true",
                    help="accuracy of each digit configuration of the amplitude GEMM against the "
                         "double-double oracle (one JSON line per configuration)")
    ap.add_argument("--adjoint", action="store_true",
                    help="gradient of a line-strength loss over all block pairs of J=0..5, checked "
                         "against central differences (one JSON line)")
    ap.add_argument("--adj-nv", type=int, default=1000, help="vibrational basis size of --adjoint")
    ap.add_argument("--adj-fd", type=int, default=200, help="entries checked by central differences")
    ap.add_argument("--adj-fd-direct", type=int, default=4,
                    help="of those, entries also checked with two plain FP64 forwards each")
    ap.add_argument("--rule", choices=["c4", "c4m"], default="c4",
                    help="symmetrisation of the workload: c4 (selection, the headline) or c4m (functions "
                         "that combine two primitives, as TROVE's symmetry-adapted functions do)")
    ap.add_argument("--batch", action="store_true",
                    help="every allowed block pair of J=0..--batch-jmax through the split path (one JSON line)")
    ap.add_argument("--batch-nv", type=int, default=200, help="vibrational basis size of --batch")
    ap.add_argument("--batch-engines", type=int, default=4,
                    help="engines (streams, host threads) of the --batch plan run through gain_run_plan")
    ap.add_argument("--degenerate", action="store_true",
                    help="a doubly degenerate E -> E pair at N_v = 2000, J''=10 -> J'=11 (rule c3e), every component pair")
    ap.add_argument("--batch-jmax", type=int, default=30, help="largest J of --batch")
    ap.add_argument("--batch-stream", action="store_true",
                    help="many block pairs at the full size (N_v from --batch-nv, default 2000 here), in waves")
    ap.add_argument("--stream-upper-j", type=int, default=-1,
                    help="--batch-stream: only the waves whose upper J is this one, each also run pair by pair")
    return ap.parse_args()


def dist_info():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


# ------------------------------------------------------------------------- sharding
def lower_first(rank: int, n_lower: int, n_block: int) -> int:
    """First lower level of rank's batch: consecutive, disjoint batches of n_lower levels
    while they fit in the block, wrapping around (replicas) beyond that."""
    nb = max(n_block // n_lower, 1)
    return (rank % nb) * n_lower if n_block >= n_lower else 0


def max_over_ranks(value: float, dist=None, device=None) -> float:
    """The step time the bench reports: the slowest rank's."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ------------------------------------------------------------------------- inputs
def make_inputs(small: bool, rank: int, device: str | None, orthonormal: bool = True, n_lower_override: int = 0,
                rule: str = "c4"):
    """orthonormal=False replaces the QR eigenvectors by normalised Gaussian rows of the same
    shape (used only where the values do not matter: timing the CPU reference formula)."""
    import synth
    nv, n_lower = (200, 64) if small else (NV, N_LOWER)
    if n_lower_override > 0:
        n_lower = n_lower_override
    bI, bF = synth.make_basis(JI, nv), synth.make_basis(JF, nv)
    iI, iF = synth.inflation_of(bI, rule, 4), synth.inflation_of(bF, rule, 4)
    nI, nF = int(iI.Ntot[GI]), int(iF.Ntot[GF])
    # each rank takes its own batch of lower states (weak scaling, no data exchange)
    first = lower_first(rank, n_lower, nI)
    if orthonormal:
        # QR eigenvectors are cached between runs of the same workload (profilers cannot
        # always load torch's linear-algebra library inside their injected process)
        import tempfile
        cdir = os.environ.get("GAIN_BENCH_CACHE", os.path.join(tempfile.gettempdir(), "gain_bench_inputs"))
        cfile = os.path.join(cdir, f"eig_{rule}_nv{nv}_J{JI}g{GI}_{first}_{n_lower}_J{JF}g{GF}.npz")
        if os.path.exists(cfile):
            z = np.load(cfile)
            vl, vu = z["vl"], z["vu"]
        else:
            vl = synth.make_eigvecs(nI, JI, GI, device=device, nstates=first + n_lower)[first:first + n_lower]
            vu = synth.make_eigvecs(nF, JF, GF, device=device)
            try:
                os.makedirs(cdir, exist_ok=True)
                np.savez(cfile + ".tmp.npz", vl=vl, vu=vu)
                os.replace(cfile + ".tmp.npz", cfile)
            except OSError:
                pass
    else:
        rng = np.random.default_rng(synth.vec_seed(JI, GI))
        vl = rng.standard_normal((n_lower, nI)) / np.sqrt(nI)
        vu = np.random.default_rng(synth.vec_seed(JF, GF)).standard_normal((nF, nF)) / np.sqrt(nF)
    eI = synth.make_energies(nI, JI, GI)[first:first + n_lower]
    eF = synth.make_energies(nF, JF, GF)
    return dict(nv=nv, bases=[bI, bF], infl=[iI, iF], dipole=synth.make_dipole(nv), vl=np.ascontiguousarray(vl),
                vu=np.ascontiguousarray(vu), eI=eI, eF=eF, first=first, rule=rule)


_PINNED = []   # pinned host tensors backing the arrays handed out by pinned()


def pinned(a: np.ndarray) -> np.ndarray:
    """A page-locked copy of a (the torch tensor that owns it is kept alive)."""
    import torch
    t = torch.empty(a.shape, dtype=torch.float64, pin_memory=True)
    _PINNED.append(t)
    out = t.numpy()
    out[...] = a
    return out


def setup_engine(inp, device_index: int):
    import gainls
    eng = gainls.Engine(11, 4, 1, device=device_index)
    for jind, (b, inf) in enumerate(zip(inp["bases"], inp["infl"])):
        eng.upload_basis(jind, b.J, b.K, b.tau, b.vib, b.kblock, b.kstart)
        eng.upload_inflation(jind, inf.icontr, inf.ijterms, b.dimen, inf.maxcoeff, inf.matsize, inf.N, inf.repres,
                             inf.Ntot, inf.sdeg)
    nv = inp["nv"]
    eng.upload_dipole(inp["dipole"].reshape(-1), nv, 0, nv, nv)
    eng.upload_eigvecs(0, GI, inp["vl"])
    eng.upload_eigvecs(1, GF, inp["vu"])
    return eng


# ------------------------------------------------------------------------- clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def line_text_bench(eng, inp, steps: int) -> dict:
    """The line list of the last run as text (Output.cpp:99-111 format, intensity column on),
    built on the device and copied into page-locked host memory as it forms
    (gain_pair_lines_text_host); wall time per call."""
    import torch
    text, nl = eng.lines_text(inp["eI"], inp["eF"], JI, JF, GI, GF)
    host = torch.empty(max(1, len(text)), dtype=torch.uint8, pin_memory=True)
    _PINNED.append(host)
    buf = host.numpy()
    ms = []
    for i in range(steps + 1):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        _, nl = eng.lines_text_host(inp["eI"], inp["eF"], JI, JF, GI, GF, buf)
        if i:
            ms.append((time.perf_counter() - t0) * 1e3)
    m = float(np.median(ms))
    return {"lines": int(nl), "bytes": len(text), "ms": m, "lines_per_s": nl / (m * 1e-3),
            "GB_per_s": len(text) / (m * 1e-3) / 1e9,
            "intensity_evaluated_on_host": eng.intensity_host(),
            "includes": "S/A/I, text on the device, copy to pinned host overlapped part by part; the "
                        "intensity of lines whose printed digits depend on exp's last bit from the host"}


def cpu_text_baseline(eng, inp, rows: int) -> dict:
    """The reference's sprintf/fprintf text (Output.cpp:52-112, restated in the oracle) of
    the first rows lower states of the last run's amplitudes, one host thread."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.build()
    amp = eng.fetch_amp()[:rows].copy()
    NU = amp.shape[1]
    t0 = time.perf_counter()
    text, nl = oracle.line_list(amp, inp["eI"][:rows], inp["eF"], list(range(rows)), list(range(NU)), JI, JF,
                                GI, GF)
    secs = time.perf_counter() - t0
    return {"lines_per_s": nl / secs, "cores": 1, "kind": "port",
            "sample": f"{rows} lower states x {NU} upper states ({nl} lines, {len(text)} bytes)"}


# ------------------------------------------------------------------------- CPU baseline
def cpu_baseline(inp, n_sample: int):
    """The reference's FP64 formula restated in C (oracle), OpenMP over upper states as in
    main.cpp:292, on all host cores; a bounded sample of lower states of the workload."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    import threej
    import synth
    oracle.build()
    nv = inp["nv"]
    rule = inp.get("rule", "c4")
    p = synth.Problem(nv, [JI, JF], rule, 4, np.ones(4, np.int32), synth.selection_of(rule),
                      synth.igamma_pair_of(synth.selection_of(rule)), inp["bases"], inp["infl"],
                      [synth.classes_of(b, rule) for b in inp["bases"]], inp["dipole"],
                      {(0, GI): synth.Block(JI, 0, GI, inp["vl"][:n_sample], inp["eI"][:n_sample]),
                       (1, GF): synth.Block(JF, 1, GF, inp["vu"], inp["eF"])})
    cores = os.cpu_count() or 1
    tj = threej.threej_table(11)
    t0 = time.perf_counter()
    oracle.run_pair(p, 0, GI, 1, GF, list(range(n_sample)), list(range(inp["vu"].shape[0])), tj, 11,
                    oracle.REF, cores, fast=True)
    secs = time.perf_counter() - t0
    n = n_sample * inp["vu"].shape[0]
    return {"value": n / secs, "unit": UNIT, "cores": cores, "kind": "port",
            "build": "gcc " + " ".join(oracle.FAST_FLAGS),
            "sample": f"{n_sample} lower states x {inp['vu'].shape[0]} upper states of the workload "
                      f"({n} transitions, {secs:.1f} s)"}


def oracle_sample(inp, sample, nthreads: int = 0) -> np.ndarray:
    """Amplitudes of the sampled lower states (indices into the workload's lower states)
    against every upper state, from the double-double oracle (the accurate FP64 answer of
    the reference's formula); all host cores."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    import synth
    import threej
    oracle.build()
    rule = inp.get("rule", "c4")
    sample = list(sample)
    p = synth.Problem(inp["nv"], [JI, JF], rule, 4, np.ones(4, np.int32), synth.selection_of(rule),
                      synth.igamma_pair_of(synth.selection_of(rule)), inp["bases"], inp["infl"],
                      [synth.classes_of(b, rule) for b in inp["bases"]], inp["dipole"],
                      {(0, GI): synth.Block(JI, 0, GI, inp["vl"][sample], inp["eI"][sample]),
                       (1, GF): synth.Block(JF, 1, GF, inp["vu"], inp["eF"])})
    return oracle.run_pair(p, 0, GI, 1, GF, list(range(len(sample))), list(range(inp["vu"].shape[0])),
                           threej.threej_table(11), 11, oracle.DD, nthreads or (os.cpu_count() or 1))


def s_rel_err(S: np.ndarray, Sref: np.ndarray, floor: float = 1e-10):
    """max and p99 relative error of S against Sref over the lines with Sref > floor Sref_max,
    and the number of such lines."""
    m = Sref > floor * Sref.max()
    r = np.abs(S[m] - Sref[m]) / Sref[m]
    return float(r.max()), float(np.quantile(r, 0.99)), int(m.sum())


def _peak(key: str, default: float = 1900.0) -> float:
    try:
        return float(json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))[key])
    except Exception:
        return default


def precision_sweep(args):
    """Digit configurations of the amplitude GEMM (8-bit digits x 3..7 slices, 7-bit x 5..7) on
    the workload: time, refinement counts, and the relative error of S = amp^2 for lines with
    S > 1e-10 S_max against (a) the double-double oracle on a sample of lower states and (b) the
    plain FP64 path on all transitions.  One JSON line per configuration, then a summary."""
    import torch
    torch.cuda.set_device(0)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import gainls
    import oracle
    import synth
    import threej
    oracle.build()
    inp = make_inputs(args.small, 0, "cuda", n_lower_override=args.lower)
    eng = setup_engine(inp, 0)
    B, NU = inp["vl"].shape[0], inp["vu"].shape[0]
    lo, up = list(range(B)), list(range(NU))
    sample = list(range(0, B, max(1, B // 8)))[:8]
    p = synth.Problem(inp["nv"], [JI, JF], "c4", 4, np.ones(4, np.int32), synth.selection_of("c4"),
                      synth.igamma_pair_of(synth.selection_of("c4")), inp["bases"], inp["infl"],
                      [synth.classes_of(b, "c4") for b in inp["bases"]], inp["dipole"],
                      {(0, GI): synth.Block(JI, 0, GI, inp["vl"][sample], inp["eI"][sample]),
                       (1, GF): synth.Block(JF, 1, GF, inp["vu"], inp["eF"])})
    t0 = time.perf_counter()
    dd = oracle.run_pair(p, 0, GI, 1, GF, list(range(len(sample))), up, threej.threej_table(11), 11, oracle.DD,
                         os.cpu_count() or 1)
    dd_secs = time.perf_counter() - t0
    Sdd = dd ** 2
    mdd = Sdd > 1e-10 * Sdd.max()

    def err(S, Sr, m):
        r = np.abs(S[m] - Sr[m]) / Sr[m]
        return float(r.max()), float(np.quantile(r, 0.99))

    sp = eng.run_pair(0, GI, 1, GF, lo, up, gainls.PATH_PLAIN_FP64)
    plain = eng.fetch_amp().copy()
    Sp = plain ** 2
    mp = Sp > 1e-10 * Sp.max()
    e_plain = err(Sp[sample], Sdd, mdd)
    print(json.dumps({"config": "plain FP64 path", "ms": sp["device_ms"],
                      "max_rel_err_S_vs_dd": e_plain[0], "p99_rel_err_S_vs_dd": e_plain[1]}), flush=True)
    best = None
    for beta, slices in [(8, 3), (8, 4), (8, 5), (8, 6), (8, 7), (7, 5), (7, 6), (7, 7)]:
        eng.run_pair(0, GI, 1, GF, lo, up, gainls.PATH_SPLIT, beta=beta, slices=slices, raise_on_error=False)
        st = eng.run_pair(0, GI, 1, GF, lo, up, gainls.PATH_SPLIT, beta=beta, slices=slices, raise_on_error=False)
        amp = eng.fetch_amp()
        S = amp ** 2
        e_dd = err(S[sample], Sdd, mdd)
        e_fp = err(S, Sp, mp)
        nprod = st["slices2"] * (st["slices2"] + 1) // 2
        row = {"config": f"beta={st['beta2']} x{st['slices2']} ({st['slices2'] * beta} bits), "
                         f"{nprod} digit products x {st['chunks2']} chunks",
               "status": ["OK", "INVALID_ARG", "OOM", "CUDA", "TIMEOUT", "TOL_NOT_MET", "NOT_READY",
                          "UNSUPPORTED"][st["status"]],
               "ms": st["device_ms"], "gemm2_ms": st["gemm2_ms"], "refined": st["refined"],
               "uncertified": st["uncertified"], "max_rel_err_S_vs_dd": e_dd[0], "p99_rel_err_S_vs_dd": e_dd[1],
               "max_rel_err_S_vs_fp64": e_fp[0], "p99_rel_err_S_vs_fp64": e_fp[1]}
        print(json.dumps(row), flush=True)
        if beta == 8 and st["status"] == gainls.OK and e_dd[0] <= 1e-8 and best is None:
            best = slices
    print(json.dumps({"summary": "smallest 8-bit slice count meeting S rel-err <= 1e-8 against the "
                                 "double-double oracle (sampled lower states), with certification",
                      "slices": best, "oracle_sample": f"{len(sample)} lower x {NU} upper states "
                      f"({dd_secs:.1f} s on {os.cpu_count()} cores)",
                      "domain": "S > 1e-10 S_max"}), flush=True)


class _DeviceMatrix:
    """A read view of an engine's device amplitude matrix for torch (no copy)."""

    def __init__(self, ptr: int, rows: int, cols: int, ld: int):
        self.__cuda_array_interface__ = {"shape": (rows, cols), "strides": (8 * ld, 8), "typestr": "<f8",
                                         "data": (ptr, False), "version": 3, "stream": None}


def adjoint_check(args):
    """Gradient of a line-strength loss with respect to the dipole matrix elements.

    All allowed block pairs of J = 0..5 (the reference's intensity filter with open energy and
    frequency windows, J = J_max pairs excluded).  L = sum w (log S - log S_t)^2, S_t the line
    strengths of a dipole perturbed elementwise by mu (1 + 0.01 N(0,1)) (seed 77); w = 1 on the
    lines with S_t > 1e-10 max S_t and S > 1e-10 max S (a fixed mask: a line whose strength is
    near zero has an unbounded log derivative).  dL/dmu comes from gain_adjoint_pair summed
    over the pairs (FP64) and is checked on random entries with a non-zero gradient (seed 78)
    and along random directions against (a) central differences of L (plain FP64 forwards,
    h = 1e-6) and (b) the exact directional derivative: amp is linear in mu, so
    dL/dmu . d = sum dL/dS 2 amp amp(d) with amp(d) the forward pass of the dipole d (one
    plain FP64 forward per entry or direction, no step-size error).  One JSON line."""
    import torch
    torch.cuda.set_device(0)
    import gainls
    import synth
    nv = args.adj_nv
    t0 = time.perf_counter()
    p = synth.make_problem(nv, list(range(6)), "c4", qr_device="cuda")
    eng = gainls.Engine(5, p.nsym, 1)
    gainls.upload_problem(eng, p)
    filt = gainls.make_filters([1.0] * p.nsym, p.isym_pairs, p.igamma_pair, p.sym_degen, (-1e9, 1e9),
                               (-1e9, 1e9), (-1e9, 1e9), 0.0, 5)
    table = gainls.state_table(p.st_energy, p.st_J, p.st_jind, p.st_gamma, p.st_ndeg, p.st_ilevel)
    pairs = gainls.plan_pairs(filt, table)
    setup_s = time.perf_counter() - t0
    mu0 = np.ascontiguousarray(p.dipole)
    n_lines = sum(len(lo) * len(up) for *_, lo, up in pairs)

    def amp_now(lo, up):
        ptr, ld = eng.amp_device()
        return torch.as_tensor(_DeviceMatrix(ptr, len(lo), len(up), ld), device="cuda")

    def forward(mu, path=gainls.PATH_PLAIN_FP64, keep=False):
        eng.upload_dipole(mu.reshape(-1), nv, 0, nv, nv)
        out = []
        for jI, gI, jF, gF, lo, up in pairs:
            eng.run_pair(jI, gI, jF, gF, lo, up, path)
            if keep:
                out.append(amp_now(lo, up).clone())
        torch.cuda.synchronize()
        return out

    # the target and the reference point
    mu_t = mu0 * (1.0 + 0.01 * np.random.default_rng(77).standard_normal(mu0.shape))
    S_t = [a * a for a in forward(mu_t, keep=True)]
    S_0 = [a * a for a in forward(mu0, keep=True)]
    smax_t = max(float(s.max()) for s in S_t)
    smax_0 = max(float(s.max()) for s in S_0)
    masks = [(st > 1e-10 * smax_t) & (s0 > 1e-10 * smax_0) for st, s0 in zip(S_t, S_0)]
    logS_t = [torch.log(torch.where(m, st, torch.ones_like(st))) for st, m in zip(S_t, masks)]
    del S_t

    def loss(mu):
        eng.upload_dipole(mu.reshape(-1), nv, 0, nv, nv)
        total = torch.zeros((), dtype=torch.float64, device="cuda")
        for (jI, gI, jF, gF, lo, up), m, lt in zip(pairs, masks, logS_t):
            eng.run_pair(jI, gI, jF, gF, lo, up, gainls.PATH_PLAIN_FP64)
            a = amp_now(lo, up)
            d = torch.where(m, torch.log(a * a) - lt, torch.zeros_like(lt))
            total += torch.sum(d * d)
            torch.cuda.synchronize()   # the next run overwrites the amplitudes
        return float(total)

    # forward times over all pairs: plain FP64 and split paths
    times = {}
    for name, path in (("plain_fp64", gainls.PATH_PLAIN_FP64), ("split", gainls.PATH_SPLIT)):
        forward(mu0, path)
        t1 = time.perf_counter()
        forward(mu0, path)
        times[f"forward_{name}_s"] = time.perf_counter() - t1
    # dL/dS at mu0, then the adjoint of every pair
    amp0 = forward(mu0, keep=True)
    dLdS_dev = []
    for s0, m, lt in zip(S_0, masks, logS_t):
        dLdS_dev.append(torch.where(m, 2.0 * (torch.log(s0) - lt) / s0, torch.zeros_like(s0)))
    dLdS = [g.cpu().numpy() for g in dLdS_dev]
    del S_0

    def jvp(d):
        """Exact dL/dmu . d from the forward pass of the dipole d (amp is linear in mu)."""
        eng.upload_dipole(np.ascontiguousarray(d).reshape(-1), nv, 0, nv, nv)
        total = torch.zeros((), dtype=torch.float64, device="cuda")
        for (jI, gI, jF, gF, lo, up), g, a0 in zip(pairs, dLdS_dev, amp0):
            eng.run_pair(jI, gI, jF, gF, lo, up, gainls.PATH_PLAIN_FP64)
            total += torch.sum(g * 2.0 * a0 * amp_now(lo, up))
            torch.cuda.synchronize()
        return float(total)
    L0 = loss(mu0)
    grad = np.zeros(mu0.size)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    chain_ms = {"f64": 0.0, "f32": 0.0}
    for (jI, gI, jF, gF, lo, up), g in zip(pairs, dLdS):
        eng.adjoint(jI, gI, jF, gF, lo, up, g, grad)
        chain_ms["f64"] += eng.last_adjoint_stats.device_ms
    times["adjoint_s"] = time.perf_counter() - t1
    grad = grad.reshape(mu0.shape)
    # the same gradient with the adjoint chain in FP32 arithmetic
    grad32 = np.zeros(mu0.size)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    for (jI, gI, jF, gF, lo, up), g in zip(pairs, dLdS):
        eng.adjoint(jI, gI, jF, gF, lo, up, g, grad32, precision="f32")
        chain_ms["f32"] += eng.last_adjoint_stats.device_ms
    times["adjoint_fp32_s"] = time.perf_counter() - t1
    fp32_vs_fp64 = float(np.max(np.abs(grad32 - grad.reshape(-1))) / np.abs(grad).max())
    # algorithmic flops of the chain's two products: dL/dH = G U (2 B N_upper Ntot_F) and
    # dM = dh^T v over the (F, I) with |K_I - K_F| <= 1 (2 B per pair)
    chain_flops = 0.0
    for jI, gI, jF, gF, lo, up in pairs:
        B, Nu, NtF = len(lo), len(up), int(p.infl[jF].Ntot[gF])
        kI = np.bincount(p.bases[jI].K, minlength=7)[:7].astype(np.float64)
        kF = np.bincount(p.bases[jF].K, minlength=7)[:7].astype(np.float64)
        band = sum(kF[a] * kI[b] for a in range(7) for b in range(7) if abs(a - b) <= 1)
        chain_flops += 2.0 * B * Nu * NtF + 2.0 * B * band
    # the same gradient from the split path's amplitudes: per pair the tensor-core forward,
    # dL/dS on the device, then the adjoint (which takes the run's amplitudes)
    grad_split = np.zeros(mu0.size)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    for (jI, gI, jF, gF, lo, up), m, lt in zip(pairs, masks, logS_t):
        eng.run_pair(jI, gI, jF, gF, lo, up, gainls.PATH_SPLIT)
        s0 = amp_now(lo, up) ** 2
        g = torch.where(m, 2.0 * (torch.log(s0) - lt) / s0, torch.zeros_like(s0)).cpu().numpy()
        eng.adjoint(jI, gI, jF, gF, lo, up, g, grad_split)
    times["gradient_split_forward_s"] = time.perf_counter() - t1
    split_vs_fp64 = float(np.max(np.abs(grad_split - grad.reshape(-1))) / np.abs(grad).max())
    # the tensor-core adjoint (GAIN_ADJOINT_SPLIT): both products as digit GEMMs, each pair's
    # own split forward (nothing kept from an earlier forward)
    eng.upload_dipole(mu0.reshape(-1), nv, 0, nv, nv)
    grad_tc = np.zeros(mu0.size)
    tc_flops = 0.0
    chain_ms["split_tensor_core"] = 0.0
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    for (jI, gI, jF, gF, lo, up), g in zip(pairs, dLdS):
        eng.adjoint(jI, gI, jF, gF, lo, up, g, grad_tc, precision="split")
        chain_ms["split_tensor_core"] += eng.last_adjoint_stats.device_ms
        tc_flops += eng.last_adjoint_stats.tensor_flops
    times["adjoint_tensor_core_s"] = time.perf_counter() - t1
    tc_vs_fp64 = float(np.max(np.abs(grad_tc - grad.reshape(-1))) / np.abs(grad).max())

    # central differences (h = 1e-6) of L on args.adj_fd random entries with a non-zero gradient.
    # amp is linear in mu, so the perturbed forwards are amp(mu0 +- h e_k) = amp0 +- h amp(e_k),
    # amp(e_k) the forward of the one-hot dipole e_k (split path, certified); the difference
    # L(mu0 + h e_k) - L(mu0 - h e_k) is summed line by line as (d+ - d-)(d+ + d-), with
    # d+ - d- = 2 [log1p(h r) - log1p(-h r)], r = amp(e_k) / amp0, so that no cancellation
    # between the two losses limits it.  A few entries are also checked with two plain FP64
    # forwards at mu0 +- h e_k and the difference of the two losses.
    h = 1e-6
    rng = np.random.default_rng(78)
    gflat = grad.reshape(-1)
    gflat_tc = grad_tc.reshape(-1)
    gmax = float(np.abs(gflat).max())
    cand = np.flatnonzero(np.abs(gflat) > 0)
    picks = rng.choice(cand, size=min(args.adj_fd, cand.size), replace=False)
    rel, absn, jrel, rel32, reltc = [], [], [], [], []
    lt_all = logS_t

    def fd_linear(k):
        """(central difference of L at h, exact partial derivative) for entry k, both from
        amp(e_k); the exact partial is sum dL/dS 2 amp0 amp(e_k)."""
        e = np.zeros(mu0.size)
        e[k] = 1.0
        ak = forward(e.reshape(mu0.shape), gainls.PATH_SPLIT, keep=True)
        num = torch.zeros((), dtype=torch.float64, device="cuda")
        exact = torch.zeros((), dtype=torch.float64, device="cuda")
        for a0, a1, m, lt, g in zip(amp0, ak, masks, lt_all, dLdS_dev):
            r = torch.where(m, a1 / a0, torch.zeros_like(a0))
            dm = torch.where(m, 2.0 * torch.log(torch.abs(a0)) - lt, torch.zeros_like(a0))
            diff = 2.0 * (torch.log1p(h * r) - torch.log1p(-h * r))   # d+ - d-
            num += torch.sum(diff * (2.0 * dm + 2.0 * (torch.log1p(h * r) + torch.log1p(-h * r))))   # d+ + d-
            exact += torch.sum(g * 2.0 * a0 * a1)
        return float(num) / (2 * h), float(exact)

    t1 = time.perf_counter()
    for k in picks:
        fd, ex = fd_linear(k)
        rel.append(abs(fd - gflat[k]) / abs(gflat[k]))
        absn.append(abs(fd - gflat[k]) / gmax)
        rel32.append(abs(fd - grad32[k]) / abs(gflat[k]))
        reltc.append(abs(fd - gflat_tc[k]) / abs(gflat[k]))
        jrel.append(abs(ex - gflat[k]) / abs(gflat[k]))
    times["fd_s"] = time.perf_counter() - t1
    direct = []
    t1 = time.perf_counter()
    for k in picks[:args.adj_fd_direct]:
        mp, mm = mu0.copy(), mu0.copy()
        mp.reshape(-1)[k] += h
        mm.reshape(-1)[k] -= h
        fd = (loss(mp) - loss(mm)) / (2 * h)
        direct.append(abs(fd - gflat[k]) / abs(gflat[k]))
    times["fd_direct_s"] = time.perf_counter() - t1
    dirs, jdirs = [], []
    for _ in range(3):
        # a unit direction: h d then moves each entry by about h / sqrt(entries), the regime in
        # which the central difference of this (weak-line dominated) loss is accurate
        d = rng.standard_normal(mu0.shape)
        d /= np.linalg.norm(d)
        gd = float(np.sum(grad * d))
        fd = (loss(mu0 + h * d) - loss(mu0 - h * d)) / (2 * h)
        dirs.append(abs(fd - gd) / abs(gd))
        jdirs.append(abs(jvp(d) - gd) / abs(gd))
    rel, jrel = np.asarray(rel), np.asarray(jrel)
    out = {"mode": "adjoint", "workload": f"N_v={nv}, J=0..5, all allowed block pairs",
           "pairs": len(pairs), "lines": n_lines, "lines_in_loss": int(sum(int(m.sum()) for m in masks)),
           "loss": L0, "gradient_dtype": "f64 (and f32: fp32_*)", "fd_step": h, "fd_entries": int(len(picks)),
           "fd_max_rel_err": float(rel.max()), "fd_median_rel_err": float(np.median(rel)),
           "fd_p99_rel_err": float(np.quantile(rel, 0.99)),
           "fd_max_err_over_max_grad": float(max(absn)), "fd_direction_rel_err": [float(x) for x in dirs],
           "exact_partials_max_rel_err": float(jrel.max()), "exact_partials_median_rel_err": float(np.median(jrel)),
           "exact_direction_rel_err": [float(x) for x in jdirs],
           "fd_method": "central differences of L at h, perturbed forwards formed as amp0 +- h amp(e_k) "
                        "(amp linear in mu), loss difference summed line by line",
           "fd_direct_entries": len(direct), "fd_direct_max_rel_err": float(max(direct)) if direct else None,
           "fd_direct_median_rel_err": float(np.median(direct)) if direct else None,
           "tensor_core_adjoint": {"max_err_over_max_grad_vs_fp64": tc_vs_fp64,
                                   "fd_max_rel_err": float(max(reltc)), "fd_median_rel_err": float(np.median(reltc)),
                                   "fd_p99_rel_err": float(np.quantile(reltc, 0.99)),
                                   "chain_device_ms": chain_ms["split_tensor_core"],
                                   "tensor_flops": tc_flops,
                                   "tensor_tflops": tc_flops / (chain_ms["split_tensor_core"] * 1e-3) / 1e12,
                                   "peak_bf16_tflops": _peak("bf16_tflops"),
                                   "digits": "48 bits (8-bit digits x 6, exact FP32 accumulation)"},
           "split_forward_gradient_max_err_over_max_grad": split_vs_fp64,
           "fp32_gradient_max_err_over_max_grad": fp32_vs_fp64,
           "fp32_fd_median_rel_err": float(np.median(rel32)), "fp32_fd_p99_rel_err": float(np.quantile(rel32, 0.99)),
           "adjoint_chain_device_ms": chain_ms, "adjoint_chain_flops": chain_flops,
           "adjoint_chain_tflops": {k: chain_flops / (v * 1e-3) / 1e12 for k, v in chain_ms.items()},
           "nonzero_gradient_entries": int(cand.size), "gradient_entries": int(mu0.size),
           "setup_s": setup_s}
    out.update(times)
    print(json.dumps(out), flush=True)
    eng.close()


def degenerate_pair(args):
    """Degenerate symmetries at the sizes of the N_v = 2000 pair: rule c3e (A1, A2, doubly
    degenerate E), N_v = 2000, J'' = 10 E (the 2000 lowest states) -> J' = 11 E (every state).  A step is
    gain_run_pair_degenerate over the four component pairs (generic symmetry type: all pass)
    through the split path; the lines combine the four slots (S = sum amp^2 / 2).  S is checked
    against the plain FP64 path's four components on the same lines.  One JSON line."""
    import torch
    torch.cuda.set_device(0)
    import gainls
    import synth
    nv = 200 if args.small else NV
    n_lower = 64 if args.small else N_LOWER
    E = 2
    t0 = time.perf_counter()
    bI, bF = synth.make_basis(JI, nv), synth.make_basis(JF, nv)
    iI, iF = synth.make_degenerate_inflation(bI), synth.make_degenerate_inflation(bF)
    nI, nF = int(iI.Ntot[E]), int(iF.Ntot[E])
    vl = synth.make_eigvecs(nI, JI, E, device="cuda", nstates=n_lower)
    vu = synth.make_eigvecs(nF, JF, E, device="cuda")
    eI = synth.make_energies(nI, JI, E)[:n_lower]
    eF = synth.make_energies(nF, JF, E)
    p = synth.Problem(nv, [JI, JF], "c3e", 3, synth.degen_of("c3e"), synth.selection_of("c3e"),
                      synth.igamma_pair_of(synth.selection_of("c3e")), [bI, bF], [iI, iF],
                      [synth.classes_of(b, "c3e") for b in (bI, bF)], synth.make_dipole(nv),
                      {(0, E): synth.Block(JI, 0, E, vl, eI), (1, E): synth.Block(JF, 1, E, vu, eF)})
    eng = gainls.Engine(11, 3, 2)
    gainls.upload_problem(eng, p)
    f = gainls.make_filters([1.0] * 3, p.isym_pairs, p.igamma_pair, p.sym_degen, (-1e9, 1e9), (-1e9, 1e9))
    lo, up = list(range(n_lower)), list(range(nF))
    setup_s = time.perf_counter() - t0
    for _ in range(args.warmup):
        eng.run_pair(0, E, 1, E, lo, up, gainls.PATH_SPLIT, filters=f)
    torch.cuda.synchronize()
    dev, g1, g2 = [], [], []
    t1 = time.perf_counter()
    for _ in range(args.steps):
        st = eng.run_pair(0, E, 1, E, lo, up, gainls.PATH_SPLIT, filters=f)
        dev.append(st["device_ms"])
        g1.append(st["gemm1_ms"])
        g2.append(st["gemm2_ms"])
    torch.cuda.synchronize()
    wall_ms = (time.perf_counter() - t1) * 1e3 / args.steps
    S_split = eng.lines(eI, eF, JI, JF, ndeg=(2, 2), want=("S",))["S"].copy()
    sp = eng.run_pair(0, E, 1, E, lo, up, gainls.PATH_PLAIN_FP64, filters=f)
    S_plain = eng.lines(eI, eF, JI, JF, ndeg=(2, 2), want=("S",))["S"]
    m = S_plain > 1e-10 * S_plain.max()
    rel = np.abs(S_split[m] - S_plain[m]) / S_plain[m]
    ms = float(np.median(dev))
    lines = n_lower * nF
    out = {"mode": "degenerate", "workload": f"N_v={nv}, J''={JI} E ({nI} functions) -> J'={JF} E ({nF} functions), "
                                             f"{n_lower} lowest lower states x {nF} upper states, 4 component pairs",
           "lines": lines, "component_pairs": 4, "setup_s": setup_s,
           "split_device_ms": ms, "split_wall_ms": wall_ms, "lines_per_s_device": lines / (ms * 1e-3),
           "gemm1_ms": float(np.median(g1)), "gemm2_ms": float(np.median(g2)),
           "plain_fp64_device_ms": sp["device_ms"], "speedup_vs_plain_fp64": sp["device_ms"] / ms,
           "max_rel_err_S_vs_plain": float(rel.max()), "p99_rel_err_S_vs_plain": float(np.quantile(rel, 0.99)),
           "lines_checked": int(m.sum()), "domain": "S > 1e-10 S_max"}
    print(json.dumps(out), flush=True)
    eng.close()


def batch_plan(args):
    """Many block pairs: every allowed (J'', Gamma'') -> (J', Gamma') pair of J = 0..jmax, four
    symmetries, lower states below 4000 cm^-1 against every upper state (the reference's
    intensity filter; J = J_max pairs excluded), run one after another through the split
    path and once through the plain FP64 path.  One JSON line: transitions per second over
    the whole plan (device time and wall time), the time of the largest pairs, and the
    accuracy of S against the plain path."""
    import torch
    torch.cuda.set_device(0)
    import gainls
    import synth
    nv, jmax = args.batch_nv, args.batch_jmax
    t0 = time.perf_counter()
    p = synth.make_problem(nv, list(range(jmax + 1)), "c4", qr_device="cuda")
    eng = gainls.Engine(jmax, p.nsym, 1)
    gainls.upload_problem(eng, p)
    filt = gainls.make_filters([1.0] * p.nsym, p.isym_pairs, p.igamma_pair, p.sym_degen, (0.0, 4000.0),
                               (-1e9, 1e9), (-1e9, 1e9), 0.0, jmax)
    table = gainls.state_table(p.st_energy, p.st_J, p.st_jind, p.st_gamma, p.st_ndeg, p.st_ilevel)
    pairs = gainls.plan_pairs(filt, table)
    setup_s = time.perf_counter() - t0
    trans = [len(lo) * len(up) for *_, lo, up in pairs]
    total = int(sum(trans))

    def sweep(path):
        dev, amps = [], []
        torch.cuda.synchronize()
        w0 = time.perf_counter()
        for jI, gI, jF, gF, lo, up in pairs:
            st = eng.run_pair(jI, gI, jF, gF, lo, up, path)
            dev.append(st["device_ms"])
        torch.cuda.synchronize()
        return dev, (time.perf_counter() - w0) * 1e3

    for _ in range(max(1, args.warmup)):
        sweep(gainls.PATH_SPLIT)
    runs = [sweep(gainls.PATH_SPLIT) for _ in range(max(1, args.steps))]
    dev_ms = [float(np.sum(d)) for d, _ in runs]
    wall_ms = [w for _, w in runs]
    per_pair = np.median(np.array([d for d, _ in runs]), axis=0)
    # the same plan over several engines of this GPU (gain_run_plan: one stream and host
    # thread each, largest pairs first), wall time of the whole plan
    plan = None
    if args.batch_engines > 1:
        engines = [eng]
        for _ in range(args.batch_engines - 1):
            e2 = gainls.Engine(jmax, p.nsym, 1)
            gainls.upload_problem(e2, p)
            engines.append(e2)
        for _ in range(max(1, args.warmup)):
            gainls.run_plan(engines, pairs, gainls.PATH_SPLIT)
        pw = []
        for _ in range(max(1, args.steps)):
            torch.cuda.synchronize()
            w0 = time.perf_counter()
            gainls.run_plan(engines, pairs, gainls.PATH_SPLIT)
            torch.cuda.synchronize()
            pw.append((time.perf_counter() - w0) * 1e3)
        plan = {"engines": len(engines), "wall_ms": float(np.median(pw)),
                "transitions_per_s_wall": total / (np.median(pw) * 1e-3),
                "speedup_vs_one_engine_wall": float(np.median(wall_ms)) / float(np.median(pw))}
        for e2 in engines[1:]:
            e2.close()
    # the grouped plan: every pair's split path in two grouped tensor-core launches, captured
    # in a CUDA graph and replayed; tile shape and second-GEMM digits per size class from the
    # autotuner (first use, included in the creation time)
    c0 = time.perf_counter()
    gplan = gainls.Plan(eng, pairs, autotune=True)
    create_s = time.perf_counter() - c0
    for _ in range(max(1, args.warmup)):
        gplan.run()
    gdev, gwall = [], []
    for _ in range(max(1, args.steps)):
        torch.cuda.synchronize()
        w0 = time.perf_counter()
        ps, _, _ = gplan.run()
        gwall.append((time.perf_counter() - w0) * 1e3)
        gdev.append(ps["device_ms"])
    grouped = {"device_ms": float(np.median(gdev)), "wall_ms": float(np.median(gwall)),
               "transitions_per_s_device": total / (np.median(gdev) * 1e-3),
               "transitions_per_s_wall": total / (np.median(gwall) * 1e-3),
               "speedup_vs_one_engine_wall": float(np.median(wall_ms)) / float(np.median(gwall)),
               "gemm1_ms": ps["gemm1_ms"], "gemm2_ms": ps["gemm2_ms"],
               "stages_ms": {"eigenvector_digits": ps["digits_ms"], "gemm1": ps["gemm1_ms"],
                             "h_refinement_and_digits": ps["middle_ms"], "gemm2": ps["gemm2_ms"],
                             "amplitude_refinement": ps["refine_ms"]},
               "grouped_launches": 2, "graph_nodes": ps["graph_nodes"], "kernel_nodes": ps["kernel_launches"],
               "gemm1_tiles": ps["gemm1_tiles"], "gemm2_tiles": ps["gemm2_tiles"], "units": ps["units"],
               "tile": "256x128 (CTA pairs)" if ps["pair"] else "128x128",
               "autotuned": {"tune_ms": ps["tune_ms"], "create_s": create_s,
                             "gemm2_digits_by_K_class": {c: (f"beta={b} x{sl}" if b else None) for c, b, sl in
                                                         zip(("K<=2048", "K<=8192", "K<=16384", "K>16384"),
                                                             ps["beta2"], ps["slices2"])}},
               "tensor_flops": ps["tensor_flops"],
               "tensor_tflops_in_gemms": ps["tensor_flops"] / ((ps["gemm1_ms"] + ps["gemm2_ms"]) * 1e-3) / 1e12}
    # accuracy and time of the plain FP64 path, pair by pair (split amplitudes from the plan)
    worst, plain_ms, nchk = 0.0, 0.0, 0
    for q, (jI, gI, jF, gF, lo, up) in enumerate(pairs):
        a = gplan.amp(q)
        st = eng.run_pair(jI, gI, jF, gF, lo, up, gainls.PATH_PLAIN_FP64)
        plain_ms += st["device_ms"]
        r = eng.fetch_amp()
        S, Sr = a * a, r * r
        m = Sr > 1e-10 * Sr.max()
        if m.any():
            worst = max(worst, float(np.max(np.abs(S[m] - Sr[m]) / Sr[m])))
            nchk += int(m.sum())
    gplan.close()
    order = np.argsort(-per_pair)[:5]
    out = {"mode": "batch", "workload": f"N_v={nv}, J=0..{jmax}, 4 symmetries, all allowed block pairs, "
                                        "lower states E < 4000 cm^-1 x all upper states",
           "pairs": len(pairs), "transitions": total, "setup_s": setup_s,
           "split_device_ms": float(np.median(dev_ms)), "split_wall_ms": float(np.median(wall_ms)),
           "transitions_per_s_device": total / (np.median(dev_ms) * 1e-3),
           "transitions_per_s_wall": total / (np.median(wall_ms) * 1e-3),
           "plain_fp64_device_ms": plain_ms, "speedup_vs_plain_fp64": plain_ms / float(np.median(dev_ms)),
           "max_rel_err_S_vs_plain": worst, "lines_checked": nchk, "domain": "S > 1e-10 S_max of each pair",
           "largest_pairs": [{"pair": list(pairs[i][:4]), "lower": len(pairs[i][4]), "upper": len(pairs[i][5]),
                              "ms": float(per_pair[i])} for i in order],
           "pairs_under_1M_transitions_ms": float(np.sum([per_pair[i] for i in range(len(pairs))
                                                          if trans[i] < 1_000_000])),
           "plan": plan, "grouped_plan": grouped}
    print(json.dumps(out), flush=True)
    eng.close()


def batch_stream(args):
    """Many block pairs at the full batching size: N_v = 2000, J = 0..30, four symmetries,
    every allowed (J'', Gamma'') -> (J', Gamma') pair (|dJ| <= 1, Gamma' = Gamma'' ^ 1,
    J'' + J' >= 1, not both J_max), lower states below 4000 cm^-1 against every upper state.
    The upper eigenvectors alone (318 GB in FP64) exceed one GPU, so the pairs run in waves,
    one wave per upper block: its eigenvectors and the lower states of its (up to three) lower
    blocks are made on the device (a fast orthonormal generator: Kronecker products of QR
    factors, rows and columns permuted), uploaded into the engine (device to device), the
    wave's jobs run as one grouped plan (two grouped tensor-core launches in a CUDA graph), and
    the blocks are released.  Each wave's plan is replayed once after its first (capturing)
    run; the device time of that replay is summed.  A sample of lower states of the largest
    job of every tenth wave is checked against the plain FP64 path.  One JSON line."""
    import torch
    torch.cuda.set_device(0)
    import gainls
    import synth
    nv, jmax = args.batch_nv, args.batch_jmax
    t0 = time.perf_counter()
    bases = [synth.make_basis(J, nv) for J in range(jmax + 1)]
    infl = [synth.inflation_of(b, "c4", 4) for b in bases]
    eng = gainls.Engine(jmax, 4, 1)
    for jind, (b, inf) in enumerate(zip(bases, infl)):
        eng.upload_basis(jind, b.J, b.K, b.tau, b.vib, b.kblock, b.kstart)
        eng.upload_inflation(jind, inf.icontr, inf.ijterms, b.dimen, inf.maxcoeff, inf.matsize, inf.N, inf.repres,
                             inf.Ntot, inf.sdeg)
    eng.upload_dipole(synth.make_dipole(nv).reshape(-1), nv, 0, nv, nv)
    dims = {(J, c): int(infl[J].Ntot[c]) for J in range(jmax + 1) for c in range(4)}
    nlow = {k: int(np.searchsorted(synth.make_energies(n, k[0], k[1]), 4000.0)) for k, n in dims.items()}
    waves = []
    for JF in range(jmax + 1):
        for cF in range(4):
            jobs = []
            for JI in (JF - 1, JF, JF + 1):
                cI = cF ^ 1
                if JI < 0 or JI > jmax or JI + JF < 1 or (JI == jmax and JF == jmax):
                    continue
                if nlow[(JI, cI)] == 0 or dims[(JF, cF)] == 0:
                    continue
                jobs.append((JI, cI, JF, cF, list(range(nlow[(JI, cI)])), list(range(dims[(JF, cF)]))))
            if jobs and (args.stream_upper_j < 0 or JF == args.stream_upper_j):
                waves.append(((JF, cF), jobs))
    setup_s = time.perf_counter() - t0
    total = sum(len(j[4]) * len(j[5]) for _, jobs in waves for j in jobs)
    dev_ms, wall_ms, gen_s, worst, nchk = 0.0, 0.0, 0.0, 0.0, 0
    biggest = None
    sampled = []
    t_all = time.perf_counter()
    for w, ((JF, cF), jobs) in enumerate(waves):
        g0 = time.perf_counter()
        need = {(JF, cF): dims[(JF, cF)]}
        for JI, cI, *_ in jobs:
            need.setdefault((JI, cI), nlow[(JI, cI)])
        for (J, c), rows in need.items():
            U = synth.make_eigvecs_kron(dims[(J, c)], J, c, "cuda")
            rows_t = U[:rows].contiguous() if (J, c) != (JF, cF) else U
            eng.upload_eigvecs_device(J, c, rows_t.data_ptr(), int(rows_t.shape[0]), dims[(J, c)])
            del U, rows_t
        torch.cuda.synchronize()
        torch.cuda.empty_cache()   # the generator's blocks go back to the device for the plan
        gen_s += time.perf_counter() - g0
        w0 = time.perf_counter()
        try:
            plan = gainls.Plan(eng, [(a, b, c, d, lo, up) for a, b, c, d, lo, up in jobs])
        except gainls.GainError as exc:
            free, total = torch.cuda.mem_get_info()
            raise RuntimeError(f"wave {w} (upper block J={JF} Gamma={cF}, {len(jobs)} jobs): {exc}; device memory "
                               f"free {free / 1e9:.1f} of {total / 1e9:.1f} GB") from exc
        plan.run()
        ps, js, st = plan.run()
        wall_ms += (time.perf_counter() - w0) * 1e3
        dev_ms += ps["device_ms"]
        trans = sum(len(j[4]) * len(j[5]) for j in jobs)
        if args.stream_upper_j >= 0:   # the same jobs one by one through single-pair runs
            single = []
            for JI, cI, _, _, lo, up in jobs:
                eng.run_pair(JI, cI, JF, cF, lo, up, gainls.PATH_SPLIT)
                s1 = eng.run_pair(JI, cI, JF, cF, lo, up, gainls.PATH_SPLIT)
                single.append({"device_ms": s1["device_ms"], "gemm1_ms": s1["gemm1_ms"], "gemm2_ms": s1["gemm2_ms"],
                               "beta2": s1["beta2"], "slices2": s1["slices2"], "chunks2": s1["chunks2"],
                               "refined": s1["refined"], "tensor_flops": s1["tensor_flops"]})
            print(json.dumps({"wave": [JF, cF], "plan": {k: ps[k] for k in ("device_ms", "gemm1_ms", "gemm2_ms",
                                                                           "tensor_flops", "refined", "pair")},
                              "jobs": [[len(j[4]), len(j[5])] for j in jobs], "single_pair_runs": single}),
                  flush=True)
        if biggest is None or trans > biggest["transitions"]:
            biggest = {"upper_block": [JF, cF], "jobs": len(jobs), "transitions": trans, "device_ms": ps["device_ms"],
                       "gemm1_ms": ps["gemm1_ms"], "gemm2_ms": ps["gemm2_ms"], "graph_nodes": ps["graph_nodes"],
                       "tiles": [ps["gemm1_tiles"], ps["gemm2_tiles"]],
                       "tensor_tflops_in_gemms": ps["tensor_flops"] / ((ps["gemm1_ms"] + ps["gemm2_ms"]) * 1e-3) / 1e12}
        if w % 10 == 0 or args.stream_upper_j >= 0:   # accuracy sample: two lower states of the largest job
            q = int(np.argmax([len(j[4]) * len(j[5]) for j in jobs]))
            JI, cI, _, _, lo, up = jobs[q]
            a = plan.amp(q)
            rows = [0, len(lo) // 2]
            eng.run_pair(JI, cI, JF, cF, [lo[r] for r in rows], up, gainls.PATH_PLAIN_FP64)
            ref = eng.fetch_amp()
            S, Sr = a[rows] ** 2, ref ** 2
            if not (np.isfinite(S).all() and np.isfinite(Sr).all()):
                raise RuntimeError(f"wave {w} (upper block J={JF} Gamma={cF}): non-finite line strengths")
            m = Sr > 1e-10 * Sr.max()
            err = float(np.max(np.abs(S[m] - Sr[m]) / Sr[m])) if m.any() else 0.0
            worst = max(worst, err)
            nchk += int(m.sum())
            sampled.append({"upper_block": [JF, cF], "lower_block": [JI, cI], "lines_checked": int(m.sum()),
                            "max_rel_err_S": err, "S_max": float(Sr.max())})
        plan.close()
        for (J, c) in need:
            eng.release_eigvecs(J, c)
    total_wall = time.perf_counter() - t_all
    out = {"mode": "batch_stream",
           "workload": f"N_v={nv}, J=0..{jmax}, 4 symmetries, all allowed block pairs, lower states E < 4000 cm^-1 "
                       "x all upper states; one grouped plan per upper block (wave)",
           "pairs": sum(len(j) for _, j in waves), "waves": len(waves), "transitions": total,
           "largest_block": max(dims.values()), "setup_s": setup_s,
           "device_ms": dev_ms, "transitions_per_s_device": total / (dev_ms * 1e-3),
           "plan_wall_ms": wall_ms, "generation_and_upload_s": gen_s, "total_wall_s": total_wall,
           "largest_wave": biggest,
           "accuracy_sample": {"max_rel_err_S_vs_plain": worst, "lines_checked": nchk,
                               "sample": "2 lower states of the largest job of every 10th wave, all upper states",
                               "domain": "S > 1e-10 S_max", "waves": sampled},
           "eigenvectors": "Kronecker products of seeded QR factors, rows/columns permuted (device)"}
    print(json.dumps(out), flush=True)
    eng.close()


def reference_gpu_sample(inp, n_lower: int) -> dict:
    """The reference's own GPU kernels (GPU/dipole_GPU.cu, compiled unmodified into
    oracle/_ref/dipole_GPU.cubin) in GpuManager's call pattern (oracle/ref_harness.cu): per
    lower state the expansion and one K-block launch per K'; per upper state the expansion,
    cublasDdot, an 8-byte copy back and a synchronisation.  One host thread (the reference
    overlaps such loops over its OpenMP threads, main.cpp:292); a sample of lower states of
    the workload; wall time of the whole call."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import ref_harness
    import synth
    import threej
    nv = inp["nv"]
    rule = inp.get("rule", "c4")
    p = synth.Problem(nv, [JI, JF], rule, 4, np.ones(4, np.int32), synth.selection_of(rule),
                      synth.igamma_pair_of(synth.selection_of(rule)), inp["bases"], inp["infl"],
                      [synth.classes_of(b, rule) for b in inp["bases"]], inp["dipole"],
                      {(0, GI): synth.Block(JI, 0, GI, inp["vl"][:n_lower], inp["eI"][:n_lower]),
                       (1, GF): synth.Block(JF, 1, GF, inp["vu"], inp["eF"])})
    NU = inp["vu"].shape[0]
    tj = threej.threej_table(11)
    t0 = time.perf_counter()
    _, _, loop_s = ref_harness.run_pair(p, 0, GI, 1, GF, list(range(n_lower)), list(range(NU)), tj, 11)
    secs = time.perf_counter() - t0
    n = n_lower * NU
    return {"value": n / secs, "unit": UNIT, "per_transition_loop_us": 1e6 * loop_s / n,
            "sample": f"{n_lower} lower states x {NU} upper states of the workload ({n} transitions, {secs:.2f} s)",
            "method": "reference GPU kernels, one host thread, GpuManager call pattern"}


def reference_arm(args, ws, rank):
    if rank != 0:
        return
    inp = make_inputs(args.small, 0, None, orthonormal=False)
    sample = 2 if not args.small else 4
    vals = []
    for i in range(args.warmup + args.steps):
        r = cpu_baseline(inp, sample)
        if i >= args.warmup:
            vals.append(r["value"])
    v = float(np.median(vals))
    out = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": 1e3 * sample * inp["vu"].shape[0] / v,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
           "data": "synthetic", "impl": "reference",
           "config": {"workload": WORKLOAD, "sample": f"{sample} lower states per step"},
           "cpu_baseline": {"value": v, "unit": UNIT, "cores": r["cores"], "kind": "port",
                            "sample": r["sample"]},
           "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    # an extra data point beside the CPU arm: the reference's own GPU kernels on this GPU
    try:
        import torch
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import ref_harness
        if torch.cuda.is_available() and ref_harness.available():
            out["reference_gpu_kernels"] = reference_gpu_sample(inp, 2)
        else:
            out["reference_gpu_kernels"] = {"unavailable": "no GPU or no compiled reference kernels"}
    except Exception as exc:   # the extra data point never fails the arm
        out["reference_gpu_kernels"] = {"unavailable": str(exc).splitlines()[0][:200]}
    print(json.dumps(out), flush=True)


# ------------------------------------------------------------------------- our arm
def main():
    args = parse()
    ws, rank, local = dist_info()
    if args.precision_sweep:
        return precision_sweep(args)
    if args.adjoint:
        return adjoint_check(args)
    if args.batch_stream:
        if args.batch_nv == 200:
            args.batch_nv = 2000
        return batch_stream(args)
    if args.batch:
        return batch_plan(args)
    if args.degenerate:
        return degenerate_pair(args)
    if args.impl == "reference":
        if ws > 1 and rank != 0:
            return
        return reference_arm(args, ws, rank)
    import torch
    torch.cuda.set_device(local)
    dist = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    import gainls
    inp = make_inputs(args.small, rank, "cuda", n_lower_override=args.lower, rule=args.rule)
    eng = setup_engine(inp, local)
    B, NU = inp["vl"].shape[0], inp["vu"].shape[0]
    lo, up = list(range(B)), list(range(NU))
    transitions = B * NU

    def step():
        return eng.run_pair(0, GI, 1, GF, lo, up, gainls.PATH_SPLIT)

    for _ in range(args.warmup):
        st = step()
    # timed region: device time of each step from CUDA events on the engine's stream
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    ms_list, g1, g2 = [], [], []
    with ClockSampler(local) as clk:
        t0 = time.perf_counter()
        for _ in range(args.steps):
            st = step()
            ms_list.append(st["device_ms"])
            g1.append(st["gemm1_ms"])
            g2.append(st["gemm2_ms"])
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
    total_ms = max_over_ranks(float(np.sum(ms_list)), dist, "cuda")
    if dist:
        dist.barrier()
    ms_step = total_ms / args.steps
    value = ws * transitions / (ms_step * 1e-3)

    # accuracy of this run against (a) the double-double oracle on sampled lower states and
    # (b) the plain FP64 path (the reference's own method) on every transition
    split_amp = eng.fetch_amp().copy()
    extra = {}
    if rank == 0 and not args.no_cpu:
        sample = list(range(0, B, max(1, B // 8)))[:8]
        t0 = time.perf_counter()
        dd = oracle_sample(inp, sample)
        dd_secs = time.perf_counter() - t0
        e_split = s_rel_err(split_amp[sample] ** 2, dd ** 2)
        extra["accuracy"] = {"reference": "double-double oracle (oracle/gain_oracle.c, DD mode)",
                             "oracle_sample": f"{len(sample)} lower states (rows {sample[0]}..{sample[-1]} step "
                                              f"{sample[1] - sample[0] if len(sample) > 1 else 0}) x {NU} upper "
                                              f"states ({dd_secs:.1f} s on {os.cpu_count()} cores)",
                             "lines_checked": e_split[2], "max_rel_err_S": e_split[0], "p99_rel_err_S": e_split[1],
                             "domain": "S > 1e-10 S_max", "refined_lines": st["refined"],
                             "uncertified": st["uncertified"], "uncertified_weak": st["uncertified_weak"]}
    if not args.no_plain:
        sp = eng.run_pair(0, GI, 1, GF, lo, up, gainls.PATH_PLAIN_FP64)
        plain_amp = eng.fetch_amp()
        e_fp = s_rel_err(split_amp ** 2, plain_amp ** 2)
        extra["plain_fp64"] = {"value": transitions / (sp["device_ms"] * 1e-3), "unit": UNIT,
                               "ms_per_step": sp["device_ms"], "kernel_launches": sp["kernel_launches"]}
        extra["speedup_vs_plain_fp64"] = extra["plain_fp64"]["ms_per_step"] / ms_step
        acc = extra.setdefault("accuracy", {"domain": "S > 1e-10 S_max", "refined_lines": st["refined"],
                                            "uncertified": st["uncertified"]})
        acc["vs_plain_fp64_all_lines"] = {"lines_checked": e_fp[2], "max_rel_err_S": e_fp[0],
                                          "p99_rel_err_S": e_fp[1]}
        if "oracle_sample" in acc:
            e_pl = s_rel_err(plain_amp[sample] ** 2, dd ** 2)
            acc["plain_fp64_vs_oracle"] = {"max_rel_err_S": e_pl[0], "p99_rel_err_S": e_pl[1]}
        eng.run_pair(0, GI, 1, GF, lo, up, gainls.PATH_SPLIT)   # leave the split result resident

    # e2e: host buffers through the C ABI (inputs up, S and A down), every step
    vl_h, vu_h = pinned(inp["vl"]), pinned(inp["vu"])
    S_h, A_h = pinned(np.zeros((B, NU))), pinned(np.zeros((B, NU)))
    def e2e_step_once():
        # queued copies: the upper vectors stream in while the lower side is computed; the
        # S and A copies of this step overlap the next step's uploads and run (the link is
        # full duplex), and every step's copies land before the next step's line assembly
        eng.upload_eigvecs_async(0, GI, vl_h)
        eng.upload_eigvecs_async(1, GF, vu_h)
        eng.run_pair(0, GI, 1, GF, lo, up, gainls.PATH_SPLIT)
        eng.lines(inp["eI"], inp["eF"], JI, JF, intensity=False, want=("S", "A"), out_S=S_h, out_A=A_h,
                  asynchronous=True)

    for _ in range(args.warmup):
        e2e_step_once()
    eng.lines_wait()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_step_once()
    eng.lines_wait()
    torch.cuda.synchronize()
    e2e_serial = (time.perf_counter() - t0) * 1e3 / args.steps
    # the end-to-end route (asynchronous uploads, the upper side in two halves while the upper
    # vectors arrive) gives the device-resident run's line strengths, bit for bit
    e2e_same = bool(np.array_equal(S_h.reshape(B, NU), split_amp * split_amp))

    # pipelined: two eigenvector slots (the same blocks uploaded under a second pair of block
    # indices); each step first queues the NEXT step's uploads into the other slot, then runs
    # its own pair, so the copies of step k+1 overlap the run of step k.  Every step still
    # copies its own inputs and reads back its S and A inside the timed region.
    for jind, (b, inf) in enumerate(zip(inp["bases"], inp["infl"])):
        eng.upload_basis(2 + jind, b.J, b.K, b.tau, b.vib, b.kblock, b.kstart)
        eng.upload_inflation(2 + jind, inf.icontr, inf.ijterms, b.dimen, inf.maxcoeff, inf.matsize, inf.N,
                             inf.repres, inf.Ntot, inf.sdeg)
    slots = [(0, 1), (2, 3)]

    def e2e_pipelined(n):
        eng.upload_eigvecs_async(slots[0][0], GI, vl_h)
        eng.upload_eigvecs_async(slots[0][1], GF, vu_h)
        for k in range(n):
            a, b = slots[k % 2]
            if k + 1 < n:
                na, nb = slots[(k + 1) % 2]
                eng.upload_eigvecs_async(na, GI, vl_h)
                eng.upload_eigvecs_async(nb, GF, vu_h)
            eng.run_pair(a, GI, b, GF, lo, up, gainls.PATH_SPLIT)
            eng.lines(inp["eI"], inp["eF"], JI, JF, intensity=False, want=("S", "A"), out_S=S_h, out_A=A_h,
                      asynchronous=True)
        eng.lines_wait()

    e2e_pipelined(max(2, args.warmup))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e2e_pipelined(args.steps)
    torch.cuda.synchronize()
    e2e_pipe = (time.perf_counter() - t0) * 1e3 / args.steps
    e2e_same = e2e_same and bool(np.array_equal(S_h.reshape(B, NU), split_amp * split_amp))
    e2e_step = min(e2e_serial, e2e_pipe)
    h2d = inp["vl"].nbytes + inp["vu"].nbytes
    d2h = 2 * B * NU * 8
    text = line_text_bench(eng, inp, max(2, min(args.steps, 5)))

    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    peak = peaks.get("bf16_tflops", 1900.0)
    # algorithmic tensor work of the amplitude GEMM: digit products x 2 B N_up N_F
    NF = int(inp["infl"][1].Ntot[GF])
    prods2 = st["slices2"] * (st["slices2"] + 1) // 2
    alg2 = prods2 * 2.0 * B * NU * NF
    g2ms = float(np.median(g2))
    achieved = alg2 / (g2ms * 1e-3) / 1e12
    traffic = None
    try:
        traffic = json.load(open(os.path.join(ROOT, "profiles", "roofline_traffic.json")))["gemm2_bytes_per_launch"]
    except Exception:
        pass

    cpu = None
    if rank == 0 and not args.no_cpu:
        cpu = cpu_baseline(inp, 4 if args.small else 8)

    if rank == 0:
        out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
               "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
               "vs_baseline": None, "dtype": "bf16", "data": "synthetic",
               "config": {"workload": WORKLOAD + ("" if args.rule == "c4" else f", symmetrisation {args.rule}"),
                          "symmetrisation": args.rule, "lower_states": B, "upper_states": NU, "N_v": inp["nv"],
                          "lower_dim": int(inp["infl"][0].Ntot[GI]), "upper_dim": NF,
                          "l2": "inputs larger than L2 (BF16 digits of the upper vectors ~2 GB per step)",
                          "parallelism": f"replicas by lower-state range x{ws}",
                          "precision": f"Ozaki digits: GEMM1 beta={st['beta1']} x{st['slices1']}, "
                                       f"GEMM2 beta={st['beta2']} x{st['slices2']} chunks={st['chunks2']}; "
                                       "exact FP32 accumulation, FP64 recombination + refinement"},
               "roofline": {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                            "frac": achieved / peak, "traffic": traffic,
                            "kernel": "k_digit_gemm (amplitude GEMM)", "kernel_ms": g2ms,
                            "algorithmic_flops": alg2, "peak_source": "MEASURED_PEAKS.json bf16_tflops (burst)"},
               "cpu_baseline": cpu,
               "e2e": {"value": ws * transitions / (e2e_step * 1e-3), "unit": UNIT, "ms_per_step": e2e_step,
                       "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h, "S_equals_device_run": e2e_same,
                       "ms_per_step_one_slot": e2e_serial, "ms_per_step_pipelined": e2e_pipe,
                       "route": "pipelined: step k+1's uploads queued into a second eigenvector slot during step "
                                "k's run" if e2e_pipe <= e2e_serial else
                                "one slot: each step's uploads stream in while its own run starts"},
               "clocks": clk.summary(),
               "gpu_launches": int(st["kernel_launches"]) * args.steps,
               "gemm1_ms": float(np.median(g1)), "gemm2_ms": g2ms, "wall_ms_per_step": wall * 1e3 / args.steps,
               "tensor_flops_executed_per_step": st["tensor_flops"]}
        if rank == 0 and not args.no_cpu:
            text["cpu_snprintf"] = cpu_text_baseline(eng, inp, 16)
        out["line_list_text"] = text
        out.update(extra)
        print(json.dumps(out), flush=True)
    eng.close()
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
