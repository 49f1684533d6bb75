"""Benchmark of the GB300 three-phonon scattering path.

Default workload (the configuration the benchmark spec's targets are stated on): 5-atom cubic
perovskite (15 modes), 16x16x16 Gamma-centred mesh, adaptive Gaussian smearing, T = 300 K,
seeded per-q1 q' samples of uneven sizes (200-4000 points) in one persistent launch,
seeded Lennard-Jones + Born-Mayer force constants, mixed precision (tensor-core or FP32
contraction, FP64 delta weights and accumulation). The same line carries the
three-plus-four-phonon leg, the adjoint ratio and, as a sub-record, the 2-atom rocksalt
24x24x24 configuration.

One step = one pass of the scattering path (sr%generate: triplet enumeration, fused
pretransform/contraction/accumulation, symmetrisation) over the whole mesh.
  value : accepted irreducible q-triplets per second, device time of the pipeline with all
          inputs resident in HBM (CUDA events on the library's stream)
  e2e   : the same metric through the public API with host buffers: context creation
          (H2D of phonons and force constants), generate (H2D of the samples, D2H of the
          linewidths) and the kappa solve, per step
  cpu_baseline / --impl reference : the oracle's restatement of the reference on the host
          cores (OpenMP), timed on complete q1 groups of the same workload.
  parity : the oracle's linewidths and Xi rows of those q1 groups against the GPU's FP64 and
          mixed-precision results of the same run.

  python bench.py [--gpus 1] [--steps K] [--warmup W] [--impl gb300|reference] [--config NAME]
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "3-phonon triplets/s & κ wall time at 1 GB300, mixed vs FP64 at ≤1e-4 κ rel err"
KAPPA_TIGHT_TOL = 1e-12  # BTE tolerance of the mixed-vs-FP64 kappa comparisons
KAPPA_TIGHT_MAXITER = 400

CONFIGS = {
    "rocksalt24": dict(synth="rocksalt", grid=(24, 24, 24), it=2, temperature=300.0,
                       workload="rocksalt Na/Cl 2-atom (6 modes), 24x24x24 mesh, adaptive smearing, T=300 K, "
                                "full q' grid, no isotope"),
    "perovskite16": dict(synth="perovskite", grid=(16, 16, 16), it=2, temperature=300.0, uneven=(200, 4000),
                         workload="cubic perovskite 5-atom (15 modes), 16x16x16 mesh, adaptive smearing, T=300 K, "
                                  "seeded per-q1 q' samples of 200-4000 points, no isotope"),
    "fcc12": dict(synth="fcc_morse", grid=(12, 12, 12), it=1, temperature=300.0,
                  workload="fcc Morse 1-atom (3 modes), 12x12x12 mesh, Gaussian smearing 1 THz, T=300 K"),
    # small cases of the same kernels for ncu captures (a few hundred MB on the device)
    "rocksalt12": dict(synth="rocksalt", grid=(12, 12, 12), it=2, temperature=300.0,
                       workload="rocksalt Na/Cl 2-atom (6 modes), 12x12x12 mesh, adaptive smearing, T=300 K"),
    "perovskite8": dict(synth="perovskite", grid=(8, 8, 8), it=2, temperature=300.0,
                        workload="cubic perovskite 5-atom (15 modes), 8x8x8 mesh, adaptive smearing, T=300 K"),
    # the smallest cases whose scattering matrix (171 MB, 261 MB) exceeds the 129 MB L2
    "rocksalt16": dict(synth="rocksalt", grid=(16, 16, 16), it=2, temperature=300.0,
                       workload="rocksalt Na/Cl 2-atom (6 modes), 16x16x16 mesh, adaptive smearing, T=300 K, "
                                "full q' grid"),
    "perovskite12": dict(synth="perovskite", grid=(12, 12, 12), it=2, temperature=300.0, uneven=(200, 1700),
                         workload="cubic perovskite 5-atom (15 modes), 12x12x12 mesh, adaptive smearing, T=300 K, "
                                  "seeded per-q1 q' samples of 200-1700 points"),
    # large cell: tcgen05 contraction (beyond 18 modes), mixed precision only
    "supercell40": dict(synth="perovskite_supercell", reps=(2, 2, 2), grid=(8, 8, 8), it=2, temperature=300.0,
                        workload="2x2x2 perovskite supercell, 40 atoms (120 modes), seeded 0.05 A displacements "
                                 "(identity only), 8x8x8 mesh, adaptive smearing, T=300 K, full q' grid"),
    "supercell40_m4": dict(synth="perovskite_supercell", reps=(2, 2, 2), grid=(4, 4, 4), it=2, temperature=300.0,
                           workload="40-atom perovskite supercell (120 modes), 4x4x4 mesh (capture case)"),
}


def log(*a):
    print(*a, file=sys.stderr, flush=True)


INPUT_DIRS = {}  # workload -> directory of its infile.* files (written by setup)


def setup(cfg_name, precision="mixed"):
    from tdep_gb300 import Options, Problem, QLists, synth

    cfg = CONFIGS[cfg_name]
    tmp = tempfile.mkdtemp(prefix="tdg_bench_")
    extra = {"reps": cfg["reps"]} if "reps" in cfg else {}
    d = synth.write_config(cfg["synth"], Path(tmp) / cfg["synth"], seed=1, **extra)
    INPUT_DIRS[cfg_name] = d
    t0 = time.perf_counter()
    prob = Problem.load(d, cfg["grid"], readiso=True)
    log(f"[bench] problem: n_mode={prob.n_mode} n_full={prob.n_full} n_irr={prob.n_irr} n_fc3={prob.n_fc3} "
        f"({time.perf_counter() - t0:.1f}s)")
    opts = Options(temperature=cfg["temperature"], integrationtype=cfg["it"], sigma=1.0, isotopescattering=False,
                   seed=1, precision=precision, itertol=1e-6, itermaxsteps=200)
    if "uneven" in cfg:
        lo, hi = cfg["uneven"]
        rng = np.random.default_rng(1)
        samples = {q: np.sort(rng.choice(np.arange(1, prob.n_full + 1), size=int(rng.integers(lo, hi + 1)),
                                         replace=False)).astype(np.int32) for q in range(1, prob.n_irr + 1)}
        lists = QLists.per_irreducible(prob, samples3=samples)
    else:
        lists = QLists.monte_carlo(prob, opts)
    return cfg, prob, opts, lists


# DRAM bytes (read + write) of one launch of the fused kernel, keyed by workload and path (0 the
# SIMT kernel k_threephonon, 1 the tensor-core kernel k_threephonon_tc), from
# `ncu --metrics dram__bytes_read.sum,dram__bytes_write.sum --clock-control none -k regex:k_threephonon`
# on `python bench.py --profile --config <name> --steps 1 --warmup 1` (a one-pass capture),
# summarised in profiles/. The tensor-core kernel's figure for perovskite16 is its perovskite12
# capture (224.8 MB for 19404 q-triplets) scaled by the q-triplets of one launch (101233):
# its traffic is the Xi row scatter, which grows with the q-triplets.
TRAFFIC_PER_LAUNCH = {("rocksalt16", 0): 40_693_760, ("rocksalt24", 0): 460_600_000,
                      ("perovskite16", 0): 1_098_100_000, ("perovskite12", 1): 224_781_312,
                      ("perovskite16", 1): 1_172_700_000}
KERNEL_NAMES = {
    0: "k_threephonon (fused pretransform, FP32 SIMT contraction, FP64 delta weights)",
    1: "k_threephonon_tc (fused pretransform, tcgen05 BF16x3 contraction with FP32 accumulation in tensor "
       "memory, FP32 delta weights, FP64 sums)",
    2: "large-cell stage: phases, pretransform, 3 tcgen05 BF16x3 GEMM stages, FP64 delta kernel (time of the "
       "whole stage)"}
PRECISION_NOTES = {
    0: "mixed: FP32 pretransform+contraction, FP64 delta weights/occupations/accumulation",
    1: "mixed: FP32 pretransform, BF16x3 tensor-core contraction with FP32 accumulation, FP32 delta weights "
       "of the survivors (FP64 centre differences), FP64 sums/accumulation",
    2: "mixed: FP32 pretransform, BF16x3 tensor-core contraction with FP32 accumulation, FP64 delta "
       "weights/occupations/accumulation"}


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-i", os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0],
                                          "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["active", "hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names[1:], parts[4:8]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return d["hbm_gbs"], d["bf16_tflops"], "measured"
    return 6800.0, 1900.0, "fallback"


def cpu_sample(prob, opts, lists, budget_s=12.0, nthreads=None, keep=False):
    """Time the oracle on complete q1 groups until the budget is used; returns
    (distinct q-triplets covered, seconds, description, threads, rows) where rows holds the
    oracle's (r0, r1, gamma, xi) of every block when keep is set."""
    from oracle import binding as orc

    nthreads = nthreads or os.cpu_count() or 1
    q1s = np.unique(lists.row_q1)
    # blocks of consecutive q1 groups from the middle of the wedge, so that one call keeps
    # every thread busy; each block is whole rows of whole q1 groups
    per_block = max(1, -(-nthreads // max(1, prob.n_mode)))
    start = len(q1s) // 2
    done_trip, done_s, used, kept = 0, 0.0, [], []
    for b0 in range(start, start + len(q1s), per_block):
        block = [q1s[i % len(q1s)] for i in range(b0, b0 + per_block)]
        if len(set(block)) < len(block) or any(q in used for q in block):
            break
        rows = np.nonzero(np.isin(lists.row_q1, block))[0]
        r0, r1 = int(rows[0]), int(rows[-1]) + 1
        if r1 - r0 != rows.size:
            break
        t0 = time.perf_counter()
        gamma, xi, _ = orc.scattering(prob, opts, lists, nthreads=nthreads, rows=(r0, r1))
        done_s += time.perf_counter() - t0
        if keep:
            kept.append((r0, r1, gamma, xi))
        for q1 in block:
            rr = np.nonzero(lists.row_q1 == q1)[0]
            union = np.unique(np.concatenate([lists.list3[lists.ptr3[r]:lists.ptr3[r + 1]] for r in rr]))
            done_trip += len(orc.triplets(prob, int(q1), union.astype(np.int32)))
            used.append(int(q1))
        if done_s >= budget_s:
            break
    desc = (f"oracle restatement (per-row zgeru/dot_product contraction as in scattering_threephonon.f90), "
            f"{len(used)} complete irreducible q1 groups ({done_trip} q-triplets) of the same workload")
    return done_trip, done_s, desc, nthreads, kept


def large_sample_lists(prob, lists):
    """Large cells: one accepted q-triplet (q1 from the middle of the wedge, its first
    accepted q2) sampled by every row; returns (sample lists, q1, its rows)."""
    from oracle import binding as orc
    from tdep_gb300 import QLists

    q1s = np.unique(lists.row_q1)
    q1 = int(q1s[len(q1s) // 2])
    rows = np.nonzero(lists.row_q1 == q1)[0]
    full = lists.list3[lists.ptr3[rows[0]]:lists.ptr3[rows[0] + 1]]
    q2 = next(int(q) for q in full if orc.triplets(prob, q1, np.array([q], np.int32)))
    one = np.full(lists.n_row, q2, np.int32)
    return QLists(lists.row_q1, lists.row_b1, np.arange(lists.n_row + 1, dtype=np.int64), one), q1, rows


def cpu_sample_large(prob, opts, lists, nthreads=None):
    """Large cells: one accepted q-triplet per row for as many rows of one q1 as there are
    host threads (the oracle's cost per q-triplet and row grows as n^5); a GPU q-triplet
    covers all rows of its q1, so the rate is scaled by the rows of that q1. Returns
    (q-triplet equivalents, seconds, description, threads, rows) with rows = [(r0, r1,
    gamma, xi)] of the oracle."""
    from oracle import binding as orc

    nthreads = nthreads or os.cpu_count() or 1
    sample, q1, rows = large_sample_lists(prob, lists)
    r0 = int(rows[0])
    r1 = min(int(rows[-1]) + 1, r0 + nthreads)
    t0 = time.perf_counter()
    gamma, xi, _ = orc.scattering(prob, opts, sample, nthreads=nthreads, rows=(r0, r1))
    secs = time.perf_counter() - t0
    done = (r1 - r0) / rows.size  # q-triplet equivalents: (rows done) / (rows per q-triplet)
    desc = (f"oracle restatement on {r1 - r0} of the {rows.size} rows of one q1, one accepted q-triplet each "
            f"(one q-triplet of the GPU covers all {rows.size} rows)")
    return done, secs, desc, nthreads, [(r0, r1, gamma, xi)]


def oracle_rows_finish(prob, opts, lists, kept):
    """Boundary term, degeneracy averaging and symmetrize_scatmat of the oracle's rows (whole
    q1 groups): returns (row indices, linewidths [n_irr, n_mode] with only those q1 filled,
    symmetrised Xi rows)."""
    from oracle import binding as orc
    from tdep_gb300 import QLists

    idx = np.concatenate([np.arange(r0, r1) for r0, r1, _, _ in kept])
    gamma = np.concatenate([g for _, _, g, _ in kept])
    xi = np.concatenate([x for _, _, _, x in kept])
    sub = QLists(lists.row_q1[idx], lists.row_b1[idx])
    lw, _, _ = orc.finish(prob, opts, sub, gamma, xi)
    return idx, lw, xi


def parity_record(prob, lists, idx, lw_ref, xi_ref, runs):
    """Largest relative linewidth difference over the rows' q1 groups and the Xi entry
    differences (relative to the largest |Xi| of those rows) of each GPU run against the
    oracle. Xi entries that differ beyond 1e-9 of the largest are counted as flips of the
    od_terms > 0 filter (an analytically zero sum rounded to either side of 0 changes how
    many images enter an orbit average); their fraction is reported beside the largest
    difference of the other entries."""
    q1s = np.unique(lists.row_q1[idx]) - 1
    ref = lw_ref[q1s]
    mask = np.abs(ref) > 1e-12 * np.abs(ref).max()
    out = {"rows": int(idx.size), "q1_groups": int(q1s.size)}
    for name, (lw, xi) in runs.items():
        got = lw[q1s]
        out[f"lw_max_rel_{name}"] = float(np.max(np.abs(got[mask] - ref[mask]) / np.abs(ref[mask])))
        if xi is not None and xi_ref is not None:
            d = np.abs(xi - xi_ref) / float(np.abs(xi_ref).max())
            if name == "fp64":
                flips = d > 1e-9
                out["xi_max_rel_fp64"] = float(d[~flips].max()) if (~flips).any() else 0.0
                out["xi_flip_frac_fp64"] = float(flips.mean())
            else:
                out[f"xi_max_rel_{name}"] = float(d.max())
    return out


def setup_oracle(cfg_name):
    """The reference arm's workload built without the library: the oracle's own problem from
    the input files (oracle/problem.py: readers, symmetry, mesh, phonons in numpy) and its own
    MT19937-64 samples, so that this arm runs the oracle alone."""
    from oracle import binding as orc
    from oracle.problem import OracleProblem
    from tdep_gb300 import Options, QLists, synth

    cfg = CONFIGS[cfg_name]
    tmp = tempfile.mkdtemp(prefix="tdg_ref_")
    extra = {"reps": cfg["reps"]} if "reps" in cfg else {}
    d = synth.write_config(cfg["synth"], Path(tmp) / cfg["synth"], seed=1, **extra)
    t0 = time.perf_counter()
    prob = OracleProblem(d, cfg["grid"]).to_problem()
    log(f"[bench] oracle problem: n_mode={prob.n_mode} n_full={prob.n_full} n_irr={prob.n_irr} "
        f"({time.perf_counter() - t0:.1f}s)")
    opts = Options(temperature=cfg["temperature"], integrationtype=cfg["it"], sigma=1.0, isotopescattering=False,
                   seed=1, precision="fp64", itertol=1e-6, itermaxsteps=200)
    if "uneven" in cfg:
        lo, hi = cfg["uneven"]
        rng = np.random.default_rng(1)
        samples = {q: np.sort(rng.choice(np.arange(1, prob.n_full + 1), size=int(rng.integers(lo, hi + 1)),
                                         replace=False)).astype(np.int32) for q in range(1, prob.n_irr + 1)}
        lists = QLists.per_irreducible(prob, samples3=samples)
    else:
        lists = orc.mc_qlists(prob, opts)
    return cfg, prob, opts, lists


def run_reference(args):
    cfg, prob, opts, lists = setup_oracle(args.config)
    per_step = max(2.0, 20.0 / max(1, args.steps))
    large = prob.n_mode > 18
    if not large:
        for _ in range(args.warmup):
            cpu_sample(prob, opts, lists, budget_s=0.5)
    trip, secs = 0, 0.0
    desc, cores = "", os.cpu_count()
    for _ in range(args.steps if not large else 1):
        if large:
            t, s, desc, cores, _ = cpu_sample_large(prob, opts, lists)
        else:
            t, s, desc, cores, _ = cpu_sample(prob, opts, lists, budget_s=per_step)
        trip += t
        secs += s
    value = trip / secs
    line = {"metric": METRIC, "value": value, "unit": "q-triplets/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * secs / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
            "config": {"workload": cfg["workload"]},
            "cpu_baseline": {"value": value, "unit": "q-triplets/s", "cores": cores, "kind": "port", "sample": desc},
            "e2e": {"value": value, "unit": "q-triplets/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def run_profile(args):
    """--profile: warm-up passes then `steps` passes of one stage, nothing else (for ncu):
    scattering (generate), kappa (one generate, then BTE solves), offdiag (one generate,
    then off-diagonal kappa), adjoint (one generate and kappa_SMA, then d kappa_xx / d Phi3
    passes) or fourphonon (the four-phonon terms alone, 27 x 27 pair samples per irreducible
    point)."""
    from tdep_gb300 import Options, Problem, QLists, ScatteringRates, synth

    if args.stage == "fourphonon":
        # the four-phonon terms alone on the workload's cell: seeded pair samples of 27 x 27
        # points per irreducible point (the size of the reference's -qg4ph 3 3 3), as in the
        # three-plus-four-phonon leg of the default run
        cfg = CONFIGS[args.config]
        d = synth.write_config(cfg["synth"], Path(tempfile.mkdtemp(prefix="tdg_prof4_")) / cfg["synth"], seed=1,
                               order4=True)
        prob = Problem.load(d, cfg["grid"], fourthorder=True, readiso=True)
        rng4 = np.random.default_rng(2)
        s4 = {q: tuple(np.sort(rng4.choice(np.arange(1, prob.n_full + 1), size=27, replace=False)).astype(np.int32)
                       for _ in range(2)) for q in range(1, prob.n_irr + 1)}
        lists = QLists.per_irreducible(prob, samples4=s4)
        opts = Options(temperature=cfg["temperature"], integrationtype=cfg["it"], isotopescattering=False, seed=1,
                       precision=args.precision, thirdorder=False, fourthorder=True)
        sr = ScatteringRates(prob)
        for _ in range(args.warmup + args.steps):
            sr.generate(opts, lists)
        log(f"[bench] profile (fourphonon): {sr.stats}")
        sr.close()
        return
    cfg, prob, opts, lists = setup(args.config, precision=args.precision)
    sr = ScatteringRates(prob)
    if args.stage == "scattering":
        for _ in range(args.warmup + args.steps):
            sr.generate(opts, lists)
    elif args.stage == "adjoint":
        sr.generate(opts, lists)
        sr.kappa(opts, maxiter=0)
        kb = np.zeros((3, 3))
        kb[0, 0] = 1.0
        lw_bar = sr.kappa_sma_vjp(opts, kb)
        for _ in range(args.warmup + args.steps):
            sr.adjoint_fc3(opts, lw_bar)
    else:
        sr.generate(opts, lists)
        for _ in range(args.warmup + args.steps):
            if args.stage == "kappa":
                sr.kappa(opts)
            else:
                sr.kappa_offdiag(opts)
    from tdep_gb300._native import autotune_table

    log(f"[bench] profile ({args.stage}): {sr.stats} launch shapes {autotune_table()} graphs {sr.graph_counts()}")
    sr.close()


def fourphonon_leg(cfg_name, steps):
    """Three- plus four-phonon scattering on the C3 perovskite (its batched configuration):
    the same uneven three-phonon samples plus seeded four-phonon pair samples per
    irreducible point (two lists of 27 points, the size of the reference's -qg4ph 3 3 3),
    mixed precision and FP64. Returns q-quartets/s of the added four-phonon work and the
    pass and kappa times."""
    from tdep_gb300 import Options, Problem, QLists, ScatteringRates, synth

    cfg = CONFIGS[cfg_name]
    tmp = tempfile.mkdtemp(prefix="tdg_bench4_")
    d = synth.write_config(cfg["synth"], Path(tmp) / cfg["synth"], seed=1, order4=True)
    prob = Problem.load(d, cfg["grid"], fourthorder=True, readiso=True)
    lo, hi = cfg["uneven"]
    rng = np.random.default_rng(1)
    s3 = {q: np.sort(rng.choice(np.arange(1, prob.n_full + 1), size=int(rng.integers(lo, hi + 1)),
                                replace=False)).astype(np.int32) for q in range(1, prob.n_irr + 1)}
    rng4 = np.random.default_rng(2)
    s4 = {q: tuple(np.sort(rng4.choice(np.arange(1, prob.n_full + 1), size=27, replace=False)).astype(np.int32)
                   for _ in range(2)) for q in range(1, prob.n_irr + 1)}
    lists = QLists.per_irreducible(prob, samples3=s3, samples4=s4)
    out = {"workload": cfg["workload"] + "; plus four-phonon: seeded pair samples of 27 x 27 points per irreducible q"}
    sr = ScatteringRates(prob)
    for prec in ("mixed", "fp64"):
        o34 = Options(temperature=cfg["temperature"], integrationtype=cfg["it"], isotopescattering=False, seed=1,
                      precision=prec, fourthorder=True, itertol=1e-6, itermaxsteps=200)
        o3 = Options(**{**o34.__dict__, "fourthorder": False})
        ms34, ms3 = [], []
        for i in range(steps + 1):  # the first of each is a warm-up
            sr.generate(o3, lists)
            if i:
                ms3.append(sr.stats["device_ms"])
            sr.generate(o34, lists)
            if i:
                ms34.append(sr.stats["device_ms"])
        quart = sr.stats["quartets"]
        t0 = time.perf_counter()
        sr.kappa(o34)
        kms = 1e3 * (time.perf_counter() - t0)
        _, ki = sr.kappa(o34, maxiter=KAPPA_TIGHT_MAXITER, tol=KAPPA_TIGHT_TOL)
        d4 = float(np.median(ms34)) - float(np.median(ms3))
        out[prec] = {"q_quartets": int(quart), "pass_ms_3ph_4ph": float(np.median(ms34)),
                     "pass_ms_3ph_only": float(np.median(ms3)), "fourphonon_ms": d4,
                     "q_quartets_per_s": quart / (d4 / 1e3) if d4 > 0 else None, "kappa_wall_ms": kms,
                     "kappa_xx": float(ki[0, 0]), "kappa_tol": KAPPA_TIGHT_TOL}
    sr.close()
    out["mixed_speedup_3ph_4ph"] = out["fp64"]["pass_ms_3ph_4ph"] / out["mixed"]["pass_ms_3ph_4ph"]
    out["kappa_rel_err_mixed_vs_fp64"] = abs(out["mixed"]["kappa_xx"] / out["fp64"]["kappa_xx"] - 1)
    return out


def measure(cfg_name, args, cpu_budget, with_adjoint=True):
    """Device passes, FP64 leg, adjoint ratio, e2e, CPU sample and parity rows of one
    configuration; returns a dict (the bench line's fields for that configuration)."""
    import torch

    from tdep_gb300 import ScatteringRates
    from tdep_gb300._native import autotune_table

    cfg, prob, opts, lists = setup(cfg_name, precision="mixed")
    n = prob.n_mode
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")  # > 129 MB L2
    small = n <= 18  # the FP64 path exists

    sr = ScatteringRates(prob)
    for _ in range(args.warmup):
        sr.generate(opts, lists)
    # ---- resident timing: device time of each pipeline pass, L2 flushed between passes ----
    clocks = ClockSampler()
    clocks.start()
    dev_ms, fused_ms, launches, trip = [], [], 0, 0
    torch.cuda.synchronize()
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        sr.generate(opts, lists)
        st = sr.stats
        dev_ms.append(st["device_ms"])
        fused_ms.append(st["threephonon_ms"])
        launches += st["launches"]
        trip = st["triplets"]
    torch.cuda.synchronize()
    clk = clocks.stop()
    graphs = sr.graph_counts()
    path, shape = sr.last_path(), sr.last_launch()
    lw_mixed = sr.linewidth.copy()
    xi_mixed = sr.Xi if small else None
    t0 = time.perf_counter()
    ks32, ki32 = sr.kappa(opts)
    kappa_ms = 1e3 * (time.perf_counter() - t0)
    kappa_iters = sr.n_iter
    # the precision figure compares BTE solutions converged far below the default tolerance,
    # so that a different stopping iteration does not count as arithmetic error
    _, ki32 = sr.kappa(opts, maxiter=KAPPA_TIGHT_MAXITER, tol=KAPPA_TIGHT_TOL)
    stats = dict(sr.stats)

    adjoint = fp64 = None
    if with_adjoint:
        # ---- adjoint pass (d kappa_sma,xx / d Phi3) on the same workload, against the forward ----
        kb = np.zeros((3, 3))
        kb[0, 0] = 1.0
        adj_ms = []
        for _ in range(max(2, args.steps // 2) if small else 1):
            sr.generate(opts, lists)
            fwd_ms = sr.stats["device_ms"]
            sr.kappa(opts, maxiter=0)
            sr.adjoint_fc3(opts, sr.kappa_sma_vjp(opts, kb))
            adj_ms.append(sr.adjoint_stats["ms"])
        adjoint = {"ms": float(np.median(adj_ms)), "forward_ms": fwd_ms,
                   "ratio_to_forward": float(np.median(adj_ms)) / fwd_ms,
                   "what": "tdg_adjoint_fc3 after tdg_kappa_sma_vjp: d kappa_xx / d mwm for all "
                           f"{prob.n_fc3 * 27} third-order entries, mixed precision, Psi recomputed"
                           + ("" if small else "; large-cell path: back-contraction on the tensor cores")}
    lw64 = xi64 = None
    o64 = type(opts)(**{**opts.__dict__, "precision": "fp64"})
    if small:
        # ---- FP64 path on the same workload: kappa error bar and speedup ----
        sr.generate(o64, lists)  # warm-up: the first FP64 call also runs the launch-shape trials
        sr.generate(o64, lists)
        fp64_ms = sr.stats["device_ms"]
        lw64 = sr.linewidth.copy()
        xi64 = sr.Xi
        _, ki64 = sr.kappa(o64, maxiter=KAPPA_TIGHT_MAXITER, tol=KAPPA_TIGHT_TOL)
        kappa_err = float(np.max(np.abs(ki32 - ki64)) / np.max(np.abs(ki64)))
        fp64 = {"value": trip / (fp64_ms / 1e3), "ms_per_step": fp64_ms,
                "mixed_speedup": fp64_ms / float(np.mean(dev_ms)), "kappa_rel_err_mixed_vs_fp64": kappa_err}
    sr.close()

    # ---- end to end through the public API with host buffers ----
    def e2e_run(o, steps):
        e2e_s, parts = [], []
        h2d = d2h = 0
        for _ in range(steps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            s2 = ScatteringRates(prob)
            t1 = time.perf_counter()
            s2.generate(o, lists)
            t2 = time.perf_counter()
            s2.kappa_offdiag(o)
            s2.kappa(o)
            t3 = time.perf_counter()
            h2d, d2h = s2.transfer_bytes()
            s2.close()
            torch.cuda.synchronize()
            t4 = time.perf_counter()
            e2e_s.append(t4 - t0)
            parts.append((t1 - t0, t2 - t1, t3 - t2, t4 - t3))
        return {"value": trip / float(np.mean(e2e_s)), "unit": "q-triplets/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "includes": "context creation, generate, off-diagonal kappa, kappa solve",
                "ms": {k: 1e3 * float(np.median([p[i] for p in parts]))
                       for i, k in enumerate(("create", "generate", "kappa", "destroy"))}}

    def e2e_files_run(o, steps):
        # from the input files: readers, symmetry and mesh on the host, the harmonic stage on
        # the device (tdg_problem_load_device), then the scattering pass and kappa
        from tdep_gb300 import Problem

        e2e_s, parts = [], []
        h2d = d2h = 0
        for _ in range(steps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            p2 = Problem.load(INPUT_DIRS[cfg_name], cfg["grid"], readiso=True, device=0)
            t1 = time.perf_counter()
            s2 = ScatteringRates(p2)
            s2.generate(o, lists)
            s2.kappa_offdiag(o)
            s2.kappa(o)
            h2d, d2h = s2.transfer_bytes()
            s2.close()
            torch.cuda.synchronize()
            t2 = time.perf_counter()
            e2e_s.append(t2 - t0)
            parts.append((t1 - t0, t2 - t1))
        return {"value": trip / float(np.mean(e2e_s)), "unit": "q-triplets/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h),
                "includes": "infile.* read, symmetry and mesh (host), harmonic stage (device), context creation, "
                            "generate, off-diagonal kappa, kappa solve",
                "ms": {k: 1e3 * float(np.median([p[i] for p in parts])) for i, k in enumerate(("load", "rest"))}}

    e2e = e2e_run(opts, args.steps)
    e2e_files = e2e_files_run(opts, max(2, args.steps // 2)) if small else None
    if fp64 is not None:
        fp64["e2e"] = e2e_run(o64, max(2, args.steps // 2))

    # ---- roofline of the dominant kernel (fused pretransform + contraction + epilogue) ----
    # Per-unit work of a q-triplet: the pretransform streams N_t force-constant triplets
    # (27 values + 6 lattice indices, 4 bytes each in mixed precision) and writes n^3
    # complex values (8 bytes); the contraction is 24 n^4 flops. For n <= 6 the kernel is
    # reported against HBM with the pretransform bytes, for larger n against the tensor
    # peak with the contraction flops.
    hbm, bf16, src = peaks()
    fused_s = float(np.mean(fused_ms)) / 1e3
    bytes_per_trip = prob.n_fc3 * 33 * 4 + n**3 * 8
    flop_per_trip = 24 * n**4
    gbs = bytes_per_trip * trip / fused_s / 1e9
    tfs = flop_per_trip * trip / fused_s / 1e12
    traffic = TRAFFIC_PER_LAUNCH.get((cfg_name, path))
    if n <= 6:
        roof = {"bound": "hbm", "achieved": gbs, "peak": hbm, "unit": "GB/s", "frac": gbs / hbm,
                "traffic": traffic, "per_unit": f"{bytes_per_trip} bytes per q-triplet (N_t*33*4 + n^3*8)",
                "units_per_launch": trip, "peak_source": f"{src} copy bandwidth",
                "tensor_frac_of_contraction": tfs / bf16}
    else:
        roof = {"bound": "tensor", "achieved": tfs, "peak": bf16, "unit": "TFLOP/s", "frac": tfs / bf16,
                "traffic": traffic, "per_unit": f"{flop_per_trip} flop per q-triplet (24 n^4)",
                "units_per_launch": trip, "peak_source": f"{src} dense bf16",
                "hbm_frac_of_pretransform": gbs / hbm}
    roof["kernel"] = KERNEL_NAMES[path]

    # ---- CPU baseline sample and parity of its rows against the GPU runs ----
    if small:
        cpu_trip, cpu_s, desc, cores, kept = cpu_sample(prob, opts, lists, budget_s=cpu_budget, keep=True)
        idx, lw_ref, xi_ref = oracle_rows_finish(prob, o64, lists, kept)
        runs = {"fp64": (lw64, xi64[idx]), "mixed": (lw_mixed, xi_mixed[idx])}
        parity = parity_record(prob, lists, idx, lw_ref, xi_ref, runs)
    else:
        cpu_trip, cpu_s, desc, cores, kept = cpu_sample_large(prob, opts, lists)
        sample, q1, rows = large_sample_lists(prob, lists)
        s3 = ScatteringRates(prob)
        lw_gpu = s3.generate(opts, sample)
        s3.close()
        r0, r1, gamma, _ = kept[0]
        b1 = lists.row_b1[r0:r1] - 1
        f = prob.irr_full[q1 - 1] - 1
        nondeg = prob.degen[f, b1] == 1  # linewidths without degeneracy averaging equal gamma
        ref = gamma[nondeg]
        got = lw_gpu[q1 - 1, b1[nondeg]]
        mask = np.abs(ref) > 1e-12 * np.abs(ref).max()
        parity = {"rows": int(nondeg.sum()), "q1_groups": 1, "what": "one q-triplet per row, rows of one q1 "
                  "without degenerate partners: tensor-core mixed path against the FP64 oracle",
                  "lw_max_rel_mixed": float(np.max(np.abs(got[mask] - ref[mask]) / np.abs(ref[mask])))}
    value = trip * args.steps / (sum(dev_ms) / 1e3)
    return {
        "cfg": cfg, "n": n, "small": small, "value": value, "ms_per_step": float(np.mean(dev_ms)),
        "trip": trip, "xi_gb": lists.n_row * prob.n_full * n * 8 / 1e9, "e2e": e2e, "e2e_files": e2e_files,
        "adjoint": adjoint,
        "roofline": roof, "clocks": clk, "launches": launches, "graphs": graphs, "stats": stats,
        "kappa_ms": kappa_ms, "kappa_iters": kappa_iters, "fp64": fp64, "lw_max": float(lw_mixed.max()),
        "cpu": {"value": cpu_trip / cpu_s, "unit": "q-triplets/s", "cores": cores, "kind": "port", "sample": desc},
        "parity": parity, "tune": autotune_table(), "path": path, "shape": shape,
    }


def run_gb300(args):
    import torch

    torch.cuda.init()
    m = measure(args.config, args, args.cpu_budget)
    n, small = m["n"], m["small"]
    cfg = m["cfg"]
    line = {
        "metric": METRIC, "value": m["value"], "unit": "q-triplets/s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": m["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": cfg["workload"], "mesh": list(cfg["grid"]), "n_mode": n, "q_triplets_per_step": m["trip"],
                   "precision": PRECISION_NOTES[m["path"]],
                   "l2": "256 MB buffer written between steps (L2 flush); Xi+od working set 2x%.2f GB" % m["xi_gb"]},
        # end to end from the input files (readers, symmetry and mesh on the host, the harmonic
        # stage on the device, then the scattering pass and kappa); the figure with the problem
        # already built follows it
        "e2e": m["e2e_files"] or m["e2e"],
        "e2e_problem_resident": m["e2e"],
        "adjoint": m["adjoint"],
        "roofline": m["roofline"],
        "cpu_baseline": m["cpu"],
        "parity": m["parity"],
        "clocks": m["clocks"],
        "gpu_launches": int(m["launches"]),
        "launch_shapes": {"autotuned": m["tune"], "fused_kernel": m["shape"],
                          "graph_counts_direct_recorded_replayed": m["graphs"],
                          "note": "warm-up calls run the autotuner trials and record the CUDA graph of the "
                                  "three-phonon kernels; timed calls replay it"},
        "stage_ms": {k: m["stats"][k] for k in ("enumerate_ms", "threephonon_ms", "symmetrize_ms", "device_ms")},
        "mode_triplets_per_s": m["value"] * n**3,
        "kappa_wall_ms": m["kappa_ms"], "kappa_iterations": m["kappa_iters"],
        "fp64": m["fp64"] if small else {"value": None, "reason": "beyond 18 modes the contraction runs only on the "
                                                                   "tensor cores (mixed precision)"},
        "linewidth_max_hartree": m["lw_max"],
    }
    if "uneven" in cfg and args.config == "perovskite16":
        line["three_plus_four_phonon"] = fourphonon_leg(args.config, max(2, args.steps // 2))
    if args.config == "perovskite16" and not args.no_sub:
        # the 2-atom rocksalt 24^3 configuration (6 modes, full q' grid) measured in the same run
        r = measure("rocksalt24", args, min(6.0, args.cpu_budget), with_adjoint=True)
        line["rocksalt24"] = {
            "workload": r["cfg"]["workload"], "value": r["value"], "unit": "q-triplets/s",
            "ms_per_step": r["ms_per_step"], "q_triplets_per_step": r["trip"], "e2e": r["e2e_files"] or r["e2e"],
            "e2e_problem_resident": r["e2e"], "fp64": r["fp64"],
            "adjoint": r["adjoint"], "roofline": r["roofline"], "cpu_baseline": r["cpu"], "parity": r["parity"],
            "clocks": r["clocks"], "gpu_launches": int(r["launches"]), "kappa_wall_ms": r["kappa_ms"]}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--config", default="perovskite16", choices=sorted(CONFIGS))
    ap.add_argument("--no-sub", action="store_true", help="skip the rocksalt 24^3 sub-record of the default run")
    ap.add_argument("--cpu-budget", type=float, default=12.0)
    ap.add_argument("--profile", action="store_true", help="only run passes of one stage, see --stage (for ncu captures)")
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"], help="with --profile")
    ap.add_argument("--stage", default="scattering", choices=["scattering", "kappa", "offdiag", "adjoint", "fourphonon"],
                    help="with --profile")
    args = ap.parse_args()
    if args.profile:
        run_profile(args)
        return
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.impl == "reference":
        if rank == 0:
            run_reference(args)
        return
    if world > 1:
        # The path does not shard across GPUs in this build: replicas only. Rank 0 reports.
        local = int(os.environ.get("LOCAL_RANK", "0"))
        os.environ["CUDA_VISIBLE_DEVICES"] = str(local)
        if rank != 0:
            return
    run_gb300(args)


if __name__ == "__main__":
    main()
