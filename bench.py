#!/usr/bin/env python3
"""Benchmark: chunks/s of one Newton-Raphson iteration of lyspeq's per-chunk
QMLE on one GB300, mixed precision vs FP64, with the CPU baseline beside it.

Workload (the DESI-like configuration): 4096 synthetic chunks, N_pix
log-uniform in [200, 1200], dv = 50 km/s, R uniform in [2000, 5000], 35 k bins,
13 triangular z bins, S/N per pixel lognormal(ln 1, 0.8), continuum
marginalisation of amplitude + slope.  Inputs are seeded synthetic data of
those shapes (lyspeq_gb300.synth); the per-iteration working set (tens of GB
of operand planes) is far larger than L2, so no L2 flush is needed.

`--workload desi_reso` runs the resolution-matrix configuration instead:
16384 chunks, N log-uniform in [150, 1000], 11-diagonal resolution matrices
deconvolved and oversampled x 3 (S and Q_k built as R M R^T), 20 k x 3 z
bins; the matrices are prepared on the host before timing, as lyspeq does
while reading its files.

A step is one Newton-Raphson iteration: lqg_nr_iteration over the whole
batch (table interpolation -> C -> df64 Cholesky and inverse factor -> the
Q_k products on tensor cores -> traces) plus the global Fisher inversion and
theta update.  Steps alternate between the two kinds an NR run is made of:
the first iteration (theta = 0) and a later one (theta from the previous
solve, which adds sum theta_k Q_k to C).  `value` times steps with the chunks
resident on the device; `e2e` times the same through the C ABI from host
buffers (chunk upload, iteration, result download, solve), and reports the
host time of each step's batch add (Chunk::Chunk and the pixel arrays) as
`batch_add_ms`.

Beside it: the FP64 GPU path on a subset stratified by chunk size (both kinds
of iteration) with the mixed path's errors against it, a DFMA probe for the
FP64 roofline, and the CPU restatement of the reference on a fixed sample of
64 chunks stratified by size (16 quantile groups x 4), the same sample the
`--impl reference` arm times, with its relative standard error.
The default precision, mixed_auto, runs the autotuner before the timed
region (its time is reported) and then iterates with the chosen plan per
chunk size; `--precision mixed` uses the fixed whitened plan.  `--fp64-full`
runs the FP64 comparison over every chunk (one iteration, minutes).

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
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

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

METRIC = "chunks/s per NR iteration (mixed precision, one GB300)"
UNIT = "chunks/s"
PEAKS_FILE = os.path.join(HERE, "MEASURED_PEAKS.json")


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.idx = device_index
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-i", str(self.idx), "-lms", "200"], stdout=subprocess.PIPE,
                stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in self.rows if len(r) > 2 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) > 2 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            for k, nm in enumerate(names):
                if len(r) > 5 + k and r[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(self.rows)}


def chunk_arrays(w, lib=None):
    """Chunks as lqg_batch_add takes them: lambda (A), delta, ivar, R.  For a
    resolution-matrix workload the last item is the spectrum's matrix after
    deconvolution and oversampling: through the library's host routines when
    lib is given, else None (the CPU legs prepare it with the oracle)."""
    out = []
    for s in w.spectra:
        ivar = 1.0 / np.asarray(s.sigma) ** 2
        if not w.reso:
            out.append((s.wave, s.delta, ivar, s.r_fwhm))
            continue
        rows = None
        if lib is not None:
            v = lib.resomat_deconvolve(s.resomat, w.deconv_m) if w.deconv_m > 0 else s.resomat
            rows = lib.resomat_oversample(v, w.oversample, float(np.median(np.diff(s.wave)))) \
                if w.oversample > 0 else np.ascontiguousarray(v.T)
        out.append((s.wave, s.delta, ivar, rows))
    return out


def pack(chunks, reso=False):
    offs = np.zeros(len(chunks) + 1, dtype=np.int64)
    for i, c in enumerate(chunks):
        offs[i + 1] = offs[i] + len(c[0])
    cat = lambda j: np.ascontiguousarray(np.concatenate([np.asarray(c[j], np.float64) for c in chunks]))
    last = cat(3).reshape(int(offs[-1]), -1) if reso else np.array([c[3] for c in chunks], dtype=np.int32)
    return cat(0), cat(1), cat(2), offs, last


def add_packed(eng, w, packed):
    lam, delta, ivar, offs, last = packed
    if w.reso:
        return eng.add_chunks_reso(lam, delta, ivar, offs, w.oversample, last)
    return eng.add_chunks(lam, delta, ivar, offs, last)


def describe(w, n_ok):
    if w.name == "echelle":
        return (f"echelle: {n_ok} chunks, N uniform-int 1000-4000, dv 2.5-5 km/s, R 30000-50000, "
                "40 k x 6 z bins, no marginalisation")
    if w.reso:
        return (f"{w.name}: {n_ok} chunks, N log-uniform 150-1000, dv 50 km/s, 11-diagonal resolution "
                f"matrices deconvolved and oversampled x{w.oversample}, 20 k x 3 z bins, no marginalisation")
    return (f"{w.name}: {n_ok} chunks, N log-uniform 200-1200, dv 50 km/s, R 2000-5000, 35 k x 13 z bins, "
            "amplitude+slope marginalisation")


def flop_counts(ns_list, n_list):
    """Algorithmic FLOPs of the per-chunk work (the same for every precision):
    factorisation n^3 (Cholesky + triangular inverse + C^-1 assembly, n^3/3
    each), products 2 (ns + 1) n^3, traces 2 (ns + 2) ns n^2."""
    n = np.asarray(n_list, dtype=np.float64)
    ns = np.asarray(ns_list, dtype=np.float64)
    return dict(factor=float(np.sum(n ** 3)), products=float(np.sum(2 * (ns + 1) * n ** 3)),
                traces=float(np.sum(2 * (ns + 2) * ns * n ** 2)))


def stratified_sample(n_list, strata=16, per=4, seed=12345):
    """A fixed sample of the workload's chunks for the CPU legs: the chunks
    sorted by size N, cut into `strata` equal quantile groups, `per` chunks
    drawn from each (seeded); ordered round by round, so that every run of
    `strata` consecutive entries holds one chunk of each group.  The cost of a
    chunk grows like N^3, so a sample that follows the N distribution keeps the
    rate estimate unbiased and its error small."""
    order = np.argsort(np.asarray(n_list), kind="stable")
    groups = np.array_split(order, strata)
    rng = np.random.Generator(np.random.PCG64(seed))
    picks = [rng.choice(g, size=min(per, len(g)), replace=False) for g in groups]
    return [int(picks[h][r]) for r in range(per) for h in range(strata) if r < len(picks[h])]


def cpu_port_times(w, chunks, indices):
    """Seconds per chunk of the CPU restatement of lyspeq's per-chunk path
    (numpy + scipy's OpenBLAS, all host threads) for the given chunks.
    Resolution matrices are prepared by the restatement's own reader steps,
    outside the timed work (the reference does it while reading files)."""
    from oracle import qmle_port as P
    s = P.Settings(max_forest_length=w.max_forest_length, cont_logl_order=w.cont_logl_order,
                   cont_l_order=w.cont_l_order)
    keys = w.table_index()
    tvs = {}
    times = []
    for i in indices:
        lam, delta, ivar, r = chunks[i]
        reso = rm = None
        if w.reso:
            reso = (w.oversample, w.deconv_m)
            v = P.dia_deconvolve(np.array(w.spectra[i].resomat), w.deconv_m) if w.deconv_m > 0 \
                else np.array(w.spectra[i].resomat)
            rm = P.dia_oversample(v, w.oversample, P._median(np.diff(lam))) if w.oversample > 0 else v
        t0 = time.perf_counter()
        try:
            ch = P.make_chunk(lam, delta, ivar, 0 if w.reso else r, w.bins, keys, s, reso, rm)
        except (ValueError, KeyError):
            continue
        if ch.res_index not in tvs:
            tvs[ch.res_index] = P.table_view(w.tables[ch.res_index], w.bins, w.nv, w.lenv, w.nzp)
        P.chunk_iteration(ch, w.bins, tvs[ch.res_index], np.zeros(w.bins.nkz), s)
        times.append(time.perf_counter() - t0)
    return np.asarray(times)


def stratified_rate(times, strata):
    """chunks/s of a round-ordered stratified sample and the relative standard
    error of that rate (within-group variance of the per-chunk times)."""
    t = np.asarray(times)
    groups = [t[h::strata] for h in range(strata) if len(t[h::strata])]
    mean = float(np.mean([g.mean() for g in groups]))
    var = sum((g.var(ddof=1) / len(g) if len(g) > 1 else 0.0) for g in groups) / len(groups) ** 2
    return 1.0 / mean, float(np.sqrt(var) / mean)


def cpu_sample_desc(w, strata, per):
    return (f"{strata * per} chunks of the {w.name} workload stratified by N ({strata} quantile groups "
            f"x {per}, seed 12345), numpy + scipy OpenBLAS on all host threads")


def run_reference(args, rank, world):
    """The reference arm: lyspeq's per-chunk path on the host cores (the numpy
    restatement; the compiled reference does not exist on the GPU machine).  Each
    timed step is one round of the stratified sample (one chunk of every size
    group); warm-up steps run two chunks."""
    if rank != 0:
        return 0
    from lyspeq_gb300 import synth
    w = synth.make_workload(args.workload)
    chunks = chunk_arrays(w)
    strata, per = args.cpu_strata, args.cpu_per
    sample = stratified_sample([len(c[0]) for c in chunks], strata, per)
    for step in range(args.warmup):
        cpu_port_times(w, chunks, sample[:2])
    times, steps = [], []
    for step in range(args.steps):
        r = step % per
        t = cpu_port_times(w, chunks, sample[r * strata:(r + 1) * strata])
        times.extend(t.tolist())
        steps.append(float(t.sum()))
    value = len(times) / float(np.sum(times))
    # step-to-step spread of the round means, as a relative standard error
    rates = np.asarray([strata / x for x in steps])
    rel_se = float(np.std(rates, ddof=1) / np.sqrt(len(rates)) / value) if len(rates) > 1 else None
    cores = os.cpu_count()
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": float(np.mean(steps) * 1e3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded, DESI-like shapes)",
        "config": {"workload": describe(w, len(w.spectra)),
                   "sample": f"step k: round k mod {per} of the stratified sample ({strata} chunks, one per N group)"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": cpu_sample_desc(w, strata, per), "rel_stderr": rel_se},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def p1d_errors(w, g_ref, g_mix, fsum):
    """Mixed against FP64: P1D relative error on the bins measured at 5 sigma
    or more (the others are noise), and the largest |dP| in sigma."""
    from lyspeq_gb300 import synth
    pfid = synth.pd13_power(np.tile(w.bins.k_centers, w.bins.nz), np.repeat(w.bins.z_centers, w.bins.nk))
    p_ref, p_mix = pfid + g_ref["theta"], pfid + g_mix["theta"]
    sig = np.sqrt(np.abs(np.diag(g_ref["inverse"])))
    used = (np.diag(fsum) > 0) & (sig > 0)
    good = used & (np.abs(p_ref) > 5 * sig)
    rel = float(np.max(np.abs(p_mix - p_ref)[good] / np.abs(p_ref)[good])) if good.any() else None
    insig = float(np.max(np.abs(p_mix - p_ref)[used] / sig[used])) if used.any() else None
    return rel, int(good.sum()), insig


def mixed_vs_fp64(w, e64, theta, precision="mixed"):
    """One FP64 and one mixed iteration of the engine at theta: the FP64 device
    time and the mixed errors (global F per element normalised by
    sqrt(F_ii F_jj), d, b, t normwise, d - b - t normwise on max |b|, P1D)."""
    e64.iterate(theta=theta, precision="fp64")
    fp64_ms = e64.timings()[7]
    ref = e64.download()
    g_ref = e64.fisher_solve(ref["fisher"], np.stack([ref["d"], ref["b"], ref["t"]]))
    e64.iterate(theta=theta, precision=precision)
    mix = e64.download()
    g_mix = e64.fisher_solve(mix["fisher"], np.stack([mix["d"], mix["b"], mix["t"]]))
    dg = np.sqrt(np.abs(np.diag(g_ref["fisher"])))
    den = np.outer(dg, dg)
    den[den == 0] = 1
    err_f = float(np.max(np.abs(g_mix["fisher"] - g_ref["fisher"]) / den))
    dbt_ref = np.stack([ref["d"], ref["b"], ref["t"]])
    dbt_mix = np.stack([mix["d"], mix["b"], mix["t"]])
    err_dbt = float(np.max(np.abs(dbt_mix - dbt_ref) / np.max(np.abs(dbt_ref), axis=1, keepdims=True)))
    e_ref, e_mix = dbt_ref[0] - dbt_ref[1] - dbt_ref[2], dbt_mix[0] - dbt_mix[1] - dbt_mix[2]
    err_e = float(np.max(np.abs(e_mix - e_ref)) / np.max(np.abs(dbt_ref[1])))
    p1d, nbins, insig = p1d_errors(w, g_ref, g_mix, ref["fisher"])
    return fp64_ms, {"fisher": err_f, "dbt": err_dbt, "d_minus_b_minus_t": err_e, "p1d": p1d,
                     "p1d_bins": nbins, "p1d_in_sigma": insig}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=4)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="desi")
    ap.add_argument("--chunks", type=int, default=None)
    ap.add_argument("--precision", default="mixed_auto", choices=["mixed", "mixed_direct", "mixed_auto"])
    ap.add_argument("--fp64-chunks", type=int, default=128,
                    help="chunks of the FP64 GPU comparison (a stratified subset); 0: all")
    ap.add_argument("--fp64-full", action="store_true",
                    help="FP64 GPU path over every chunk instead: one theta = 0 iteration, no warm-up")
    ap.add_argument("--cpu-strata", type=int, default=16)
    ap.add_argument("--cpu-per", type=int, default=4)
    ap.add_argument("--no-cpu", action="store_true")
    args = ap.parse_args()
    rank, world, local = dist_env()

    if args.impl == "reference":
        return run_reference(args, rank, world)

    import torch
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    from lyspeq_gb300 import build, lqg, synth
    build.build()
    seed = None if world == 1 else 20240602 + 7919 * rank
    w = synth.make_workload(args.workload, seed=seed, n_chunks=args.chunks)
    chunks = chunk_arrays(w, lqg)
    lam, delta, ivar, offs, rr = pack(chunks, w.reso)
    pinned = tuple(torch.from_numpy(x).pin_memory().numpy() for x in (lam, delta, ivar))
    if w.reso:
        rr = torch.from_numpy(rr).pin_memory().numpy()
    packed = pinned + (offs, rr)
    eng = lqg.Engine(w.bins, w.tables, w.nv, w.lenv, w.nzp, w.max_forest_length,
                     cont=(w.cont_logl_order, w.cont_l_order), device=local)
    st = add_packed(eng, w, packed)
    n_ok = int((st == 0).sum())
    infos = [eng.chunk_info(i) for i in range(eng.size)]
    ns_list = [(i["nq"] // w.bins.nk) * i["kbin_upp"] for i in infos]
    n_list = [i["n"] for i in infos]
    nkz = w.bins.nkz
    tune_s = None
    if args.precision == "mixed_auto":
        t0 = time.perf_counter()
        eng.autotune()
        tune_s = time.perf_counter() - t0

    def allreduce(out):
        if world == 1:
            return out
        from lyspeq_gb300.distributed import allreduce_sums
        f, d, b, t = allreduce_sums(out["fisher"], out["d"], out["b"], out["t"], device=f"cuda:{local}")
        return dict(fisher=f, d=d, b=b, t=t, status=out["status"])

    def nr_step(theta):
        eng.iterate(theta=theta, precision=args.precision)
        out = allreduce(eng.download())
        return eng.fisher_solve(out["fisher"], np.stack([out["d"], out["b"], out["t"]]))

    # A step is one Newton-Raphson iteration.  An NR run is one iteration at
    # theta = 0 and then iterations at the theta of the previous solve; the
    # steps alternate between the two (theta_1 from a first iteration before
    # the warm-up), so that both kinds are timed.  Each kind replays its own
    # captured graph after its second occurrence.
    theta1 = nr_step(None)["theta"]
    thetas = [theta1, None]

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()
        torch.cuda.synchronize()

    for k in range(args.warmup):
        nr_step(thetas[k % 2])
    phase = np.zeros(8)
    kind_ms = {0: [], 1: []}
    launches = 0
    waves = 1
    barrier()
    with ClockSampler(local) as clk:
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for k in range(args.steps):
            th = thetas[(args.warmup + k) % 2]
            nr_step(th)
            tm = eng.timings()
            phase += tm
            kind_ms[0 if th is None else 1].append(float(tm[7]))
            launches += eng.launch_count()
            waves = eng.wave_count()
        e1.record()
        barrier()
    ms = e0.elapsed_time(e1) / args.steps
    if world > 1:
        import torch.distributed as dist
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    value = n_ok * world / (ms / 1e3)
    phase /= args.steps

    # end to end through the C ABI from pinned host buffers: upload, iteration,
    # download of the sums, Fisher solve
    barrier()
    e2 = torch.cuda.Event(enable_timing=True)
    e3 = torch.cuda.Event(enable_timing=True)
    e2.record()
    add_s = 0.0
    h2d_sum = 0
    for k in range(args.steps):
        t_add = time.perf_counter()
        eng.clear()
        add_packed(eng, w, packed)
        add_s += time.perf_counter() - t_add      # host: Chunk::Chunk and the pixel arrays
        nr_step(thetas[(args.warmup + k) % 2])
        h2d_sum += eng.h2d_bytes()                # what the library copied for this step
    e3.record()
    barrier()
    ms_e2e = e2.elapsed_time(e3) / args.steps
    e2e_value = n_ok * world / (ms_e2e / 1e3)
    # the host Fisher solve of a step on its own (part of every timed step)
    out = allreduce(eng.download())
    dbt = np.stack([out["d"], out["b"], out["t"]])
    t0 = time.perf_counter()
    for _ in range(5):
        eng.fisher_solve(out["fisher"], dbt)
    solve_ms = (time.perf_counter() - t0) / 5 * 1e3
    # bytes copied per e2e step: host to device as the library counts them (the
    # batch's derived pixel arrays and metadata, theta, the launch plan), device
    # to host the sums and the chunk statuses the download reads
    h2d = int(round(h2d_sum / max(args.steps, 1)))
    input_bytes = int(lam.nbytes + delta.nbytes + ivar.nbytes + 8 * nkz + (rr.nbytes if w.reso else 0))
    d2h = int(8 * (nkz * nkz + 3 * nkz) + 4 * eng.size)

    if rank != 0:
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()
        return 0

    # FP64 GPU path on a stratified subset (or all chunks), and the accuracy of
    # the mixed path against it at theta = 0 and at theta_1
    if args.fp64_chunks and args.fp64_chunks < len(chunks) and not args.fp64_full:
        per = max(1, args.fp64_chunks // 16)
        sub_idx = stratified_sample([len(c[0]) for c in chunks], 16, per, seed=777)
    else:
        sub_idx = list(range(len(chunks)))
    sub = [chunks[i] for i in sub_idx]
    e64 = lqg.Engine(w.bins, w.tables, w.nv, w.lenv, w.nzp, w.max_forest_length,
                     cont=(w.cont_logl_order, w.cont_l_order), device=local)
    if w.reso:
        e64.add_chunks_reso(*pack(sub, True)[:4], w.oversample, pack(sub, True)[4])
    else:
        e64.add_chunk_list(sub)
    if args.precision == "mixed_auto":
        e64.set_tuning(eng.tuning())
    if args.fp64_full:
        # every chunk once at theta = 0 (an FP64 iteration of the whole set takes
        # minutes; its first-iteration planning is a negligible part of it)
        fp64_ms, err0 = mixed_vs_fp64(w, e64, None, args.precision)
        fp64_ms1, err1 = None, None
        fp64_rate = len(sub) / (fp64_ms / 1e3)
    else:
        e64.iterate(precision="fp64")   # warm-up
        fp64_ms, err0 = mixed_vs_fp64(w, e64, None, args.precision)
        fp64_ms1, err1 = mixed_vs_fp64(w, e64, theta1, args.precision)
        # the same alternation as the timed steps: the mean of the two kinds
        fp64_rate = len(sub) / ((fp64_ms + fp64_ms1) / 2e3)
    e64.close()
    fp64_peak = lqg.probe_fp64_rate(local)

    # roofline of the dominant phase
    fl = flop_counts(ns_list, n_list)
    names = ["build_s_c", "factor", "build_q", "products_tc", "traces_tc", "finish", "accumulate"]
    shares = {nm: float(phase[i] / phase[7]) for i, nm in enumerate(names)}
    dom = max(range(7), key=lambda i: phase[i])
    peaks = {}
    if os.path.exists(PEAKS_FILE):
        peaks = json.load(open(PEAKS_FILE))
    if names[dom] == "build_q" and w.reso:
        # the resolution-matrix Q build, FP32 pipe: algorithmic flops of R M R^T
        # per stored band, half of the symmetric product (nelem n (nf + n))
        ne = 2 * (w.spectra[0].resomat.shape[0] // 2) * max(w.oversample, 1) + 1
        osm = max(w.oversample, 1)
        n_a = np.asarray(n_list, dtype=np.float64)
        kup = np.asarray([i["kbin_upp"] for i in infos], dtype=np.float64)
        flops = float(np.sum(kup * 2.0 * ne * n_a * (n_a * osm + ne - 1 + n_a) / 2.0))
        achieved = flops / (phase[2] / 1e3) / 1e12
        props = torch.cuda.get_device_properties(local)
        mhz = clk.summary().get("sm_max_mhz") or 2070.0
        pk = props.multi_processor_count * 128 * 2 * mhz * 1e6 / 1e12
        roof = {"kernel": "k_build_q_reso_f32", "bound": "fp32", "achieved": achieved, "peak": pk,
                "unit": "TFLOP/s", "frac": achieved / pk, "traffic": None,
                "peak_source": "nominal FP32 FMA rate at the sampled maximum SM clock "
                               "(MEASURED_PEAKS.json has no FP32 figure)"}
    elif names[dom] == "factor":
        achieved = fl["factor"] / (phase[1] / 1e3) / 1e12
        roof = {"kernel": "k_factor_tiled", "bound": "fp64", "achieved": achieved, "peak": fp64_peak,
                "unit": "TFLOP/s", "frac": achieved / fp64_peak, "traffic": None,
                "peak_source": "DFMA probe (lqg_probe_fp64_rate) run by this bench"}
    else:
        key = "products" if names[dom] == "products_tc" else "traces"
        achieved = fl[key] / (phase[dom] / 1e3) / 1e12
        pk = peaks.get("bf16_tflops_sustained", 1700.0)
        # DRAM traffic per launch of the first product kernel, X_s = W Q_s (one
        # launch per wave, the larger of the two product stages): its
        # algorithmic bytes (Q_s read and X_s written as fp16 hi/lo, ns + 1
        # slots) times 0.99, the measured/algorithmic ratio of an ncu capture
        # of the same kernel on 64 chunks of this workload
        traffic = None
        if key == "products" and waves > 0:
            ld = np.ceil(np.asarray(n_list) / 64.0) * 64.0
            alg = float(np.sum(2.0 * (np.asarray(ns_list) + 1) * ld * ld * 4.0))
            traffic = 0.99 * alg / waves
        roof = {"kernel": "k_tc_gemm<1> + k_tc_gemm<2> (phase); traffic of k_tc_gemm<1>" if key == "products"
                else "k_tc_gram", "bound": "tensor",
                "achieved": achieved, "peak": pk, "unit": "TFLOP/s", "frac": achieved / pk,
                "traffic": traffic, "traffic_unit": "bytes per launch",
                "peak_source": "MEASURED_PEAKS.json bf16_tflops_sustained (the kernel runs inside a "
                               "seconds-long step), of measured"}
    tensor_tf = fl["products"] / (phase[3] / 1e3) / 1e12 if phase[3] > 0 else None
    df64_tf = fl["factor"] / (phase[1] / 1e3) / 1e12 if phase[1] > 0 else None

    cpu = None
    if not args.no_cpu:
        sample = stratified_sample([len(c[0]) for c in chunks], args.cpu_strata, args.cpu_per)
        times = cpu_port_times(w, chunks, sample)
        rate, rel_se = stratified_rate(times, args.cpu_strata)
        cpu = {"value": rate, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
               "sample": cpu_sample_desc(w, args.cpu_strata, args.cpu_per) + f", {float(np.sum(times)):.1f} s",
               "rel_stderr": rel_se}

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f16x3 products / df64 factorisation", "data": "synthetic (seeded)",
        "config": {"workload": describe(w, n_ok), "precision": args.precision,
                   "step": "one NR iteration; steps alternate theta = 0 and theta from the previous solve",
                   "l2": "working set of tens of GB per iteration (>> 129 MB L2); no flush"},
        "gpu_launches": int(launches),
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "ms_per_step": ms_e2e, "batch_add_ms": add_s * 1e3 / args.steps,
                "input_bytes_per_step": input_bytes},
        "roofline": roof,
        "cpu_baseline": cpu,
        "clocks": clk.summary(),
        "iteration_ms": {"theta_0": float(np.mean(kind_ms[0])) if kind_ms[0] else None,
                         "theta_1": float(np.mean(kind_ms[1])) if kind_ms[1] else None},
        "fp64_gpu": {"value": fp64_rate, "unit": UNIT, "chunks": len(sub), "ms_theta_0": fp64_ms,
                     "ms_theta_1": fp64_ms1,
                     "sample": "stratified by N" if len(sub) < len(chunks)
                     else ("all, one theta = 0 iteration" if args.fp64_full else "all")},
        "fp64_peak_tflops": fp64_peak,
        "mixed_over_fp64": value / fp64_rate if fp64_rate else None,
        "mixed_rel_err": {"theta_0": err0, "theta_1": err1},
        "phase_ms": {nm: float(phase[i]) for i, nm in enumerate(names)},
        "phase_share": shares,
        "fisher_solve_ms": solve_ms,
        "achieved_tflops": {"factor_df64": df64_tf, "tensor_products": tensor_tf},
    }
    if tune_s is not None:
        line["autotune_s"] = tune_s
        # the chosen plan per padded size: ld, whitened form, drain, Gram K per split, CTA pairs
        line["tuning"] = eng.tuning().tolist()
    print(json.dumps(line))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    eng.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
