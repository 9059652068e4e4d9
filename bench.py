#!/usr/bin/env python3
"""Benchmark of the GB300 Cooper-Frye sampler.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Workload (N = 1): the viscous 3+1D surface -- 200,000 cells on 64 eta slices,
20 % spacelike cells, shear with |pi|/(e+P) up to 0.3, 14-moment bulk delta f
-- with the s95p-v1 species list (319 species) and 1,000 oversampled events
per GPU.  One step = one full generate: local-rest-frame prologue, yields
for every (cell, species), per-species CDFs, Poisson counts, momentum
sampling and the hadron records, with the surface resident in HBM.  Inputs
are synthetic (iss_gb300.surfaces, seed 2).  Intermediate buffers (yields
256 MB, CDF 510 MB, hadrons ~0.8 GB) exceed L2 and a 256 MB buffer is
written between steps.

The launch shape comes from the library's autotuner (untimed, before the
warm-up) and each generate of the device leg replays one captured CUDA graph
(gpu_graph = 1); --no-autotune / --no-graph turn these off.

`value` is device time (CUDA events on the library's stream); `e2e` is the
same metric through the C ABI with the surface copied from pinned host
memory and all hadrons read back to pinned host memory every step
(iss_gpu_set_surface + iss_gpu_generate_into, whose device->host copies of
finished events overlap the sampling of later ones).  By default the e2e
steps run on two handles from two host threads, so that one step's device
work overlaps the other's record copy, and on one handle; both legs go
through the C ABI, the headline is the faster (on some hosts the page-locked
buffers of two handles copy slower), e2e.legs has both and
e2e.single_handle the one-handle leg (--e2e-handles 1: one leg only).

--impl reference times the CPU implementation of the path (the oracle port
of the reference's algorithm, oracle/) on the host cores with one process per
core, each sampling a disjoint share of the events on a 10 % cell sample.

The default line also carries the metric's second arm, `learned`: the
proposal network is trained on the same surface (5e7 momenta of the plain
sampler from seeds 10..19, Adam on the tensor cores, untimed), then W + K
generates with the learned proposal (gpu_sampler = 1, alpha = 0.8, exact
rejection) are timed like the plain steps.  It reports the learned
hadrons/s and its ratio to the plain arm, proposals per hadron (with and
without the network, and with the pilot envelope alone), the excess
branch's share, violations (none by construction), the network's
tensor-core throughput, and two-sample chi-square / KS p-values of pT, y,
phi and v2 of the learned species against the plain sampler on 1,000
events.  --no-learned skips it; --sampler learned makes the learned arm
the headline `value`.
"""
from __future__ import annotations

import argparse
import gc
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

METRIC = ("sampled hadrons/s on 1 GB300, learned vs plain sampler at matched spectra "
          "(χ²/KS)")
UNIT = "hadrons/s"
N_CELLS = 200_000
N_EVENTS = 1000
SEED_SURFACE = 2
PARAMS = dict(hydro_mode=2, afterburner_type=0, include_deltaf_shear=1, include_deltaf_bulk=1,
              bulk_deltaf_kind=11, turn_on_bulk=1, quantum_statistics=1,
              dN_dy_sampling_model=30, number_of_repeated_sampling=N_EVENTS)
ALG_BYTES_PER_HADRON = 40 + 96 + 4     # record write + LRF cell gather + slot/index
# network forward per (species, cell) pair: 2 x (18 x 128 + 3 x 128 x 128 + 128 x 48)
MLP_FLOPS_PER_PAIR = 2 * (18 * 128 + 3 * 128 * 128 + 128 * 48)

# the other configurations of the benchmark set, for --workload (the default
# line is always the viscous one above)
WORKLOADS = {
    "viscous": dict(cells=N_CELLS, events=N_EVENTS, species=319, params=PARAMS,
                    data="synthetic (iss_gb300.surfaces.viscous_3d, seed 2)"),
    # ideal fluid, boost-invariant, r < 10 fm on a 0.5 fm grid, T = 0.150 GeV
    "ideal": dict(cells=1245, events=100, species=319,
                  params=dict(hydro_mode=1, afterburner_type=0, include_deltaf_shear=0,
                              include_deltaf_bulk=0, quantum_statistics=1,
                              dN_dy_sampling_model=30),
                  data="synthetic (iss_gb300.surfaces.ideal_boost_invariant)"),
    # 256 independent viscous surfaces sampled by one generate: cells
    # log-uniform in [5k, 400k], events log-uniform in [10, 2000] (seeds 100..)
    "batched": dict(cells=None, events=None, species=319, params=PARAMS,
                    data="synthetic (iss_gb300.surfaces.viscous_3d, seeds 100.., sizes from seed 0)"),
    # finite baryon density with diffusion, SMASH species, 1M cells
    "finite_density": dict(cells=1_000_000, events=2000, species=400,
                           params=dict(hydro_mode=2, afterburner_type=2, include_deltaf_shear=1,
                                       include_deltaf_bulk=1, bulk_deltaf_kind=11,
                                       turn_on_bulk=1, include_deltaf_diffusion=1, turn_on_rhob=1,
                                       turn_on_diff=1, quantum_statistics=1,
                                       dN_dy_sampling_model=30),
                           data="synthetic (iss_gb300.surfaces.finite_density_3d, seed 3)"),
}


def batch_sizes(n_surfaces: int):
    rng = np.random.default_rng(0)
    cells = np.exp(rng.uniform(np.log(5e3), np.log(4e5), n_surfaces)).astype(np.int64)
    events = np.exp(rng.uniform(np.log(10), np.log(2000), n_surfaces)).astype(np.int32)
    return cells, events


def make_surface(workload: str, cells: int):
    from iss_gb300 import surfaces as S
    if workload == "ideal":
        return S.ideal_boost_invariant()
    if workload == "finite_density":
        return S.finite_density_3d(cells, seed=3)
    return S.viscous_3d(cells, seed=SEED_SURFACE)
L2_FLUSH_BYTES = 256 << 20


def peaks():
    try:
        with open(os.path.join(HERE, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


PROFILE = os.path.join("profiles", "sampler_kernel_viscous_3d.md")
SMS = 152               # GB300 streaming multiprocessors
SCHEDULERS_PER_SM = 4   # warp schedulers, one warp instruction per cycle each


def profiled(key):
    """A per-hadron figure of the sample phase from the committed ncu summary
    of the autotuned launch shape (PROFILE, line '<key>: value'): DRAM bytes
    (dram_bytes_per_hadron) or warp instructions (warp_instructions_per_hadron)
    of cell_assign_kernel + sampler_kernel per sampled hadron.  The bench
    cannot run ncu itself; these are constants from that capture."""
    try:
        for line in open(os.path.join(HERE, PROFILE)):
            if line.strip().startswith(key + ":"):
                return float(line.split(":")[1])
    except OSError:
        pass
    return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled every 20 ms from before
    the warm-up; stop() keeps the samples whose timestamps fall inside the
    timed region (mark_begin / mark_end)."""

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.file = None
        self.t0 = self.t1 = None

    def start(self):
        try:
            self.file = tempfile.NamedTemporaryFile(mode="w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}",
                 "--query-gpu=timestamp,clocks.sm,clocks.max.sm,power.draw,"
                 "clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
                 "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
                 "clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "20"],
                stdout=self.file, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def mark_begin(self):
        self.t0 = time.time()

    def mark_end(self):
        self.t1 = time.time()

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.file.flush()
        self.file.seek(0)
        import datetime
        rows = []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.file.read().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                ts = datetime.datetime.strptime(f[0], "%Y/%m/%d %H:%M:%S.%f").timestamp()
                rows.append((ts, float(f[1]), float(f[2]),
                             {n for n, v in zip(names, f[5:9]) if v.lower() == "active"}))
            except ValueError:
                continue
        os.unlink(self.file.name)
        if not rows:
            return None
        inside = [r for r in rows if self.t0 is not None and self.t0 <= r[0] <= self.t1]
        window = "timed region"
        if not inside:
            # region shorter than the sampling gap: the samples around it
            ts = [r[0] for r in rows]
            mid = 0.5 * (self.t0 + self.t1) if self.t0 is not None else ts[-1]
            inside = sorted(rows, key=lambda r: abs(r[0] - mid))[:2]
            window = "nearest samples to the timed region"
        reasons = set().union(*[r[3] for r in inside])
        return {"sm_mhz": statistics.median([r[1] for r in inside]),
                "sm_max_mhz": max(r[2] for r in inside), "reasons": sorted(reasons),
                "samples": len(inside), "window": window}


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


# ---------------------------------------------------------------------------
# CPU (oracle) leg

_CPU_SURF: dict = {}


def cpu_worker(args):
    """One process: the reference's sampling algorithm (oracle part 3:
    per-species yields, Poisson counts, cell draws from the cumulative
    yields, momentum rejection and boost, with MT19937 as in the reference)
    on the cell sample for its share of the events; returns (hadrons,
    seconds)."""
    n_sample, n_events, event_offset, seed = args
    sys.path.insert(0, os.path.join(HERE, "tests"))
    import oracle_lib as O
    from iss_gb300 import surfaces as S
    # the synthetic surface is built once per process (not timed)
    if _CPU_SURF.get("n") != n_sample:
        surf = S.viscous_3d(N_CELLS, seed=SEED_SURFACE)
        rec = surf.records[:: max(1, N_CELLS // n_sample)][:n_sample]
        _CPU_SURF.update(n=n_sample, fo=S.music_to_fo_surf(rec, 2))
    fo = _CPU_SURF["fo"]
    params = dict(S.DEFAULT_PARAMETERS, **PARAMS)
    t0 = time.perf_counter()
    lrf, keep = O.lrf_cells(fo)
    sp = O.chosen_species(S.TABLE_DIR, 0)
    oc = O.OracleConfig(params, S.TABLE_DIR, n_events=n_events, seed=seed)
    _, n, _ = O.reference_sampler(oc, sp, lrf, keep, seed=seed + event_offset)
    return int(n), time.perf_counter() - t0


def cpu_baseline(n_procs: int, n_sample: int, n_events: int, seed: int, pool=None):
    import multiprocessing as mp
    per = [n_events // n_procs + (1 if k < n_events % n_procs else 0) for k in range(n_procs)]
    offs = np.concatenate([[0], np.cumsum(per)[:-1]])
    jobs = [(n_sample, per[k], int(offs[k]), seed) for k in range(n_procs) if per[k] > 0]
    if len(jobs) == 1:
        res = [cpu_worker(jobs[0])]
    elif pool is not None:
        res = pool.map(cpu_worker, jobs, chunksize=1)
    else:
        with mp.get_context("spawn").Pool(len(jobs)) as pool:
            res = pool.map(cpu_worker, jobs)
    # the processes run side by side: the step takes as long as the slowest
    # (process start-up and building the synthetic surface are not timed)
    hadrons = sum(r[0] for r in res)
    return hadrons, max(r[1] for r in res)


def run_reference(args, ws, rank):
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(HERE, "tests"))
    import oracle_lib
    oracle_lib.lib()
    import multiprocessing as mp
    n_procs = max(1, os.cpu_count() or 1)
    n_sample = args.ref_cells
    rates = []
    # one process per core for the whole run; each builds the surface once
    with mp.get_context("spawn").Pool(n_procs) as pool:
        for step in range(args.warmup + args.steps):
            h, wall = cpu_baseline(n_procs, n_sample, N_EVENTS, seed=1000 + step, pool=pool)
            if step >= args.warmup:
                rates.append((h, wall))
    had = sum(r[0] for r in rates)
    sec = sum(r[1] for r in rates)
    value = had / sec
    sample = ((f"viscous 3+1D surface, all {N_CELLS} cells" if n_sample >= N_CELLS else
               f"viscous 3+1D surface, every {N_CELLS // n_sample}th cell ({n_sample} cells)") +
              f", {N_EVENTS} events split over {n_procs} processes (each process computes the "
              f"yields of its cells as one reference run does, then samples its events)")
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * sec / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "impl": "reference",
            "config": {"workload": ("viscous_3d_200k_cells_s95p_1000_events" if n_sample >= N_CELLS
                                    else "viscous_3d_200k_cells_s95p_1000_events (CPU cell sample)"),
                       "cells_sampled": n_sample, "events": N_EVENTS, "species": 319,
                       "bulk_deltaf_kind": 11, "l2": "n/a (CPU)",
                       "same_config": n_sample >= N_CELLS},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": n_procs, "kind": "port",
                             "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# GPU leg

def _chi2_two_sample(a, b):
    from scipy import stats
    a = np.asarray(a, float)
    b = np.asarray(b, float)
    m = (a + b) >= 10
    a, b = a[m], b[m]
    Na, Nb = a.sum(), b.sum()
    chi2 = np.sum((np.sqrt(Nb / Na) * a - np.sqrt(Na / Nb) * b) ** 2 / (a + b))
    return float(stats.chi2.sf(chi2, m.sum() - 1))


def surface_spread(s, batch, b_cells, b_events, params, iSS):
    """Per-surface spread of a batch: hadrons per surface of the last step
    (from the event offsets) and the throughput of five surfaces (cell-count
    quantiles 0, 0.25, 0.5, 0.75, 1) sampled alone with their own events."""
    off = s.event_offsets()
    e0 = np.concatenate([[0], np.cumsum(b_events)])
    had = off[e0[1:]] - off[e0[:-1]]
    per_ev = had / np.maximum(b_events, 1)
    out = {"surfaces": len(batch), "hadrons_min": int(had.min()), "hadrons_median": float(np.median(had)),
           "hadrons_max": int(had.max()), "hadrons_per_event_per_kcell_median":
               float(np.median(per_ev / (b_cells / 1000.0)))}
    order = np.argsort(b_cells)
    alone = []
    for q in (0.0, 0.25, 0.5, 0.75, 1.0):
        b = int(order[int(round(q * (len(order) - 1)))])
        one = iSS(".", inputfile="")
        one.set_params(**dict(params, number_of_repeated_sampling=int(b_events[b])))
        one.set_surface(batch[b])
        one.set_random_seed(20261203)
        ms = []
        for _ in range(3):
            one.generate_samples()
            ms.append(one.timings()["ms_total"])
        t = one.timings()
        alone.append({"cells": int(b_cells[b]), "events": int(b_events[b]),
                      "hadrons": int(t["n_hadrons"]), "ms": min(ms),
                      "hadrons_per_s": t["n_hadrons"] / (min(ms) * 1e-3)})
        one.close()
    out["alone"] = alone
    return out


def _oracle_yields_chunk(job):
    """FP64 oracle yields of one slice of the cells, summed over the slice
    (a worker of yields_vs_oracle)."""
    workload, lo, hi, run_params = job
    sys.path.insert(0, os.path.join(HERE, "tests"))
    import oracle_lib as O
    from iss_gb300 import surfaces as S
    fo = make_surface(workload, WORKLOADS[workload]["cells"]).fo_surf()[lo:hi]
    lrf, keep = O.lrf_cells(fo)
    ab = int(run_params.get("afterburner_type", 0))
    sp = O.chosen_species(S.TABLE_DIR, ab)
    oc = O.OracleConfig(dict(run_params), S.TABLE_DIR, n_events=1, seed=1)
    return O.yields(oc, sp, lrf, keep).sum(1)


def yields_vs_oracle(s, run_params, workload="viscous"):
    """Per-species yields of the timed surface (FP32 arithmetic with an FP64
    reduction on the GPU, read from the handle) against the FP64 CPU oracle
    (oracle/, the reference's yields restated, pinned bit-exact to the
    reference's own values): every cell, every species.  The cells are split
    over one process per host core (the per-cell yields are independent)."""
    import multiprocessing as mp
    sys.path.insert(0, os.path.join(HERE, "tests"))
    import oracle_lib as O
    from iss_gb300 import surfaces as S
    n = WORKLOADS[workload]["cells"]
    k = max(1, min(os.cpu_count() or 1, 32))
    edges = np.linspace(0, n, k + 1).astype(np.int64)
    jobs = [(workload, int(edges[j]), int(edges[j + 1]), dict(run_params)) for j in range(k)]
    with mp.get_context("spawn").Pool(k) as pool:
        ref = np.sum(pool.map(_oracle_yields_chunk, jobs, chunksize=1), axis=0)
    sp = O.chosen_species(S.TABLE_DIR, int(run_params.get("afterburner_type", 0)))
    gpu = s.species_yields()
    rel = np.abs(gpu - ref) / np.maximum(np.abs(ref), 1e-300)
    return {"cells": int(n), "species": int(len(sp)), "max_rel_err": float(rel.max()),
            "median_rel_err": float(np.median(rel)), "bar": 1e-6,
            "worst_species_pid": int(sp["pid"][int(rel.argmax())])}


def spectra_pvalues(plain, lrn, pids):
    """Two-sample chi-square / KS p-values of pT, y, phi and v2 (mean cos 2 phi
    in four pT bins) of each species, learned against plain."""
    from scipy import stats
    pv = {}
    for pid in pids:
        a, b = plain[plain["pid"] == pid], lrn[lrn["pid"] == pid]
        if len(a) < 1000:
            continue
        obs = []
        for h in (a, b):
            pt = np.hypot(h["px"], h["py"]).astype(np.float64)
            E, pz = h["E"].astype(np.float64), h["pz"].astype(np.float64)
            y = 0.5 * np.log((E + pz) / (E - pz))
            ph = np.arctan2(h["py"], h["px"]).astype(np.float64)
            obs.append((pt, y, ph))
        (pa, ya, fa), (pb, yb, fb) = obs
        e = np.quantile(np.concatenate([pa, pb]), np.linspace(0, 1, 41))
        pv[f"{pid}_pT_chi2"] = _chi2_two_sample(np.histogram(pa, e)[0], np.histogram(pb, e)[0])
        pv[f"{pid}_pT_ks"] = float(stats.ks_2samp(pa, pb).pvalue)
        e = np.linspace(-4.5, 4.5, 37)
        pv[f"{pid}_y_chi2"] = _chi2_two_sample(np.histogram(ya, e)[0], np.histogram(yb, e)[0])
        e = np.linspace(-np.pi, np.pi, 37)
        pv[f"{pid}_phi_chi2"] = _chi2_two_sample(np.histogram(fa, e)[0], np.histogram(fb, e)[0])
        zs = []
        for lo, hi in ((0, 0.5), (0.5, 1.0), (1.0, 2.0), (2.0, 4.0)):
            ca, cb = np.cos(2 * fa[(pa >= lo) & (pa < hi)]), np.cos(2 * fb[(pb >= lo) & (pb < hi)])
            if len(ca) > 100 and len(cb) > 100:
                zs.append((ca.mean() - cb.mean()) / np.sqrt(ca.var() / len(ca) + cb.var() / len(cb)))
        pv[f"{pid}_v2_chi2"] = float(stats.chi2.sf(np.sum(np.square(zs)), len(zs))) if zs else 1.0
    return pv


def learned_train(s, args):
    """Trains the proposal network on the handle's surface (plain-sampler
    momenta from seeds 10..19, Adam on the tensor cores); untimed."""
    t0 = time.perf_counter()
    curve = s.learned_train(n_momenta=args.train_momenta, first_seed=10, n_seeds=10,
                            n_steps=args.train_steps, batch=8192, learning_rate=2e-3,
                            init_seed=1)
    t_train = time.perf_counter() - t0
    st = s.learned_stats()
    return {"train_momenta": st["n_train_rows"], "train_steps": args.train_steps,
            "train_batch": 8192, "train_s_total": t_train,
            "train_ms_adam_steps": st["ms_train"],
            "loss_first": float(curve[:20].mean()), "loss_last": float(curve[-100:].mean()),
            "nll_plain_proposal": st["train_nll_plain"]}


def learned_timed(s, args, flush, plain_value):
    """The learned arm of the metric on the same surface and events: W + K
    generates with gpu_sampler = 1 (alpha = 0.8, exact mode), timed like the
    plain arm (device time, L2 flushed between steps)."""
    import torch
    s.set_params(gpu_sampler=1, gpu_learned_alpha=0.8, gpu_learned_exact=1)
    s.set_random_seed(20261203)
    for _ in range(args.warmup):
        s.generate_samples()
    ms, had, ltries, lhad, viol, exc_t, exc_h, over = [], [], 0, 0, 0, 0, 0, 0
    net_ms, fwd_ms, samp_ms = 0.0, 0.0, 0.0
    tries = 0
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        s.generate_samples()
        t, st = s.timings(), s.learned_stats()
        ms.append(t["ms_total"])
        had.append(t["n_hadrons"])
        tries += t["n_tries"]
        ltries += st["n_tries"]
        lhad += st["n_hadrons"]
        viol += st["n_violations"]
        exc_t += st["n_excess_tries"]
        exc_h += st["n_excess_hadrons"]
        over += st["n_over_one"]
        net_ms += st["ms_network"] / args.steps
        fwd_ms += st["ms_forward"] / args.steps
        samp_ms += t["ms_sample"] / args.steps
    value = sum(had) / (sum(ms) * 1e-3)
    return {"value": value, "unit": UNIT, "ms_per_step": sum(ms) / args.steps,
            "learned_over_plain": value / plain_value,
            "exact": True, "alpha": 0.8,
            "species": st["n_species"], "pairs": st["n_pairs"],
            "ms_network": net_ms, "ms_forward": fwd_ms, "ms_sample": samp_ms,
            "tries_per_hadron_learned_species": ltries / max(lhad, 1),
            "tries_per_hadron_all_species": tries / max(sum(had), 1),
            "violations": viol,
            "excess_branch_share_of_tries": exc_t / max(ltries, 1),
            "excess_branch_hadrons": exc_h,
            "mixture_ratios_above_one_per_try": over / max(ltries, 1)}


def learned_report(s, args):
    """What the network changes, on the same species: proposals per hadron
    without the network (alpha -> 0, every envelope at its cap: the plain
    sampler's acceptance) and with the pilot envelope alone (gpu_learned_exact
    = 0, inexact: ratios above 1 counted); then spectra of the learned
    species against the plain sampler on the same events (same seed, so the
    counts agree) over n_cmp events."""
    out = {}
    s.set_params(gpu_sampler=1, gpu_learned_alpha=1e-4, gpu_learned_safety=1e6, gpu_learned_exact=1)
    s.generate_samples()
    st0 = s.learned_stats()
    out["tries_per_hadron_without_network"] = st0["n_tries"] / max(st0["n_hadrons"], 1)
    s.set_params(gpu_learned_alpha=0.8, gpu_learned_safety=1.15, gpu_learned_exact=0)
    s.generate_samples()
    st1 = s.learned_stats()
    out["pilot_envelope_only"] = {"tries_per_hadron": st1["n_tries"] / max(st1["n_hadrons"], 1),
                                  "ratios_above_one_per_try": st1["n_violations"] / max(st1["n_tries"], 1),
                                  "ms_per_step": s.timings()["ms_total"]}
    s.set_params(gpu_learned_exact=1, gpu_sampler=0)
    n_ev = int(s.getVal("number_of_repeated_sampling"))
    n_cmp = min(args.spectra_events or (200 if args.workload == "finite_density" else 1000), n_ev)

    def first_events():
        # the first n_cmp events only (one copy per event)
        return np.concatenate([s.get_hadron_list_iev(e) for e in range(n_cmp)])

    s.set_random_seed(99)
    s.generate_samples()
    plain = first_events()
    s.set_params(gpu_sampler=1)
    s.set_random_seed(99)
    s.generate_samples()
    st = s.learned_stats()
    lrn = first_events()
    assert len(lrn) == len(plain)
    # the learned species: the most abundant ones (the pair tables take the
    # species with enough hadrons per cell)
    pid_order = s.species()[np.argsort(-s.species_yields())]
    pv = spectra_pvalues(plain, lrn, [int(q) for q in pid_order[:min(st["n_species"], 6)]])
    del plain, lrn
    vals = list(pv.values())
    # for an exact sampler every p-value is uniform: the chance that all of
    # n exceed 0.01 is 0.99^n (74 % for 30), so the family-wise figure
    # (Bonferroni: n times the smallest) is the one to hold against 0.01
    fam = min(1.0, len(vals) * min(vals)) if vals else None
    out["spectra_vs_plain"] = {"events": n_cmp, "tests": len(pv), "min_p": min(vals) if vals else None,
                               "below_0.01": int(sum(v < 0.01 for v in vals)),
                               "expected_below_0.01": 0.01 * len(vals),
                               "family_wise_p": fam,
                               "consistent_at_0.01": (fam > 0.01) if fam is not None else None,
                               "p_values": pv}
    s.set_params(gpu_sampler=0)
    return out


def batch_stream_e2e(s, batch, b_events, args):
    """End-to-end steps of a surface batch through the C ABI: every step
    uploads the batch's surfaces from pinned host memory
    (iss_gpu_set_surface_batch) and streams all its hadrons to the host
    (iss_gpu_generate_stream, chunks of --stream-events events through a
    device ring of two chunks); the consumer receives each chunk in host
    memory and counts its records (anything heavier would time the consumer,
    not the library).  Returns the e2e list of run_gpu's layout."""
    import torch
    # the batch's records concatenated once into page-locked memory, as a
    # caller that keeps its surfaces in one buffer would hold them
    flat = torch.from_numpy(np.concatenate([np.asarray(b, dtype=np.float32) for b in batch])).pin_memory()
    flat = flat.numpy()
    cell_off = np.concatenate([[0], np.cumsum([len(b) for b in batch])]).astype(np.int64)
    seen = [0]

    def consume(had, first, off):
        seen[0] += len(had)

    s.set_random_seed(20261203)
    s.set_surface_batch_flat(flat, cell_off, b_events)
    s.generate_stream(args.stream_events, consume)   # untimed: host buffers, first launches
    seen[0] = 0
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    t_set = 0.0
    for _ in range(args.steps):
        ta = time.perf_counter()
        s.set_surface_batch_flat(flat, cell_off, b_events)
        t_set += time.perf_counter() - ta
        s.generate_stream(args.stream_events, consume)
    torch.cuda.synchronize()
    sec = time.perf_counter() - t0
    n_in = flat.nbytes
    n_out = seen[0] * 40
    s.generate_samples()   # untimed: the handle's hadrons again, for the per-surface report
    return [seen[0], sec, n_in, n_out // args.steps,
            [1e3 * t_set / args.steps, 1e3 * (sec - t_set) / args.steps], None, None]


def e2e_handles(s, make_handle, n_handles, fo_pinned, out_t, steps, step_s, local):
    """End-to-end steps through the C ABI on n_handles handles, each driven by
    its own host thread with its own page-locked output buffer.  A handle's
    generate_into returns once its last records are on the host; while one
    handle's records cross the device-to-host link, another handle's surface
    upload, yields, counts and first sampling chunk run on the device.  Thread
    j starts j/n_handles of a step late so that the pipelines stay out of
    phase.  Every step still uploads its surface and copies all of its
    records to host memory inside the timed region.
    Returns (hadrons, seconds, steps per handle)."""
    import torch
    from iss_gb300 import HADRON_DTYPE
    handles = [s] + [make_handle() for _ in range(n_handles - 1)]
    bufs = [out_t.numpy().view(HADRON_DTYPE)]
    for h in handles[1:]:
        b = torch.empty(out_t.numel(), dtype=torch.uint8, pin_memory=True).numpy().view(HADRON_DTYPE)
        h.generate_into(b)      # untimed: the handle's buffers and first launches
        bufs.append(b)
    per = [steps // n_handles + (1 if j < steps % n_handles else 0) for j in range(n_handles)]
    counts = [0] * n_handles
    errors = []

    def work(j):
        try:
            torch.cuda.set_device(local)
            time.sleep(j * step_s / n_handles)
            for _ in range(per[j]):
                handles[j].set_surface(fo_pinned)
                h, _ = handles[j].generate_into(bufs[j])
                counts[j] += len(h)
        except Exception as e:  # re-raised on the main thread
            errors.append(e)

    torch.cuda.synchronize()
    t0 = time.perf_counter()
    threads = [threading.Thread(target=work, args=(j,)) for j in range(n_handles)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    torch.cuda.synchronize()
    sec = time.perf_counter() - t0
    if errors:
        raise errors[0]
    return sum(counts), sec, per


def run_gpu(args, ws, rank, local):
    import torch
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    from iss_gb300 import iSS, surfaces as S

    wl = WORKLOADS[args.workload]
    batch = None
    if args.workload == "batched":
        b_cells, b_events = batch_sizes(args.surfaces)
        batch = [S.viscous_3d(int(c), seed=100 + i).fo_surf() for i, c in enumerate(b_cells)]
        total_cells = int(b_cells.sum())
        fo = None
        n_events = int(b_events.sum())
        # the records of a batch (~1e2 GB) do not fit the host buffers of the
        # e2e leg below: the batch's e2e leg streams them (batch_stream_e2e)
        batch_e2e = not args.no_e2e
        args.no_e2e = True
    else:
        surf = make_surface(args.workload, args.cells)
        fo = surf.fo_surf()
        total_cells = int(fo.shape[0])
        n_events = args.events
    params = dict(S.DEFAULT_PARAMETERS, **wl["params"])
    params["number_of_repeated_sampling"] = n_events
    params["gpu_event_offset"] = rank * n_events
    if args.decays:
        params["perform_decays"] = 1
    if args.graph:
        params["gpu_graph"] = 1
    if args.mc_sampling == 2:
        # the lab-frame sampler with the reference's own defaults
        # (iSS_parameters.dat: bulk_deltaf_kind 1, restrict_deltaf 1,
        # sample_pT_up_to -1, sample_y_minus_eta_s_range 3)
        params.update(MC_sampling=2, bulk_deltaf_kind=1, restrict_deltaf=1, deltaf_max_ratio=1.0,
                      sample_pT_up_to=-1, sample_y_minus_eta_s_range=3)
    s = iSS(".", inputfile="")
    s.set_params(**params)
    if batch is not None:
        s.set_surface_batch(batch, b_events)
    else:
        # pinned host buffers for the end-to-end leg
        fo_pinned = torch.from_numpy(fo).pin_memory().numpy()
        s.set_surface(fo_pinned)
    s.set_random_seed(20261203)
    learned = None
    if args.sampler == "learned":
        learned = learned_train(s, args)
        s.set_params(gpu_sampler=1, gpu_learned_alpha=0.8, gpu_learned_exact=1)
        s.set_random_seed(20261203)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    tuning = None
    if args.shape:
        # an explicit launch shape (profiling runs: the autotuned shape without
        # the autotuner's own launches)
        kw = {k: int(v) for k, v in (kv.split("=") for kv in args.shape.split(","))}
        s.set_tuning(**kw)
        tuning = {"shape": s.get_tuning(), "autotuned": False, "explicit": True}
    elif args.autotune:
        # the library's autotuner on this workload (untimed; results do not
        # depend on the launch shape)
        shape, ms_before, ms_after = s.autotune()
        tuning = {"shape": shape, "ms_default": ms_before, "ms_tuned": ms_after}
        s.set_random_seed(20261203)
    else:
        tuning = {"shape": s.get_tuning(), "autotuned": False}

    def barrier():
        if ws > 1:
            import torch.distributed as dist
            dist.barrier()

    # clocks: nvidia-smi is started before the warm-up so that it samples
    # throughout the timed region
    clocks = ClockSampler(local)
    clocks.start()
    # warm-up steps are the timed steps' sequence (L2 flush, generate): the
    # first use of the flush loads its kernel, which must not fall in a
    # timed step (the first timed step otherwise took 12-250 ms on the host)
    for _ in range(args.warmup):
        flush.zero_()
        torch.cuda.synchronize()
        s.generate_samples()
    torch.cuda.synchronize()

    # device-timed steps; the garbage collector stays out of the timed region
    # (a collection over the objects of the set-up can pause a step's host
    # clock by a few hundred ms)
    gc.collect()
    gc.disable()
    barrier()
    torch.cuda.synchronize()
    clocks.mark_begin()
    dev_ms, hadrons, sampled, t_sample, t_yields = [], [], [], [], []
    phases = {k: 0.0 for k in ("ms_prologue", "ms_yields", "ms_cdf", "ms_counts", "ms_sample")}
    wall0 = time.perf_counter()
    step_wall, gen_wall = [], []
    for _ in range(args.steps):
        ta = time.perf_counter()
        flush.zero_()
        torch.cuda.synchronize()
        tb = time.perf_counter()
        s.generate_samples()
        tc = time.perf_counter()
        t = s.timings()
        step_wall.append(1e3 * (time.perf_counter() - ta))
        gen_wall.append(1e3 * (tc - tb))
        # with --decays a step also includes the decays (and counts final hadrons)
        dev_ms.append(t["ms_total"] + (t["ms_decays"] if args.decays else 0.0))
        hadrons.append(t["n_hadrons"])
        sampled.append(t["n_sampled"])
        t_sample.append(t["ms_sample"])
        t_yields.append(t["ms_yields"])
        for k in phases:
            phases[k] += t[k] / args.steps
    torch.cuda.synchronize()
    barrier()
    wall = time.perf_counter() - wall0
    gc.enable()
    clocks.mark_end()
    clk = clocks.stop()
    timings = s.timings()
    launches = args.steps * int(timings["kernel_launches"])
    oscar = None
    if args.oscar and rank == 0:
        # OSCAR text of the last step (formatted on the GPU), written to a
        # temporary file and removed
        from iss_gb300 import native
        d = tempfile.mkdtemp()
        fn = os.path.join(d, "OSCAR.DAT")
        t0 = time.perf_counter()
        s.write_output(native.OUTPUT_OSCAR, fn)
        dt = time.perf_counter() - t0
        size = os.path.getsize(fn)
        os.remove(fn)
        os.rmdir(d)
        oscar = {"seconds": dt, "bytes": size, "hadrons": timings["n_hadrons"],
                 "hadrons_per_s": timings["n_hadrons"] / dt}

    # end-to-end steps through the C ABI with host buffers
    e2e = None
    e2e_note = None
    if batch is not None and batch_e2e:
        e2e = batch_stream_e2e(s, batch, b_events, args)
        e2e_note = (f"streamed: iss_gpu_set_surface_batch from one pinned buffer, then "
                    f"iss_gpu_generate_stream in chunks of {args.stream_events} events through a "
                    f"device ring of two chunks; a host consumer receives every chunk")
    if not args.no_e2e:
        n_h = max(hadrons)
        out_t = torch.empty((int(n_h * 1.2) + 1024) * 40, dtype=torch.uint8).pin_memory()
        from iss_gb300 import HADRON_DTYPE
        out = out_t.numpy().view(HADRON_DTYPE)
        e_had, e_bytes_in, e_bytes_out = 0, 0, 0
        parts = [0.0, 0.0]   # set_surface, generate_into (host clock)
        torch.cuda.synchronize()
        barrier()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            ta = time.perf_counter()
            s.set_surface(fo_pinned)
            tb = time.perf_counter()
            h, off = s.generate_into(out)
            tc = time.perf_counter()
            parts[0] += tb - ta
            parts[1] += tc - tb
            e_had += len(h)
            e_bytes_in += fo_pinned.nbytes
            e_bytes_out += len(h) * 40 + off.nbytes
        torch.cuda.synchronize()
        barrier()
        e_sec = time.perf_counter() - t0
        # the device->host link alone: one step's record bytes in one copy
        nbytes = e_bytes_out // args.steps
        dev_buf = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        link = []
        for _ in range(3):
            ev0.record()
            out_t[:nbytes].copy_(dev_buf, non_blocking=True)
            ev1.record()
            ev1.synchronize()
            link.append(nbytes / (ev0.elapsed_time(ev1) * 1e-3) / 1e9)
        del dev_buf
        e2e = [e_had, e_sec, e_bytes_in // args.steps, e_bytes_out // args.steps,
               [1e3 * x / args.steps for x in parts], max(link), None]
        if args.e2e_handles > 1 and learned is None:
            def make_handle():
                h2 = iSS(".", inputfile="")
                h2.set_params(**params)
                h2.set_tuning(**s.get_tuning())
                h2.set_surface(fo_pinned)
                h2.set_random_seed(20261204)
                return h2
            barrier()
            try:
                e2e[6] = e2e_handles(s, make_handle, args.e2e_handles, fo_pinned, out_t, args.steps,
                                     e_sec / args.steps, local)
            except (RuntimeError, MemoryError) as exc:
                # e.g. no room for the extra page-locked buffers on this host:
                # the one-handle figure stands, and the line says why
                e2e_note = f"{args.e2e_handles}-handle leg not run: {exc}".splitlines()[0][:200]
                print(e2e_note, file=sys.stderr)
            barrier()

    local_value = sum(hadrons) / (sum(dev_ms) * 1e-3)
    if learned is not None:
        # --sampler learned: the headline was the learned arm; the plain arm
        # is timed the same way for the ratio
        s.set_params(gpu_sampler=0)
        s.set_random_seed(20261203)
        p_ms, p_had = [], []
        for _ in range(args.warmup + args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            s.generate_samples()
            p_ms.append(s.timings()["ms_total"])
            p_had.append(s.timings()["n_hadrons"])
        plain_value = sum(p_had[args.warmup:]) / (sum(p_ms[args.warmup:]) * 1e-3)
        learned.update(learned_timed(s, args, flush, plain_value))
        learned["plain_value"] = plain_value
        learned.update(learned_report(s, args))
    elif (args.learned_arm and args.workload == "viscous" and args.mc_sampling == 4
          and not args.decays):
        # the metric's second arm, on the same surface and events
        learned = learned_train(s, args)
        learned.update(learned_timed(s, args, flush, local_value))
        learned["plain_value"] = local_value
        learned.update(learned_report(s, args))
        s.set_params(gpu_sampler=0)
    yields_check = None
    if (rank == 0 and args.workload in ("viscous", "finite_density")
            and args.cells == WORKLOADS[args.workload]["cells"] and not args.no_oracle_check):
        s.set_params(gpu_sampler=0)
        s.generate_samples()
        yields_check = yields_vs_oracle(s, params, args.workload)
    per_surface = None
    if batch is not None and rank == 0:
        per_surface = surface_spread(s, batch, b_cells, b_events, params, iSS)
    sec = sum(dev_ms) / 1e3
    local_stats = [sum(hadrons), sec, sum(t_sample) / 1e3, sum(t_yields) / 1e3]
    e2e_best = 1
    if e2e:
        # the headline e2e: the faster of the one- and the multi-handle leg
        legs = {1: (e2e[0], e2e[1])}
        if e2e[6]:
            legs[args.e2e_handles] = (e2e[6][0], e2e[6][1])
        e2e_best = max(legs, key=lambda k: legs[k][0] / legs[k][1])
        local_stats += [legs[e2e_best][0], legs[e2e_best][1]]
    if ws > 1:
        import torch.distributed as dist
        v = torch.tensor(local_stats, dtype=torch.float64, device="cuda")
        tot = v.clone()
        dist.all_reduce(tot, op=dist.ReduceOp.SUM)
        mx = v.clone()
        dist.all_reduce(mx, op=dist.ReduceOp.MAX)
        all_h, max_sec = tot[0].item(), mx[1].item()
        e2e_h, e2e_sec = (tot[4].item(), mx[5].item()) if e2e else (0, 1)
    else:
        all_h, max_sec = local_stats[0], local_stats[1]
        e2e_h, e2e_sec = (local_stats[4], local_stats[5]) if e2e else (0, 1)

    if rank == 0:
        value = all_h / max_sec
        peak, peak_kind = peaks()
        # dominant kernel: the sampler
        samp_sec = local_stats[2]
        # the sample phase processes the sampled hadrons (before any decays)
        nh = sum(sampled)
        achieved = nh * ALG_BYTES_PER_HADRON / samp_sec / 1e9
        traffic_per_h = profiled("dram_bytes_per_hadron")
        inst_per_h = profiled("warp_instructions_per_hadron")
        per_launch_h = nh / args.steps
        clock_mhz = (clk or {}).get("sm_mhz") or 2070.0
        issue = None
        if inst_per_h:
            # issue roofline: warp instructions per second against every
            # scheduler issuing one per cycle at the sampled SM clock
            peak_issue = SMS * SCHEDULERS_PER_SM * clock_mhz * 1e6
            ach_issue = inst_per_h * nh / samp_sec
            issue = {"bound": "issue", "achieved": ach_issue, "peak": peak_issue,
                     "unit": "warp instructions/s", "frac": ach_issue / peak_issue,
                     "warp_instructions_per_hadron": inst_per_h, "sm_mhz": clock_mhz,
                     "source": f"ncu smsp__inst_executed.sum per hadron, {PROFILE}"}
        roofline = {"bound": "hbm", "kernel": "sample phase (cell_assign_kernel + sampler_kernel)",
                    "achieved": achieved,
                    "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                    "peak_source": peak_kind,
                    "traffic": (traffic_per_h * per_launch_h) if traffic_per_h else None,
                    "traffic_source": (f"ncu dram__bytes_read.sum + dram__bytes_write.sum per hadron "
                                       f"of the autotuned shape on the 200k-cell surface with 200 events "
                                       f"(cold cache), {PROFILE}, times the hadrons of one step"),
                    "issue": issue,
                    "algorithmic_bytes_per_launch": per_launch_h * ALG_BYTES_PER_HADRON,
                    "kernel_ms_per_launch": 1e3 * samp_sec / args.steps,
                    "yields_kernel_ms_per_launch": 1e3 * local_stats[3] / args.steps}
        cpu = None
        if not args.no_cpu_baseline and args.workload == "viscous" and args.mc_sampling == 4:
            h_cpu, t_cpu = cpu_baseline(1, args.cpu_cells, N_EVENTS, seed=7)
            cpu = {"value": h_cpu / t_cpu, "unit": UNIT, "cores": 1, "kind": "port",
                   "sample": f"viscous 3+1D surface, every {N_CELLS // args.cpu_cells}th cell "
                             f"({args.cpu_cells} cells), {N_EVENTS} events, one core "
                             f"({t_cpu:.1f} s)"}
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws,
                "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": 1e3 * max_sec / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": wl["data"],
                "config": {"workload": (f"viscous_3d_{args.cells // 1000}k_cells_s95p_"
                                        f"{n_events}_events" + ("_mc2_kind1_bulk" if
                                                                args.mc_sampling == 2 else "")
                                        if args.workload == "viscous" else
                                        f"{args.workload}_{total_cells}_cells_"
                                        f"{n_events}_events" + (f"_{args.surfaces}_surfaces"
                                                                if batch is not None else "")),
                           "cells": total_cells, "events_per_gpu": n_events,
                           "species": wl["species"],
                           "delta_f": {k: v for k, v in wl["params"].items()
                                       if k.startswith("include_") or k == "bulk_deltaf_kind"},
                           "sampler": args.sampler, "decays": bool(args.decays),
                           "MC_sampling": args.mc_sampling,
                           "graph_replay": bool(args.graph), "launch_shape": tuning,
                           "parallelism": f"event shards x{ws}",
                           "l2": "256 MB buffer written between steps; working set > L2",
                           "wall_s_timed": wall,
                           # host clock per step (flush + generate + timings read-out)
                           # and inside iss_gpu_generate alone, against ms_per_step
                           "host_ms_per_step": {"min": min(step_wall),
                                                "median": statistics.median(step_wall),
                                                "max": max(step_wall),
                                                "steps": [round(v, 3) for v in step_wall]},
                           "host_ms_generate": {"min": min(gen_wall),
                                                "median": statistics.median(gen_wall),
                                                "max": max(gen_wall)}},
                "roofline": roofline, "cpu_baseline": cpu,
                "e2e": ({"value": e2e_h / e2e_sec, "unit": UNIT,
                         "h2d_bytes_per_step": e2e[2], "d2h_bytes_per_step": e2e[3],
                         "handles": e2e_best,
                         "legs": {str(k): {"value": v[0] / v[1], "ms_per_step": 1e3 * v[1] / args.steps}
                                  for k, v in legs.items()},
                         **({"note": e2e_note} if e2e_note else {}),
                         "ms_per_step": 1e3 * e2e_sec / args.steps,
                         "single_handle": {"value": e2e[0] / e2e[1],
                                           "ms_per_step": 1e3 * e2e[1] / args.steps,
                                           "host_ms_per_step": {"set_surface": e2e[4][0],
                                                                "generate_into": e2e[4][1]}},
                         "d2h_link_gbs": e2e[5]}
                        if e2e else None),
                "gpu_launches": launches, "clocks": clk,
                "hadrons_per_step": nh / args.steps,
                "phase_ms_per_step": phases,
                "tries_per_hadron": timings["n_tries"] / max(timings["n_hadrons"], 1)}
        if per_surface is not None:
            line["per_surface"] = per_surface
        if yields_check is not None:
            line["yields_vs_fp64_oracle"] = yields_check
        if learned is not None:
            peak_tf = 1922.0
            try:
                with open(os.path.join(HERE, "MEASURED_PEAKS.json")) as f:
                    peak_tf = float(json.load(f)["bf16_tflops"])
            except Exception:
                pass
            fl = learned["pairs"] * MLP_FLOPS_PER_PAIR
            tf = fl / (learned["ms_forward"] * 1e-3) / 1e12
            learned["tensor_roofline"] = {"bound": "tensor", "kernel": "mlp_fwd_kernel",
                                          "achieved": tf, "peak": peak_tf, "unit": "TFLOP/s",
                                          "frac": tf / peak_tf, "flops_per_launch": fl}
            line["learned"] = learned
        if args.decays:
            line["decays"] = {"ms_per_step": timings["ms_decays"],
                              "final_hadrons_per_step": timings["n_hadrons"]}
        if oscar:
            line["oscar_writer"] = oscar
        print(json.dumps(line), flush=True)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="viscous")
    ap.add_argument("--events", type=int, default=None)
    ap.add_argument("--cells", type=int, default=None,
                    help="surface size (profiling runs use a smaller surface)")
    ap.add_argument("--surfaces", type=int, default=256, help="surfaces of --workload batched")
    ap.add_argument("--cpu-cells", type=int, default=20_000,
                    help="cells of the one-core cpu_baseline sample in the GPU line")
    ap.add_argument("--ref-cells", type=int, default=N_CELLS,
                    help="cells of --impl reference (default: the whole surface)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--e2e-handles", type=int, choices=[1, 2, 3, 4], default=2,
                    help="handles of the end-to-end leg, each driven by its own host thread, so "
                         "that one step's device work overlaps another's record copy")
    ap.add_argument("--no-oracle-check", action="store_true",
                    help="skip the per-species yields against the FP64 CPU oracle")
    ap.add_argument("--decays", action="store_true",
                    help="perform_decays = 1 (resonance decays after sampling, timed apart)")
    ap.add_argument("--oscar", action="store_true",
                    help="time the OSCAR writer on the last step's hadrons")
    ap.add_argument("--no-graph", dest="graph", action="store_false",
                    help="eager launches (default: gpu_graph = 1, each generate of the device "
                         "leg replays one captured CUDA graph)")
    ap.add_argument("--no-autotune", dest="autotune", action="store_false",
                    help="default launch shape (default: the library's autotuner picks it on "
                         "the workload before the warm-up)")
    ap.add_argument("--shape", default=None,
                    help="explicit launch shape, e.g. item_size=256,yield_groups=4,sampler_ctas=3,"
                         "assign_blocks=8 (replaces the autotuner)")
    ap.add_argument("--mc-sampling", type=int, choices=[2, 4], default=4,
                    help="4: the FSSW sampler; 2: the lab-frame EmissionFunctionArray sampler "
                         "(bulk delta f kind 1)")
    ap.add_argument("--sampler", choices=["plain", "learned"], default="plain",
                    help="learned: train the proposal network first, then sample with it")
    ap.add_argument("--no-learned", dest="learned_arm", action="store_false",
                    help="skip the learned arm of the default line (training, timed steps with "
                         "gpu_sampler = 1, spectra against the plain sampler)")
    ap.add_argument("--spectra-events", type=int, default=None,
                    help="events of the learned-vs-plain spectra comparison (default 1000; 200 for "
                         "the finite-density surface)")
    ap.add_argument("--stream-events", type=int, default=1024,
                    help="events per chunk of the batch workload's streamed e2e leg")
    ap.add_argument("--train-momenta", type=int, default=50_000_000)
    ap.add_argument("--train-steps", type=int, default=3000)
    args = ap.parse_args()
    wl = WORKLOADS[args.workload]
    if args.cells is None:
        args.cells = wl["cells"] or 0
    if args.events is None:
        args.events = wl["events"] or 0
    ws, rank, local = dist_setup()
    if args.impl == "reference":
        run_reference(args, ws, rank)
        return
    run_gpu(args, ws, rank, local)


if __name__ == "__main__":
    main()
