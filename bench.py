"""Benchmark: accepted Metropolis moves/s of batched water chains on one GB300 (and N GPUs).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Workload (the reference's batched configuration): 256 independent rigid 3-site water chains,
512-8192 molecules each (log-uniform), 0.0334 molecules/A^3, 280-360 K, one seed per chain,
switched LJ + Coulomb 10-12 A, Verlet skin 2 A, residue translations <= 0.15 A and rotations <=
15 deg, physical acceptance units.  One step = one sweep: every chain performs as many trial moves
as it has molecules, in one persistent kernel launch (replayed from a CUDA graph).  Data are
synthetic (seeded), the working set (2.1 M atoms, 1.5 GB of neighbour lists) exceeds L2, so no
flush is needed between steps.

Before the warm-up the autotuner picks the sweep's launch shape (threads per chain, CTAs per SM,
speculation width, two-CTA clusters for the largest chains) from trial sweeps; those sweeps are
untimed.

Reported: `value` = accepted moves/s over all GPUs (device time of whole sweeps, list rebuild
included, CUDA events on the library's stream, max over ranks); `e2e` = the same through the
host-buffer API (coordinates copied in and out every step, wall clock); `roofline` = FP32
throughput of the sweep kernel alone (its launches timed by event-record nodes inside the sweep
graph; 68 flops per pair interaction: distance + minimum image 23, square root and inverse 5,
Coulomb + LJ 30, accumulation 2, switch polynomial 8) against an FFMA probe measured in the same
run; `issue` = the sweep's warp-instruction issue rate (ncu instructions per move from
profiles/k_batch_sweep_water256.md times the live trial rate) against four issue slots per SM per
cycle at the sampled clock, the bound the sweep actually meets; `cpu_baseline` = the reference's
algorithm (oracle/ port, two full energies per move, one chain per host thread) on a bounded
stratified sample of the same chains.

N GPUs (`--gpus N`, one rank per GPU; launched with torchrun by the driver, or by this script when
started without it): the job's chains are the first 256*N of the same seeded generator, split
over the ranks by a greedy longest-first partition of their atom counts (shard_chains), so every
rank holds about 256 chains' worth of atoms (weak scaling); chains never exchange data, and the
only collectives are the timing max and the counter sums.

After the timed region (untimed): one logged sweep checks the mixed-precision dE of every move of a
sample of chains against the FP64 engine on the same coordinates (`batched_error`), every chain's
running energy is compared with an FP64 recompute (`max_rel_E_drift`), and the plain FP64 path is
timed through the drop-in call sequence (`plain_fp64.dropin`).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

FLOPS_PER_PAIR = 68.0
WORKLOAD = "256 rigid water chains, 512-8192 molecules (log-uniform), 0.0334 mol/A^3, 280-360 K"


def env_rank():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


CHAIN_SEED = 3


def job_specs(nchains: int, world: int, **kw):
    """(molecules, seed, temperature) of all the job's chains: nchains per GPU (kw: the
    generator's size and temperature ranges)."""
    from mc_cpp_gb300 import systems
    return systems.water_chain_specs(nchains=nchains * world, seed=CHAIN_SEED, **kw)


def rank_chains(rank: int, world: int, nchains: int, **kw):
    """This rank's shard of the job's chains (shard_chains over their atom counts) and its indices."""
    from mc_cpp_gb300 import systems
    specs = job_specs(nchains, world, **kw)
    mine = systems.shard_chains([3 * n for n, _, _ in specs], world)[rank]
    return systems.water_chains(nchains=nchains * world, seed=CHAIN_SEED, only=mine, **kw), mine


def workload_config(args, world: int):
    """The `config` of both arms' lines (the same dict, so the records compare)."""
    return {"workload": WORKLOAD, "chains_per_gpu": args.chains, "chains_total": args.chains * world,
            "l2": "no flush: per-sweep working set (1.5 GB lists, 134 MB coordinates per GPU) > 129 MB L2",
            "acceptance": "physical", "parallelism": "chains sharded over GPUs by atoms (shard_chains), weak scaling"}


class Reducer:
    """Max and sum of one float over the ranks (no-op for one rank).  Timing and statistics only:
    the chains never exchange data."""

    def __init__(self, world: int, device: str):
        self.world, self.device = world, device

    def _all(self, x, op):
        if self.world == 1:
            return float(x)
        import torch
        import torch.distributed as dist
        t = torch.tensor([float(x)], dtype=torch.float64, device=self.device)
        dist.all_reduce(t, op=op)
        return float(t.item())

    def max(self, x):
        import torch.distributed as dist
        return self._all(x, dist.ReduceOp.MAX if self.world > 1 else None)

    def sum(self, x):
        import torch.distributed as dist
        return self._all(x, dist.ReduceOp.SUM if self.world > 1 else None)


def aggregate(red: Reducer, accepted: float, trials: float, pairs: float, ms: float):
    """Whole-job rates: units of all ranks over the slowest rank's time."""
    ms_max = red.max(ms)
    sec = ms_max * 1e-3
    return {"ms_max": ms_max, "accepted_per_s": red.sum(accepted) / sec, "trials_per_s": red.sum(trials) / sec,
            "pairs_per_s": red.sum(pairs) / sec}


# ------------------------------------------------------------------ clocks during the timed region
class ClockSampler:
    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            # the timed region starts once sampling has (nvidia-smi takes a moment to start)
            t0 = time.perf_counter()
            while not self.lines and time.perf_counter() - t0 < 3.0 and self.proc.poll() is None:
                time.sleep(0.01)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = max(smax, float(f[2]))
            except ValueError:
                continue
            for k, n in enumerate(names):
                if f[5 + k].lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": smax, "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------------ CPU baseline (reference algorithm)
def cpu_sample(specs, budget_s: float, threads: int, seed: int = 17):
    """Runs the reference's Metropolis algorithm (two full getE per move, oracle/ port) on a
    stratified sample of the chains (specs: (molecules, seed, temperature) per chain), one chain
    per host thread, and estimates the accepted-moves/s rate of the whole workload on `threads`
    cores.  Returns (rate, description, cores)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as orc
    from mc_cpp_gb300 import systems
    orc.build()
    sizes = np.array([3 * n for n, _, _ in specs])
    order = np.argsort(sizes, kind="stable")
    nsamp = min(threads, len(specs))
    picks = [int(order[int((k + 0.5) * len(specs) / nsamp)]) for k in range(nsamp)]
    groups = np.array_split(order, nsamp)          # each sample stands for one size stratum
    weight = [float(sum(sizes[i] // 3 for i in g)) for g in groups]
    res = [None] * nsamp
    built = {i: systems.water_box(specs[i][0], 0.0334, specs[i][1], specs[i][2]) for i in picks}

    def work(k):
        s = built[picks[k]]
        o = orc.Oracle(s)
        o.set_acceptance_units("physical")
        t0 = time.perf_counter()
        o.energy()
        e_cost = time.perf_counter() - t0
        nmv = int(max(2, min(400, budget_s / max(1e-6, 2.0 * e_cost))))
        t0 = time.perf_counter()
        _, _, acc = o.mc_run(nmv, seed + k, trace=False)
        res[k] = (nmv, acc, time.perf_counter() - t0)

    th = [threading.Thread(target=work, args=(k,)) for k in range(nsamp)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    # stratum s: W_s moves per sweep, acceptance a_s/m_s, time per move t_s/m_s
    acc_moves = sum(w * r[1] / r[0] for w, r in zip(weight, res))
    cpu_time = sum(w * r[2] / r[0] for w, r in zip(weight, res))
    rate = acc_moves / cpu_time * threads
    desc = ("reference algorithm on %d chains (one per size stratum, %d-%d atoms), %d-%d moves each, "
            "weighted by molecules per stratum; %d threads" % (nsamp, min(sizes[picks]), max(sizes[picks]),
                                                              min(r[0] for r in res), max(r[0] for r in res), threads))
    return rate, desc, threads


def host_threads() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


# ------------------------------------------------------------------ reference arm
def run_reference(args):
    rank, world, _ = env_rank()
    if rank != 0:
        return 0
    specs = job_specs(args.chains, world)
    threads = host_threads()
    for _ in range(args.warmup):
        cpu_sample(specs, 0.5, threads)
    rates = []
    t0 = time.perf_counter()
    for _ in range(args.steps):
        r, desc, cores = cpu_sample(specs, args.ref_budget, threads)
        rates.append(r)
    wall = time.perf_counter() - t0
    v = float(np.mean(rates))
    line = {"impl": "reference", "metric": "accepted MC moves/s", "value": v, "unit": "moves/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * wall / max(1, args.steps),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": workload_config(args, world),
            "cpu_baseline": {"value": v, "unit": "moves/s", "cores": cores, "kind": "port", "sample": desc},
            "e2e": {"value": v, "unit": "moves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# ------------------------------------------------------------------ our arm
def hbm_rate(traffic, ms_per_sweep):
    """HBM bandwidth of the sweep kernels: the ncu DRAM bytes of one sweep (profiles/) over the
    event-timed sweep time, against the measured copy bandwidth (MEASURED_PEAKS.json)."""
    peak, src = 6800.0, "fallback 6.8 TB/s (no MEASURED_PEAKS.json)"
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        try:
            with open(p) as f:
                peak = float(json.load(f)["hbm_gbs"])
            src = "measured copy bandwidth, MEASURED_PEAKS.json"
        except (ValueError, KeyError, OSError):
            pass
    if not traffic or ms_per_sweep <= 0:
        return None
    gbs = traffic / (ms_per_sweep * 1e-3) / 1e9
    return {"traffic_bytes_per_step": traffic, "achieved_gbs": gbs, "peak_gbs": peak, "frac": gbs / peak,
            "peak_source": src, "traffic_source": "dram__bytes_read.sum + dram__bytes_write.sum of the sweep kernels, "
                                                  "profiles/k_batch_sweep_water256.md"}


def profile_figure(key):
    """A figure recorded in profiles/k_batch_sweep_water256.md as a `key: value ...` line."""
    p = os.path.join(ROOT, "profiles", "k_batch_sweep_water256.md")
    if not os.path.exists(p):
        return None
    for ln in open(p):
        if ln.startswith(key + ":"):
            try:
                return float(ln.split(":")[1].split()[0])
            except ValueError:
                return None
    return None


def traffic_from_profiles():
    return profile_figure("dram_bytes_per_launch")


def issue_rate(trials_per_s, sm_mhz, nsm):
    """The sweep's warp-instruction issue rate (ncu warp instructions per move, from the sweep's
    profile, times the live trial rate) against the SMs' issue peak at the sampled clock: four
    schedulers per SM, one warp instruction each per cycle.  The sweep is bound by issue, not by
    FP32 throughput or DRAM, so this is its own roofline."""
    per_move = profile_figure("warp_instructions_per_move")
    if not per_move or not sm_mhz or not nsm:
        return None
    achieved = per_move * trials_per_s / 1e9
    peak = 4.0 * nsm * sm_mhz * 1e6 / 1e9
    return {"achieved": achieved, "peak": peak, "unit": "G warp instructions/s", "frac": achieved / peak,
            "warp_instructions_per_move": per_move,
            "source": "ncu smsp__inst_executed.sum per move of the sweep kernels (profiles/k_batch_sweep_water256.md), "
                      "live trials/s, sampled SM clock, 4 issue slots per SM per cycle"}


def run_ours(args):
    import torch
    rank, world, local = env_rank()
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)
    from mc_cpp_gb300 import native
    from mc_cpp_gb300.engine import BatchChains, FFieldCUDA
    from mc_cpp_gb300 import systems

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()

    red = Reducer(world, "cuda")
    allmax, allsum = red.max, red.sum

    chains, mine = rank_chains(rank, world, args.chains)
    B = BatchChains(chains, dmax_trn=0.15, dmax_rot=15.0, acceptance="physical", seed=1000 + rank,
                    threads_per_chain=args.threads, ctas_per_sm=args.ctas_per_sm)
    natoms = B.natoms
    tuning = B.autotune(trial_sweeps=1) if not (args.threads or args.ctas_per_sm) else dict(B.tuning(), from_cache=False)
    B.sweep(args.warmup)
    barrier()
    t0, a0, _ = B.stats()
    p0 = B.pairs()
    _, nl0 = B.counters()
    with ClockSampler(local) as clk:
        barrier()
        ms, ms_lists, ms_sweep = B.time_phases(args.steps)
        barrier()
    clk_summary = clk.summary()
    _, nl1 = B.counters()
    t1, a1, e1 = B.stats()
    p1 = B.pairs()
    acc = float((a1 - a0).sum())
    trials = float((t1 - t0).sum())
    pairs = float((p1 - p0).sum())
    agg = aggregate(red, acc, trials, pairs, ms)
    ms_max = agg["ms_max"]
    value = agg["accepted_per_s"]
    # roofline of the sweep kernel (the only kernel in the timed region)
    peak = native.lib()
    import ctypes as C
    tf = C.c_double(0)
    native.check(peak.mcg_probe_fp32_tflops(C.byref(tf)))
    achieved = pairs * FLOPS_PER_PAIR / (ms_sweep * 1e-3) / 1e12
    traffic = traffic_from_profiles()
    # e2e: host buffers in and out through the public API every step (pinned host memory)
    hin = torch.empty((3, natoms), dtype=torch.float64, pin_memory=True).numpy()
    hout = torch.empty((3, natoms), dtype=torch.float64, pin_memory=True).numpy()
    B.run_host(None, 0, hout)
    hin[:] = hout
    a_prev, _ = B.run_host(hin, 1, hout)      # one untimed step: the import path's first-use allocations
    hin, hout = hout, hin
    barrier()
    acc_e = 0
    step_ms = []
    t_e = time.perf_counter()
    for _ in range(args.steps):
        t_s = time.perf_counter()
        a_now, _ = B.run_host(hin, 1, hout)
        step_ms.append((time.perf_counter() - t_s) * 1e3)
        acc_e += int((a_now - a_prev).sum())
        a_prev = a_now
        hin, hout = hout, hin
    barrier()
    e2e_s = allmax(time.perf_counter() - t_e)
    e2e = allsum(acc_e) / e2e_s
    # untimed checks: running energies against an FP64 recompute, then the dE of every move of a
    # logged sweep on sampled chains against the FP64 engine
    _, _, e_run = B.stats()
    e_64 = B.energy_fp64()
    drift = allmax(float(np.max(np.abs(e_run - e_64) / np.abs(e_64))))
    h2d = allsum(3 * natoms * 8)
    d2h = allsum(3 * natoms * 8 + len(chains) * 16)
    berr = batched_error(B, chains) if rank == 0 and not args.no_check else None
    # plain single-chain FP64 path (host-driven replay of MC_metropolis on one water box)
    plain = None
    if rank == 0 and not args.no_plain:
        w = systems.water_box()
        ff = FFieldCUDA(w, "fp64")
        ff.metropolis(50, 7, acceptance="physical", trace=False)
        tp = time.perf_counter()
        _, _, nacc, _ = ff.metropolis(args.plain_steps, 11, acceptance="physical", trace=False)
        dt = time.perf_counter() - tp
        plain = {"accepted_moves_per_s": nacc / dt, "moves_per_s": args.plain_steps / dt,
                 "workload": "one 4096-molecule water box, FP64, MC_metropolis replay through the C ABI",
                 "steps": args.plain_steps}
        ff.close()
        plain["dropin"] = dropin_rates(w)
    cpu = cpu_cfg = None
    if rank == 0 and not args.no_cpu:
        rate, desc, cores = cpu_sample(job_specs(args.chains, world), args.cpu_budget, host_threads())
        cpu = {"value": rate, "unit": "moves/s", "cores": cores, "kind": "port", "sample": desc}
        cpu_cfg = cpu_config_baselines(args.cpu_budget)
    rb, nl = B.counters()
    configs = None
    if rank == 0 and not args.no_configs:
        configs = config_extras(tf.value)
    if rank == 0:
        line = {
            "metric": "accepted MC moves/s", "value": value, "unit": "moves/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32",
            "precision": "f32 pair terms, f64 sums and acceptance, 64-bit fixed-point coordinates",
            "data": "synthetic",
            "config": workload_config(args, world),
            "rank0": {"chains": len(chains), "atoms": natoms, "molecules_per_sweep": int(natoms // 3), "tuning": tuning,
                      "chain_indices_first": mine[:8]},
            "max_dE_err_kcal_mol": berr["max_dE_err_kcal_mol"] if berr else None,
            "max_rel_E_drift": drift,
            "batched_error": berr,
            "phase_ms_per_step": {"list_rebuild": ms_lists / args.steps, "sweep_kernel": ms_sweep / args.steps},
            "trials_per_s": agg["trials_per_s"],
            "acceptance_ratio": acc / max(1.0, trials),
            "pair_interactions_per_s": agg["pairs_per_s"],
            "roofline": {"bound": "fp32", "achieved": achieved, "peak": tf.value, "unit": "TFLOP/s",
                         "frac": achieved / tf.value if tf.value > 0 else None, "traffic": traffic,
                         "peak_source": "FFMA-chain probe kernel measured in this run (no FP32 figure in MEASURED_PEAKS.json)",
                         "kernel": "k_batch_sweep<3>", "flops_per_pair": FLOPS_PER_PAIR},
            "hbm": hbm_rate(traffic, ms_sweep / args.steps),
            "issue": issue_rate(agg["trials_per_s"] * ms_max / max(ms_sweep, 1e-9), clk_summary.get("sm_mhz"),
                                torch.cuda.get_device_properties(0).multi_processor_count),
            "e2e": {"value": e2e, "unit": "moves/s", "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                    "step_ms_median": float(np.median(step_ms)), "step_ms_max": float(np.max(step_ms))},
            "gpu_launches": int(nl1 - nl0),
            "list_rebuilds_total": int(rb),
            "clocks": clk_summary,
            "plain_fp64": plain,
            "batched_vs_plain_accepted": (value / plain["accepted_moves_per_s"]) if plain else None,
            "cpu_baseline": cpu,
            "cpu_baseline_configs": cpu_cfg,
            "configs": configs,
        }
        print(json.dumps(line), flush=True)
    B.close()
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


# ------------------------------------------------------------------ untimed checks of the headline run
def batched_error(B, chains, nsample: int = 4, list_every: int = 10):
    """One logged sweep (the production sweep kernels with per-move records).  For a sample of
    chains (smallest, two middle, largest) every move is replayed on the plain FP64 engine from the
    chain's coordinates before the sweep: its FP64 dE of the recorded proposal against the sweep's
    mixed dE, and the FP64 decision (same draw) against the sweep's.  The FP64 engine's Verlet list
    (skin 2 A) is rebuilt every list_every moves, far below the displacement that could let a pair
    within the cutoff escape it."""
    from mc_cpp_gb300.engine import FFieldCUDA
    KCAL = 418.4
    order = np.argsort([c.natom for c in chains], kind="stable")
    pick = sorted({int(order[0]), int(order[len(order) // 3]), int(order[2 * len(order) // 3]), int(order[-1])})[:nsample]
    starts = {k: B.coords(k) for k in pick}
    recs = B.sweep_logged()
    errs, ties, moves = [], 0, 0
    t0 = time.perf_counter()
    for k in pick:
        s = chains[k].copy()
        s.set_coords(starts[k])
        ff = FFieldCUDA(s, "fp64", moves=False)
        beta = 1.0 / (0.83144621 / KCAL * s.temp) / KCAL          # physical units, dE in iu
        apr = 3
        for i, m in enumerate(recs[k]):
            if i % list_every == 0:
                ff.askListUpdate()
            r = int(m["residue"])
            d64 = ff.delta_e(np.arange(apr * r, apr * r + apr), m["xyz"][:apr])
            errs.append(abs(float(m["de"]) - d64) / KCAL)
            alpha = ((int(m["alpha_hi"]) << 21 ^ int(m["alpha_lo"]) >> 11) + 1) / 2.0 ** 53
            acc64 = d64 <= np.finfo(float).eps or alpha < math.exp(-beta * d64)
            acc = bool(m["flags"] & 2)
            ties += int(acc64 != acc)
            if acc:
                ff.commit()
            moves += 1
        ff.close()
    errs = np.array(errs)
    return {"max_dE_err_kcal_mol": float(errs.max()), "rms_dE_err_kcal_mol": float(np.sqrt((errs ** 2).mean())),
            "moves_checked": moves, "chains_checked": [int(chains[k].natom // 3) for k in pick],
            "decisions_differing_from_fp64": ties, "seconds": time.perf_counter() - t0,
            "how": "one logged sweep after the timed region; FP64 dE of each recorded proposal on the plain engine"}


def dropin_rates(w, steps_inc: int = 2000, steps_full: int = 100):
    """MC_metropolis's unmodified call sequence on one water box, FP64: getE(), move in place,
    getE(), restore when rejected, askListUpdate every 50 moves.  'incremental' is the drop-in's
    getE (mcg_energy_host, what FField_CUDA::getE calls); 'full' uploads all coordinates and
    recomputes the whole energy at every getE (what FField_CUDA did before)."""
    from mc_cpp_gb300.engine import FFieldCUDA
    KCAL = 418.4
    out = {"workload": "%d-molecule water box, FP64, residue translations <= 0.15 A, physical acceptance" % (w.natom // 3)}
    for mode, steps in (("incremental", steps_inc), ("full", steps_full)):
        ff = FFieldCUDA(w, "fp64", moves=False)
        x, y, z = w.x.copy(), w.y.copy(), w.z.copy()
        L = w.box[0]
        rng = np.random.default_rng(5)
        beta = 1.0 / (0.0019872 * w.temp * KCAL)

        def getE():
            if mode == "incremental":
                return ff.getE_host(x, y, z)
            ff.setCoords(np.stack([x, y, z], 1))
            return ff.getE()
        getE()
        nacc = 0
        t = time.perf_counter()
        for st in range(1, steps + 1):
            r = int(rng.integers(0, w.natom // 3))
            a = slice(3 * r, 3 * r + 3)
            eold = getE()
            bx, by, bz = x[a].copy(), y[a].copy(), z[a].copy()
            d = rng.uniform(-0.15, 0.15, 3)
            x[a] = bx + d[0]; y[a] = by + d[1]; z[a] = bz + d[2]
            for v in (x, y, z):
                v[a] -= L * np.round(v[a] / L)
            de = getE() - eold
            if de <= 0 or rng.random() < math.exp(-beta * de):
                nacc += 1
            else:
                x[a], y[a], z[a] = bx, by, bz
            if st % 50 == 0:
                if mode == "incremental":
                    ff.getE_host(x, y, z)
                ff.askListUpdate(st)
        dt = time.perf_counter() - t
        out[mode] = {"moves_per_s": steps / dt, "accepted_moves_per_s": nacc / dt, "steps": steps}
        ff.close()
    out["speedup"] = out["incremental"]["moves_per_s"] / out["full"]["moves_per_s"]
    return out


def cpu_config_baselines(budget_s: float):
    """The reference's algorithm (oracle/ port: FField_MDBAS getE, List_nonBonded update, the
    MC_metropolis loop with two full getE per move) on the other configurations, on this host:
    getE ms, Verlet update ms (OpenMP over the host threads, as the reference's list build), and MC
    moves/s over a bounded run (the 100,002-atom box: extrapolated from getE, two per move)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as orc
    from mc_cpp_gb300 import systems
    orc.build()
    out = {"kind": "port", "threads_list_build": host_threads(), "threads_energy": 1}
    cases = (("argon864", systems.argon_fcc, True), ("water4096", systems.water_box, True),
             ("peptide", systems.peptide_in_water, True), ("water100k", lambda: systems.water_box(33334, seed=11), False))
    for name, make, mc in cases:
        s = make()
        o = orc.Oracle(s, moves=mc)
        t = time.perf_counter()
        o.energy()
        ge = time.perf_counter() - t
        t = time.perf_counter()
        o.update_verlet()
        lu = time.perf_counter() - t
        rec = {"atoms": s.natom, "getE_ms": ge * 1e3, "list_update_ms": lu * 1e3,
               "pair_interactions_per_s": o.pairs_in_cutoff() / ge}
        if mc:
            nmv = int(max(2, min(2000, budget_s / max(1e-6, 2.0 * ge))))
            t = time.perf_counter()
            _, _, nacc = o.mc_run(nmv, 1234, trace=False)
            dt = time.perf_counter() - t
            rec.update({"mc_moves": nmv, "moves_per_s": nmv / dt, "accepted_moves_per_s": nacc / dt,
                        "acceptance": "reference units"})
        else:
            rec.update({"moves_per_s_extrapolated": 1.0 / (2.0 * ge)})
        out[name] = rec
        del o
    return out


# ------------------------------------------------------------------ the other configurations
def config_extras(tf_peak: float, only=None):
    """The reference's other configurations, each bounded to a few seconds: the argon replay in
    plain FP64 (the small CPU-runnable case), the solvated peptide in mixed precision with its
    error against FP64, the 100,002-atom water box (full recomputes/s and dE/s in FP64 and mixed,
    and the FP32 roofline of the mixed pair kernel), and 1024 batched argon chains."""
    KCAL = 418.4
    out = {}

    def want(name):
        return only is None or only == name
    if want("argon864"):
        out.update(_argon864())
    if want("peptide"):
        out.update(_peptide(KCAL))
    if want("water100k"):
        out.update(_water100k(tf_peak))
    if want("argon1024"):
        out.update(_argon1024(tf_peak))
    return out


def _argon864():
    """Argon, 864 atoms, FP64, single-atom moves <= 0.2 A at 120 K, reference acceptance units."""
    from mc_cpp_gb300 import systems
    from mc_cpp_gb300.engine import FFieldCUDA
    out = {}
    ff = FFieldCUDA(systems.argon_fcc(), "fp64")
    ff.metropolis(200, 1, trace=False)
    t = time.perf_counter()
    _, _, nacc, _ = ff.metropolis(20000, 7, trace=False)
    dt = time.perf_counter() - t
    out["argon864_plain_fp64"] = {"moves_per_s": 20000 / dt, "accepted_moves_per_s": nacc / dt, "steps": 20000}
    ff.close()
    return out


def _peptide(KCAL):
    """Solvated flexible peptide (40 atoms + 6000 waters): mixed precision against FP64."""
    from mc_cpp_gb300 import systems
    from mc_cpp_gb300.engine import FFieldCUDA
    out = {}
    s = systems.peptide_in_water()
    f64, fmx = FFieldCUDA(s, "fp64", moves=False), FFieldCUDA(s, "mixed", moves=False)
    e64, emx = f64.getE(), fmx.getE()
    rng = np.random.default_rng(5)
    xyz = s.coords()
    L = s.box[0]
    errs = []
    t_mx = 0.0
    for k in range(300):
        if k % 3 == 0:
            idx = np.array([int(rng.integers(0, 40))])                         # a peptide atom
        else:
            r = int(rng.integers(2, s.resid.max() + 1))                          # a water residue
            idx = np.nonzero(s.resid == r)[0]
        new = xyz[idx] + rng.uniform(-0.15, 0.15, 3)
        new -= L * np.round(new / L)
        d64 = f64.delta_e(idx, new)
        t = time.perf_counter()
        dmx = fmx.delta_e(idx, new)
        t_mx += time.perf_counter() - t
        errs.append(abs(dmx - d64) / KCAL)
    out["peptide_water_mixed"] = {"atoms": s.natom, "max_abs_dE_err_kcal_mol": float(max(errs)),
                                  "rel_total_E_err": abs(emx - e64) / abs(e64), "dE_per_s_mixed": 300 / t_mx,
                                  "moves": "300 random single-atom peptide and rigid-water displacements"}
    f64.close(); fmx.close()
    return out


def _water100k(tf_peak):
    """100,002-atom water box (33,334 molecules, 0.0334 mol/A^3), switch 10-12 A."""
    from mc_cpp_gb300 import systems
    from mc_cpp_gb300.engine import FFieldCUDA
    out = {}
    w = systems.water_box(33334, seed=11)
    res5 = {"atoms": w.natom}
    etot = {}
    for prec in ("fp64", "mixed"):
        ff = FFieldCUDA(w, prec, moves=False)
        etot[prec] = ff.getE()
        t = time.perf_counter()
        for _ in range(10):
            ff.getE()
        rec = 10 / (time.perf_counter() - t)
        rng = np.random.default_rng(9)
        xyz = w.coords()
        t = time.perf_counter()
        for _ in range(1000):
            r = int(rng.integers(1, w.resid.max() + 1))
            idx = np.arange(3 * (r - 1), 3 * r)
            ff.delta_e(idx, xyz[idx] + rng.uniform(-0.15, 0.15, 3))
        des = 1000 / (time.perf_counter() - t)
        lp, inc = ff.pair_count()
        kms = ff.time_nonbonded(20) / 20                 # the pair kernel alone, CUDA events
        res5[prec] = {"recomputes_per_s": rec, "dE_per_s": des, "pair_interactions_per_s": inc * rec,
                      "pair_kernel_ms": kms, "pair_kernel_pairs_per_s": inc / (kms * 1e-3)}
        if prec == "mixed" and tf_peak:
            # back to back, the rows (45 MB) stay in the 126 MB L2 as they do between the energy
            # calls of a run; the flushed figure writes 256 MiB before each launch
            kfl = ff.time_nonbonded_flushed(10) / 10
            res5[prec]["pair_kernel_ms_l2_flushed"] = kfl
            res5[prec]["pair_kernel_fp32_tflops"] = inc * FLOPS_PER_PAIR / (kms * 1e-3) / 1e12
            res5[prec]["pair_kernel_fp32_frac_of_probe"] = res5[prec]["pair_kernel_fp32_tflops"] / tf_peak
            res5[prec]["pair_kernel_fp32_frac_of_probe_l2_flushed"] = inc * FLOPS_PER_PAIR / (kfl * 1e-3) / 1e12 / tf_peak
        if prec == "mixed":
            # every variant of the mixed pair kernel (0-3 per-atom list, 4-5 cluster-pair, 6-9
            # group-pair), CUDA events, back to back and with the L2 flushed before each launch
            chosen, nv = ff.pair_kernel()
            per, per_fl = {}, {}
            for v in range(nv):
                ff.set_pair_kernel(v)
                per[str(v)] = ff.time_nonbonded(20) / 20
                per_fl[str(v)] = ff.time_nonbonded_flushed(5) / 5
            ff.set_pair_kernel(chosen)
            # pruned rows (the default) against the whole Verlet rows, same variant
            p_entries, _, p_ms = ff.prune_stats()
            ff.set_prune_buffer(0.0)
            whole_ms = ff.time_nonbonded(20) / 20
            ff.set_prune_buffer(0.5)
            ff.getE()
            res5[prec]["prune"] = {"buffer_A": 0.5, "pruned_entries": p_entries, "prune_ms": p_ms,
                                   "pair_kernel_ms_whole_list": whole_ms}
            ncl, ncp, nbits = ff.cluster_stats()
            res5[prec].update({"pair_kernel_variant": chosen, "variant_ms": per, "variant_ms_l2_flushed": per_fl,
                               "clusters": ncl, "cluster_pairs": ncp, "cluster_mask_pairs": nbits,
                               "rel_total_E_err_vs_fp64": abs(etot["mixed"] - etot["fp64"]) / abs(etot["fp64"])})
        res5["list_pairs"], res5["pairs_in_cutoff"] = lp, inc
        ff.close()
    out["water100k"] = res5
    return out


def _argon1024(tf_peak):
    """1024 independent argon chains (500-2000 atoms, 0.015-0.025 atoms/A^3, 90-150 K), one batch."""
    from mc_cpp_gb300 import systems
    from mc_cpp_gb300.engine import BatchChains
    out = {}
    B = BatchChains(systems.argon_chains(), dmax_trn=0.2, dmax_rot=0.0, acceptance="physical", seed=3)
    tune = B.autotune(trial_sweeps=1)
    B.sweep(3)
    t0, a0, _ = B.stats()
    p0 = B.pairs()
    tot, li, sw = B.time_phases(5)
    t1, a1, _ = B.stats()
    p1 = B.pairs()
    out["argon1024_batched"] = {"accepted_moves_per_s": float((a1 - a0).sum()) / (tot * 1e-3),
                                "trials_per_s": float((t1 - t0).sum()) / (tot * 1e-3),
                                "pair_interactions_per_s": float((p1 - p0).sum()) / (tot * 1e-3),
                                "fp32_frac_of_probe": (float((p1 - p0).sum()) * FLOPS_PER_PAIR / (sw * 1e-3) / 1e12 / tf_peak)
                                if tf_peak else None,
                                "atoms": int(B.natoms), "tuning": tune}
    B.close()
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--chains", type=int, default=256)
    ap.add_argument("--cpu-budget", type=float, default=15.0, help="seconds of CPU work per sampled chain")
    ap.add_argument("--ref-budget", type=float, default=3.0, help="seconds per sampled chain per reference step")
    ap.add_argument("--plain-steps", type=int, default=2000)
    ap.add_argument("--threads", type=int, default=0, help="threads per chain CTA (0 = library default)")
    ap.add_argument("--ctas-per-sm", type=int, default=0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-configs", action="store_true", help="skip the other configurations' figures")
    ap.add_argument("--no-check", action="store_true", help="skip the untimed FP64 check of a logged sweep")
    ap.add_argument("--master-port", type=int, default=29517, help="rendezvous port when this script starts the ranks")
    ap.add_argument("--config-only", choices=["argon864", "peptide", "water100k", "argon1024"],
                    help="print only that configuration's figures (one JSON line) and exit")
    args = ap.parse_args()
    if args.config_only:
        import ctypes as C
        from mc_cpp_gb300 import native
        tf = C.c_double(0)
        native.check(native.lib().mcg_probe_fp32_tflops(C.byref(tf)))
        print(json.dumps(config_extras(tf.value, args.config_only)), flush=True)
        return 0
    if args.warmup < 3:
        args.warmup = 3
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        # one rank per GPU: start them with torchrun on this node (127.0.0.1 rendezvous)
        cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", str(args.gpus),
               "--master-addr", "127.0.0.1", "--master-port", str(args.master_port), os.path.abspath(__file__)] + sys.argv[1:]
        return subprocess.call(cmd)
    world = env_rank()[1]
    if world != args.gpus:
        print(json.dumps({"error": "WORLD_SIZE %d differs from --gpus %d" % (world, args.gpus)}), flush=True)
        return 2
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
