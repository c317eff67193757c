#!/usr/bin/env python3
"""Benchmark: segments/s of Quicksilver's cycleTracking phase on one GB300.

Workload (N=1): the non-flat multi-material problem -- 40^3 cells over a
40 cm cube, 3 materials in concentric spherical shells (radii 8 and 16 cm),
2 isotopes x 3 reactions per material with polynomial cross sections,
230 groups, 1e6 particles (quicksilver_gb300/decks/config2.inp, seeded
synthetic deck).  One step = one cycle's tracking (the reference's
cycleTracking phase, its FOM denominator MC_Fast_Timer.cc:97-104) over the
particles the device-side cycle set-up produced; set-up and finalisation run
between steps, untimed.  Segments are the reference's _numSegments counter.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Prints one JSON line.  `value` = segments / device time of the tracking
calls with particles already in HBM (L2 flushed before every step);
`e2e` = the same through the C ABI from pinned host buffers: qsg_track_host
(the tracking launch reads the cycle's particles from, and appends census
particles to, the pinned host arrays over the host link) and the D2H read of
counters and flux, all inside the timed region; `e2e.staged_value` times the
staged calls on the same vaults (H2D copy, tracking, D2H copy of the census).
`--impl reference` times the CPU port of the reference algorithm
(oracle/qs_oracle.c, all host threads) on the same deck: the reference's own
C++ sources are not present where the benchmark runs, so the port --
bit-exact with the reference on the golden decks -- stands in for it.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

DECK = ROOT / "quicksilver_gb300" / "decks" / "config2.inp"
WORKLOAD = ("config2: 40^3-cell 40 cm cube, 3 materials in spherical shells (r=8, 16 cm), 2 isotopes x "
            "3 reactions each, polynomial cross sections, 230 groups, 1e6 particles, FP64")
METRIC = "segments/s per cycle on 1 GB300; batched+adjoint vs plain at matched tally error"
B_ALG_PER_SEGMENT = 288          # algorithmic HBM bytes per segment (136-B record read+write + 16-B flux RMW)
# per-segment ncu figures of the tracking kernel on this workload, with the
# hash of the kernel sources they were captured from
PROFILE_DATA = ROOT / "profiles" / "track_pool_kernel_config2.json"
# the reference algorithm's FP64 operations per segment per workload (tests/golden/count_fp64_work.py)
FP64_WORK = ROOT / "profiles" / "fp64_work_per_segment.json"
KERNEL_SOURCES = [ROOT / "quicksilver_gb300" / "csrc" / "track.cu", ROOT / "quicksilver_gb300" / "csrc" / "track_device.cuh"]


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled while the timed region runs."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.device_index = device_index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.device_index}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200", "-f", self.path],
                                         stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
        except (FileNotFoundError, OSError):
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if self.proc is None or not self.path or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        rows = []
        for line in Path(self.path).read_text().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def measured_peak_hbm():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
        except (KeyError, ValueError):
            pass
    return 6800.0, "fallback"


def kernel_source_hash() -> str:
    import hashlib
    h = hashlib.sha256()
    for p in KERNEL_SOURCES:
        h.update(p.read_bytes())
    return h.hexdigest()


def profile_figures():
    """(figures, matches): the committed ncu per-segment figures and whether
    they were captured from the kernel sources as they are now.  Figures
    from other sources are reported as stale and not used."""
    if not PROFILE_DATA.exists():
        return None, False
    data = json.loads(PROFILE_DATA.read_text())
    return data, data.get("kernel_source_sha256") == kernel_source_hash()


def fp64_roofline(fp64_per_segment, segments_per_s_per_gpu, peak):
    """The tracking kernel against its binding roof: FP64 warp instructions
    per second (ncu's count per segment x the measured segment rate) over the
    device's FP64 issue rate (qsg_measure_fp64_rate)."""
    if not fp64_per_segment or not peak:
        return None
    achieved = fp64_per_segment * segments_per_s_per_gpu
    return {"achieved": achieved, "peak": peak, "unit": "FP64 warp instructions/s", "frac": achieved / peak,
            "fp64_warp_instructions_per_segment": fp64_per_segment,
            "peak_source": "measured in this run (qsg_measure_fp64_rate: independent DFMA chains, 16 warps/SM)",
            "per_segment_source": "ncu sm__inst_executed_pipe_fp64.sum / segments, " + PROFILE_DATA.name}


def fp64_work_roofline(workload, segments_per_s_per_gpu, peak_warp_instructions):
    """The reference algorithm's FP64 work (its +, -, *, / and sqrt per
    segment as written, counted by the C restatement on this workload;
    FP64_WORK) done per second, against the device's FP64 FMA rate (the
    measured DFMA warp-instruction rate x 32 lanes x 2 FLOP).  The kernel's
    FP32 screen skips most of the algorithm's facet tests, so this can
    approach or pass 1 without the FP64 pipe doing that much."""
    if not FP64_WORK.exists() or not peak_warp_instructions:
        return None
    w = json.loads(FP64_WORK.read_text()).get("workloads", {}).get(workload)
    if not w:
        return None
    per_seg = w["fp64_ops_per_segment"]
    achieved = per_seg * segments_per_s_per_gpu
    peak = 64.0 * peak_warp_instructions
    return {"achieved": achieved, "peak": peak, "unit": "FLOP/s", "frac": achieved / peak,
            "algorithm_fp64_ops_per_segment": per_seg,
            "per_segment_source": FP64_WORK.name + " (" + w["workload"] + ")",
            "peak_source": "measured in this run: qsg_measure_fp64_rate x 32 lanes x 2 FLOP per DFMA"}


def _sync():
    import torch
    torch.cuda.synchronize()


def measure_batched(tune_space=None, n_problems=64, fixed_shape=None):
    """Batched form on the uneven ensemble (64 problems, mesh edge in
    {8..48}, 1e4-2e6 particles, 10 cycles): one persistent launch per pass
    for all problems, cycles replayed from CUDA graphs, kernel shape from the
    autotuner -- against the plain path run problem by problem
    (MonteCarlo.run: host-driven cycles, one handle per problem).  Both runs
    track the same histories (same per-problem seeds), so the tally standard
    errors are equal by construction; the balance counters are compared bit
    for bit."""
    from quicksilver_gb300 import Deck
    from quicksilver_gb300.autotune import autotune
    from quicksilver_gb300.decks.make_decks import config3
    from quicksilver_gb300.monte_carlo import BatchMonteCarlo, MonteCarlo, seed_offset
    texts = config3()[:n_problems]
    decks = [Deck.from_string(t) for t in texts]
    problems = [d.build() for d in decks]
    offs = [seed_offset(d.simulation.seed) for d in decks]
    cycles = decks[0].simulation.n_steps
    t0 = time.perf_counter()
    space = tune_space or {"block_size": (128,), "pool_collision_step": (24, 32), "pool_refill": (8, 16, 32),
                           "flux_replicas": (1,)}
    if fixed_shape is None:
        best = autotune(texts, scale=0.1, cycles=1, warmup=1, cache_path=None, space=space, problems=problems)
    else:
        best = dict(fixed_shape)
    tune_s = time.perf_counter() - t0
    bmc = BatchMonteCarlo(decks, problems=problems, seed_offsets=offs, flux_replicas=best["flux_replicas"])
    try:
        bmc.tune(**{k: best[k] for k in ("block_size", "pool_collision_step", "pool_refill") if k in best})
        bmc.run(1, use_graph=True)             # warm-up cycle (captures the graphs)
        first = bmc.cycles
        _sync()
        t0 = time.perf_counter()
        bmc.run_cycles(cycles, use_graph=True)
        _sync()
        t_batch = time.perf_counter() - t0
        hb = bmc.history(first, cycles)
        flags = bmc.device_status()
    finally:
        bmc.close()
    # the plain path, problem by problem, from the same starting state (one warm-up cycle)
    t_plain, seg_plain, same = 0.0, 0, True
    per_problem = []
    for p, (d, hp, off) in enumerate(zip(decks, problems, offs)):
        mc = MonteCarlo(d, problem=hp, seed_offset=off)
        try:
            mc.run(1)
            _sync()
            t0 = time.perf_counter()
            h = mc.run(cycles)
            _sync()
            dt = time.perf_counter() - t0
            t_plain += dt
            seg_plain += h.segments()
            per_problem.append((dt, h.segments()))
            same &= bool(np.array_equal(h.balance, hb.balance[:, p, :]))
        finally:
            mc.close()
    seg_b = hb.segments()
    # breakdown: per mesh edge, the plain path's time and rate beside the same
    # problems batched on their own; per particle-count decade, the plain rate
    edges = [int(d.simulation.nx) for d in decks]
    npart = [int(d.simulation.n_particles) for d in decks]
    by_edge = {}
    for e in sorted(set(edges)):
        idx = [p for p in range(len(decks)) if edges[p] == e]
        tp = sum(per_problem[p][0] for p in idx)
        sp = sum(per_problem[p][1] for p in idx)
        sub = BatchMonteCarlo([decks[p] for p in idx], problems=[problems[p] for p in idx],
                              seed_offsets=[offs[p] for p in idx], flux_replicas=best["flux_replicas"])
        try:
            sub.tune(**{k: best[k] for k in ("block_size", "pool_collision_step", "pool_refill") if k in best})
            sub.run(1, use_graph=True)
            f0 = sub.cycles
            _sync()
            t0 = time.perf_counter()
            sub.run_cycles(cycles, use_graph=True)
            _sync()
            tb = time.perf_counter() - t0
            sb = sub.history(f0, cycles).segments()
        finally:
            sub.close()
        by_edge[str(e)] = {"problems": len(idx), "empty_problems": sum(1 for p in idx if per_problem[p][1] == 0),
                           "segments": sp, "plain_s": tp, "plain_segments_per_s": sp / tp if tp else None,
                           "batched_alone_s": tb, "batched_alone_segments_per_s": sb / tb if tb else None,
                           "speedup_batched_alone": (tp / tb) if tb else None}
    by_particles = {}
    for lo, hi in ((1e4, 1e5), (1e5, 1e6), (1e6, 2e6 + 1)):
        idx = [p for p in range(len(decks)) if lo <= npart[p] < hi]
        tp = sum(per_problem[p][0] for p in idx)
        sp = sum(per_problem[p][1] for p in idx)
        by_particles[f"{lo:.0e}-{min(hi, 2e6):.0e}"] = {"problems": len(idx), "segments": sp, "plain_s": tp,
                                                        "plain_segments_per_s": sp / tp if tp else None}
    for hp in problems:
        hp.close()
    return {"workload": f"{n_problems} independent problems (mesh edge from {{8,16,24,32,48}} cm, 1e4-2e6 "
                        "particles log-uniform, 1-3 materials, 230 groups), 10 cycles each after 1 warm-up cycle",
            "batched_segments_per_s": seg_b / t_batch, "batched_s": t_batch,
            "plain_problem_by_problem_segments_per_s": seg_plain / t_plain, "plain_s": t_plain,
            "speedup_at_equal_tally_error": (seg_b / t_batch) / (seg_plain / t_plain),
            "segments": seg_b, "balance_bit_exact_vs_plain": same, "device_flags": flags,
            "by_mesh_edge": by_edge, "by_particle_count": by_particles,
            "tuning": {k: best[k] for k in ("block_size", "pool_collision_step", "pool_refill", "flux_replicas")},
            "tune_s": tune_s, "timing": "wall clock, whole cycles, synchronised"}


def measure_adjoint(replicas=6):
    """Differentiated form on the differentiated homogeneous-box problem
    (config4: 3 materials, escape boundaries, 1e6 particles, 20 cycles,
    12 parameters = 3 materials x {scatter, absorption} x 2 bands split at
    1 MeV).  One sensitivity run gives d(total flux)/dtheta and
    d(leakage)/dtheta for all 12 parameters; the plain kernel needs a central
    difference per parameter (2 runs each, common random numbers).  Replica
    variances (distinct seed offsets) of both estimators give the number of
    plain runs needed to match the sensitivity run's standard error:
    speedup = 2 K median_j(var_FD_j / var_score_j) T_plain / T_sens over the
    24 components j.  The central differences use step 1e-2 (lower variance
    than 1e-4, so the comparison favours the plain path); the step-1e-4
    variance ratio is reported beside it."""
    from quicksilver_gb300 import Deck
    from quicksilver_gb300.monte_carlo import MonteCarlo, seed_offset
    from quicksilver_gb300.sensitivity import Param, band_params, scaled_problem
    deck = Deck.from_file(ROOT / "quicksilver_gb300" / "decks" / "config4.inp")
    hp0 = deck.build()
    params = band_params(hp0.array("energies"), hp0.num_materials)
    hp0.close()
    K = len(params)

    def one_run(prms, off, sens=True):
        problem = scaled_problem(deck, prms)
        mc = MonteCarlo(deck, problem=problem, seed_offset=off)
        try:
            if sens:
                mc.tracker.enable_sensitivity(prms)
            _sync()
            t0 = time.perf_counter()
            h = mc.run()
            _sync()
            dt = time.perf_counter() - t0
            out = mc.tracker.read_sensitivity() if sens else None
            return out, dt, h.segments()
        finally:
            mc.close()
            problem.close()

    steps = (1e-2, 1e-4)
    lr = np.zeros((replicas, 2, K))
    fd = {h: np.zeros((replicas, 2, K)) for h in steps}
    t_sens = t_plain = 0.0
    seg_sens = seg_plain = 0
    one_run(params, 1, sens=False)   # warm-up (module load, first allocations)
    for i in range(replicas):
        off = seed_offset(4000 + i)
        out, dt, seg = one_run(params, off)
        t_sens += dt
        seg_sens += seg
        lr[i, 0] = out["dflux"].sum(axis=0)
        lr[i, 1] = out["dleak"][0]
        _, dt, seg = one_run(params, off, sens=False)
        t_plain += dt
        seg_plain += seg
        for h in steps:
            for k in range(K):
                vals = []
                for sgn in (1.0, -1.0):
                    sh = [p if j != k else Param(p.material, p.reaction, p.group_lo, p.group_hi, 1.0 + sgn * h)
                          for j, p in enumerate(params)]
                    o, _, _ = one_run(sh, off)
                    vals.append((o["flux_cell"].sum(), o["leak"][0]))
                fd[h][i, 0, k] = (vals[0][0] - vals[1][0]) / (2 * h)
                fd[h][i, 1, k] = (vals[0][1] - vals[1][1]) / (2 * h)
    var_lr = lr.var(axis=0, ddof=1).ravel()
    res = {}
    for h in steps:
        var_fd = fd[h].var(axis=0, ddof=1).ravel()
        ok = var_lr > 0
        ratio = var_fd[ok] / var_lr[ok]
        res[h] = (float(np.median(ratio)), float(ratio.min()), float(ratio.max()))
    rate_plain = seg_plain / t_plain
    rate_sens = seg_sens / t_sens
    # plain runs needed per sensitivity run at equal standard error, per
    # component: the median component is the headline, the worst and best
    # beside it
    speedup = 2 * K * res[1e-2][0] * (t_plain / t_sens)
    speedups = {"min": 2 * K * res[1e-2][1] * (t_plain / t_sens), "median": speedup,
                "max": 2 * K * res[1e-2][2] * (t_plain / t_sens)}
    return {"workload": "config4: 10^3 cells, 10 cm box, 3 materials (spheres r=2, 4 cm), escape boundaries, "
                        "230 groups, 1e6 particles, 20 cycles; 12 scale parameters",
            "params": K, "replicas": replicas,
            "plain_segments_per_s": rate_plain, "sens_segments_per_s": rate_sens,
            "sens_time_over_plain": t_sens / t_plain,
            "fd_step": 1e-2, "variance_ratio_fd_over_score": {"median": res[1e-2][0], "min": res[1e-2][1],
                                                              "max": res[1e-2][2]},
            "variance_ratio_fd_step_1e-4": {"median": res[1e-4][0], "min": res[1e-4][1], "max": res[1e-4][2]},
            "speedup_at_equal_tally_error": speedup,
            "speedup_at_equal_tally_error_over_components": speedups,
            "effective_segments_per_s": speedup * rate_plain,
            "timing": "wall clock of MonteCarlo.run (20 whole cycles), synchronised; handle set-up excluded"}


def run_config3(args):
    """--workload config3: the batched form alone (its own JSON line), the
    uneven ensemble's first --config3-problems problems; --fixed-shape skips
    the autotuner (block 128, collision step 32, refill 8, one flux replica),
    which keeps the launch sequence short for a profiler."""
    shape = ({"block_size": 128, "pool_collision_step": 32, "pool_refill": 8, "flux_replicas": 1}
             if args.fixed_shape else None)
    with ClockSampler(0) as clocks:
        b = measure_batched(n_problems=args.config3_problems, fixed_shape=shape)
    line = {"metric": METRIC, "value": b["batched_segments_per_s"], "unit": "segments/s", "n_gpus": 1,
            "steps": 10, "warmup": 1, "ms_per_step": 1e3 * b["batched_s"] / 10, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded decks make_decks.config3)",
            "config": {"workload": b["workload"], "step": "one whole cycle of every problem (CUDA graph)"},
            "forms": {"batched": b}, "clocks": clocks.summary()}
    print(json.dumps(line), flush=True)


def run_config5(args):
    """--workload config5: the large batched + differentiated run -- 8 replicas
    of a 5-slab 64^3-cell problem (1e7 particles each, distinct seeds, escape
    boundaries, 230 groups), 20 parameters (5 materials x {scatter,
    absorption} x 2 bands) tied across the replicas, every cycle one CUDA
    graph whose tracking pass is one persistent launch over all replicas with
    forward tallies and sensitivities.  20 timed cycles after 1 warm-up cycle;
    then 5 cycles with the sensitivities switched off give the forward-only
    rate of the same batch.  The replicas' spread gives the standard error of
    each derivative."""
    import torch
    from quicksilver_gb300 import Deck
    from quicksilver_gb300.decks.make_decks import config5
    from quicksilver_gb300.monte_carlo import BatchMonteCarlo, seed_offset
    from quicksilver_gb300.sensitivity import band_params, tie_across_problems
    from quicksilver_gb300 import _native as N
    n_part = int(round(1e7 * args.config5_scale))
    decks = [Deck.from_string(t) for t in config5(n_particles=n_part)]
    t0 = time.perf_counter()
    problems = [d.build() for d in decks]
    build_s = time.perf_counter() - t0
    offs = [seed_offset(d.simulation.seed) for d in decks]
    cap = int(1.3 * (n_part + n_part // 10)) + 1024
    cycles = decks[0].simulation.n_steps
    base = band_params(problems[0].array("energies"), problems[0].num_materials)
    t0 = time.perf_counter()
    bmc = BatchMonteCarlo(decks, problems=problems, seed_offsets=offs, store_capacity=cap, max_passes=2)
    params = tie_across_problems(base, bmc.tracker.material_offsets())
    bmc.tracker.enable_sensitivity(params)
    setup_s = time.perf_counter() - t0
    bmc.run(1, use_graph=True)
    bmc.tracker.reset_sensitivity()
    first = bmc.cycles
    with ClockSampler(0) as clocks:
        _sync()
        t0 = time.perf_counter()
        bmc.run_cycles(cycles, use_graph=True)
        _sync()
        t_sens = time.perf_counter() - t0
    hist = bmc.history(first, cycles)
    seg = hist.segments()
    sens = bmc.tracker.read_sensitivity()
    flags = bmc.device_status()
    # forward-only rate of the same batch
    N.check(N.lib().qsg_enable_sensitivity(bmc.tracker.handle, C.byref(N.QsgSensitivity())))
    bmc.run(1, use_graph=True)
    first2 = bmc.cycles
    _sync()
    t0 = time.perf_counter()
    bmc.run_cycles(5, use_graph=True)
    _sync()
    t_plain = time.perf_counter() - t0
    seg_plain = bmc.history(first2, 5).segments()
    flags |= bmc.device_status()
    coff = bmc.tracker.cell_offsets
    bmc.close()
    P, K = len(decks), len(params)
    dflux_p = np.array([sens["dflux"][int(coff[q]):int(coff[q + 1])].sum(axis=0) for q in range(P)])
    se = lambda a: (a.std(axis=0, ddof=1) / np.sqrt(P)).tolist()
    line = {
        "metric": METRIC, "value": seg / t_sens, "unit": "segments/s", "n_gpus": 1, "steps": cycles, "warmup": 1,
        # (each cell sources floor(volume x rate x dt / particle weight) particles, so the
        # 64^3 mesh needs >= 3e6 particles per replica for any source at all)
        "ms_per_step": 1e3 * t_sens / cycles, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic (seeded decks make_decks.config5)",
        "config": {"workload": f"config5: 8 replicas x 64^3-cell 64 cm cube, 5 slabs along z, 5 materials, escape "
                               f"boundaries, 230 groups, {n_part:.0e} particles each, 20 cycles, {K} parameters tied "
                               f"across replicas", "step": "one whole cycle (CUDA graph) with sensitivities",
                   "timing": "wall clock of 20 graph replays, synchronised", "build_s": build_s, "setup_s": setup_s},
        "forms": {"batched_adjoint_segments_per_s": seg / t_sens, "batched_forward_segments_per_s": seg_plain / t_plain,
                  "adjoint_time_over_forward": (t_sens / seg) / (t_plain / seg_plain) if seg and seg_plain else None,
                  "segments": seg, "leak_mean": float(sens["leak"].mean()),
                  "dflux_total_mean": dflux_p.mean(axis=0).tolist(), "dflux_total_se": se(dflux_p),
                  "dleak_mean": sens["dleak"].mean(axis=0).tolist(), "dleak_se": se(sens["dleak"])},
        "gpu_launches": cycles * 9, "device_flags": flags, "clocks": clocks.summary(),
    }
    for hp in problems:
        hp.close()
    print(json.dumps(line), flush=True)


def reduce_over_ranks(pg, times, counts, device):
    """Whole-job figures of a multi-rank run: the max over ranks of each
    timed duration, the sum over ranks of each count (every rank tracks its
    own replica of the workload, so the units add up).  pg None: one rank."""
    if pg is None:
        return list(times), [int(c) for c in counts]
    import torch
    t = torch.tensor(list(times), dtype=torch.float64, device=device)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    c = torch.tensor(list(counts), dtype=torch.float64, device=device)
    pg.all_reduce(c)
    return t.tolist(), [int(v) for v in c.tolist()]


def host_cpu_model() -> str:
    """The host CPU's model name (lscpu, else /proc/cpuinfo, else the machine type)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.strip().startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        for line in Path("/proc/cpuinfo").read_text().splitlines():
            if line.lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    import platform
    return platform.machine()


def run_reference_arm(args, world, rank):
    """--impl reference: the CPU port of the reference algorithm on the host cores."""
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    # one OpenMP thread per core, kept there (set before the port's OpenMP
    # runtime loads; a caller's own settings win)
    os.environ.setdefault("OMP_PROC_BIND", "close")
    os.environ.setdefault("OMP_PLACES", "cores")
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle_py
    from quicksilver_gb300 import Deck
    deck = Deck.from_file(DECK)
    sim = deck.simulation
    hp = deck.build()
    run = oracle_py.OracleRun(hp.ptr, hp.num_cells, hp.num_groups, hp.source_rates(), sim.n_particles,
                              sim.e_min, sim.e_max, sim.low_weight_cutoff, sim.load_balance, keepalive=hp)
    for _ in range(args.warmup):
        run.cycle_init()
        run.cycle_tracking(threads)
        run.cycle_finalize()
    seg, secs = 0, 0.0
    for _ in range(args.steps):
        run.cycle_init()
        t0 = time.perf_counter()
        run.cycle_tracking(threads)
        secs += time.perf_counter() - t0
        seg += int(run.balance()[12])
        run.cycle_finalize()
    value = seg / secs
    # one more cycle on one core, for the scaling of the CPU path
    run.cycle_init()
    t0 = time.perf_counter()
    run.cycle_tracking(1)
    secs1 = time.perf_counter() - t0
    seg1 = int(run.balance()[12])
    run.cycle_finalize()
    run.close()
    sample = (f"{args.steps} whole config2 cycles ({seg} segments) after {args.warmup} warm-up cycles, "
              f"{threads} OpenMP threads")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "segments/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * secs / max(args.steps, 1),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded deck config2.inp)",
            "config": {"workload": WORKLOAD, "impl": "CPU port of the reference algorithm (oracle/qs_oracle.c), "
                       "OpenMP over particles; the reference C++ sources are not present on this host"},
            "cpu_baseline": {"value": value, "unit": "segments/s", "cores": threads, "kind": "port",
                             "cpu": host_cpu_model(), "compiler": oracle_py.compiler_version(),
                             "omp": f"OMP_PROC_BIND={os.environ['OMP_PROC_BIND']} OMP_PLACES={os.environ['OMP_PLACES']}",
                             "sample": sample, "value_1_thread": seg1 / secs1,
                             "sample_1_thread": f"config2 cycle {args.warmup + args.steps} ({seg1} segments, "
                                                f"{secs1:.1f} s) on one core"},
            "e2e": {"value": value, "unit": "segments/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def reference_arm_baseline(warmup: int, steps: int):
    """cpu_baseline of the GPU line: the reference arm itself (`--impl
    reference`, same cycles) run in a fresh child process, so that both
    numbers come from one measurement path."""
    env = {k: v for k, v in os.environ.items() if k not in ("RANK", "WORLD_SIZE", "LOCAL_RANK")}
    res = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", str(steps),
                          "--warmup", str(warmup)], capture_output=True, text=True, env=env, cwd=str(ROOT))
    lines = [l for l in res.stdout.splitlines() if l.startswith("{")]
    if res.returncode != 0 or not lines:
        return {"value": None, "unavailable": (res.stderr or "no output")[-300:]}
    return json.loads(lines[-1])["cpu_baseline"]


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--flux-replicas", type=int, default=1)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-forms", action="store_true", help="skip the batched and differentiated forms")
    ap.add_argument("--workload", default="config2", choices=["config2", "config3", "config5"],
                    help="config3: the batched form alone; config5: the large batched + differentiated run "
                         "(each its own JSON line)")
    ap.add_argument("--config3-problems", type=int, default=64, help="config3: the first this many problems")
    ap.add_argument("--fixed-shape", action="store_true", help="config3: no autotuner, the default kernel shape")
    ap.add_argument("--config5-scale", type=float, default=1.0,
                    help="particle-count scale of config5 (>= 0.3: below that no cell sources a particle)")
    ap.add_argument("--kernel", type=int, default=1, choices=[0, 1],
                    help="tracking kernel: 1 warp particle pool (default), 0 one history per lane")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    world, rank, local = dist_env()

    if args.impl == "reference":
        run_reference_arm(args, world, rank)
        return
    if args.workload in ("config3", "config5"):
        if rank == 0:
            (run_config3 if args.workload == "config3" else run_config5)(args)
        return

    import torch
    from quicksilver_gb300 import Deck
    from quicksilver_gb300 import _native as N
    from quicksilver_gb300.monte_carlo import MonteCarlo

    torch.cuda.set_device(local)
    pg = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
        pg = dist

    def barrier():
        if pg is not None:
            pg.barrier()
        torch.cuda.synchronize()

    deck = Deck.from_file(DECK)
    mc = MonteCarlo(deck, flux_replicas=args.flux_replicas, device=local)
    h = mc.tracker.handle
    lib = N.lib()
    N.check(lib.qsg_set_track_kernel(h, args.kernel))
    stream = torch.cuda.current_stream()
    sp = C.c_void_p(stream.cuda_stream)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")   # 256 MiB > 129 MB L2

    def flush_l2():
        flush.add_(1.0)

    # warm-up cycles (whole cycles on the device)
    for _ in range(args.warmup):
        mc.cycle_init(stream)
        mc.cycle_tracking(stream)
        mc.cycle_finalize(stream)
    barrier()

    # ---- device-resident timed steps: tracking phase only ----
    events = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    first_cycle = mc.cycles
    with ClockSampler(local) as clocks:
        barrier()
        wall0 = time.perf_counter()
        for k in range(args.steps):
            mc.cycle_init(stream)
            flush_l2()
            events[k][0].record(stream)
            N.check(lib.qsg_track_cycle(h, sp))
            events[k][1].record(stream)
            mc.cycle_finalize(stream)
        barrier()
        wall = time.perf_counter() - wall0
    ms = [a.elapsed_time(b) for a, b in events]
    hist = mc.history(first_cycle, args.steps)
    segments = int(hist.balance[:, N.BAL["num_segments"]].sum())
    track_s = sum(ms) / 1e3
    flags = mc.device_status()

    # ---- end to end through the C ABI with pinned host buffers ----
    n_cap = int(2 * deck.simulation.n_particles)
    pinned = {name: torch.empty(n_cap, dtype={"<f8": torch.float64, "<u8": torch.int64, "<i4": torch.int32}[
        N.PARTICLE_DTYPE[name].str], pin_memory=True) for name in N.SOA_FIELDS}
    census_pinned = {name: torch.empty_like(t, pin_memory=True) for name, t in pinned.items()}
    soa_in = N.soa_from_pointers({k: v.data_ptr() for k, v in pinned.items()})
    soa_out = N.soa_from_pointers({k: v.data_ptr() for k, v in census_pinned.items()})
    ncell_g = mc.problem.num_cells * mc.problem.num_groups
    flux_host = torch.empty(ncell_g, dtype=torch.float64, pin_memory=True)
    bal_host = torch.empty(13, dtype=torch.int64, pin_memory=True)
    bal_p = C.cast(C.c_void_p(bal_host.data_ptr()), C.POINTER(C.c_uint64))
    flux_p = C.cast(C.c_void_p(flux_host.data_ptr()), C.POINTER(C.c_double))
    e2e_s, e2e_seg, h2d, d2h = 0.0, 0, 0, 0
    staged_s, staged_seg = 0.0, 0
    e2e_steps = args.steps
    for k in range(e2e_steps):
        mc.cycle_init(stream)
        n = C.c_uint64()
        N.check(lib.qsg_get_processing(h, C.byref(soa_in), n_cap, C.byref(n)))   # the host's vault, untimed
        # (a) qsg_track_host: the tracking launch reads the vault from, and
        # appends the census to, the pinned host arrays over the host link
        barrier()
        t0 = time.perf_counter()
        N.check(lib.qsg_reset_tallies(h))
        nc = C.c_uint64()
        N.check(lib.qsg_track_host(h, C.byref(soa_in), n.value, C.byref(soa_out), n_cap, C.byref(nc), sp))
        N.check(lib.qsg_read_tallies(h, bal_p, flux_p))
        torch.cuda.synchronize()
        e2e_s += time.perf_counter() - t0
        e2e_seg += int(bal_host[12])
        h2d += 136 * n.value
        d2h += 136 * nc.value + 13 * 8 + 8 * ncell_g
        # (b) the staged calls on the same vault: copy in, track, copy the
        # census out (this also leaves the census in the handle for the next
        # cycle init)
        barrier()
        t0 = time.perf_counter()
        N.check(lib.qsg_reset_tallies(h))
        N.check(lib.qsg_set_particles(h, C.byref(soa_in), n.value))
        N.check(lib.qsg_track_cycle(h, sp))
        nc2 = C.c_uint64()
        N.check(lib.qsg_get_census(h, C.byref(soa_out), n_cap, C.byref(nc2)))
        N.check(lib.qsg_read_tallies(h, bal_p, flux_p))
        torch.cuda.synchronize()
        staged_s += time.perf_counter() - t0
        staged_seg += int(bal_host[12])
        mc.cycle_finalize(stream)
    flags |= mc.device_status()

    (track_s, e2e_s, wall, staged_s), (segments, e2e_seg, staged_seg) = reduce_over_ranks(
        pg, [track_s, e2e_s, wall, staged_s], [segments, e2e_seg, staged_seg], "cuda")
    if rank != 0:
        return

    fp64_peak = N.measure_fp64_rate(local)
    value = segments / track_s
    peak, peak_kind = measured_peak_hbm()
    seg_per_launch = segments / world / args.steps
    achieved = B_ALG_PER_SEGMENT * seg_per_launch / (track_s / args.steps) / 1e9
    prof, prof_current = profile_figures()
    tps = prof.get("dram_bytes_per_segment") if (prof and prof_current) else None
    fp64_ps = prof.get("fp64_warp_instructions_per_segment") if (prof and prof_current) else None
    line = {
        "metric": METRIC, "value": value, "unit": "segments/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * track_s / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded deck config2.inp)",
        "config": {"workload": WORKLOAD, "step": "one cycle's tracking (cycleTracking phase)",
                   "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
                   "l2": "flushed (256 MiB write) before every timed step", "particles_in_hbm": True,
                   "flux_replicas": args.flux_replicas, "wall_s_timed_region": wall,
                   "kernel": "warp particle pool" if args.kernel == 1 else "one history per lane"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)",
                     "traffic": (tps * seg_per_launch) if tps else None,
                     "algorithmic_bytes_per_segment": B_ALG_PER_SEGMENT,
                     "note": "not HBM-bound: the binding roof is FP64 issue (fp64_issue)",
                     "profile": {"file": str(PROFILE_DATA.relative_to(ROOT)), "matches_kernel_source": prof_current,
                                 "captured": prof.get("captured") if prof else None},
                     "fp64_issue": fp64_roofline(fp64_ps, seg_per_launch / (track_s / args.steps), fp64_peak),
                     "fp64_algorithm": fp64_work_roofline("config2", seg_per_launch / (track_s / args.steps),
                                                          fp64_peak)},
        "e2e": {"value": e2e_seg / e2e_s, "unit": "segments/s", "h2d_bytes_per_step": h2d // e2e_steps,
                "d2h_bytes_per_step": d2h // e2e_steps,
                "path": "qsg_track_host (the tracking launch reads the vault from and appends the census to "
                        "pinned host arrays over the host link) + qsg_read_tallies (flux and counters D2H)",
                "staged_value": staged_seg / staged_s,
                "staged_path": "qsg_set_particles (H2D) + qsg_track_cycle + qsg_get_census (D2H) + "
                               "qsg_read_tallies on the same vaults"},
        # event-timed region: one tracking-kernel launch per step (config2 has no fission, so one pass)
        "gpu_launches": args.steps,
        "device_flags": flags,
        "clocks": clocks.summary(),
    }
    if not args.no_forms and world == 1:
        # the forms compare single-GPU paths; replica runs (N > 1) report the plain line only
        line["forms"] = {"batched": measure_batched(), "adjoint": measure_adjoint()}
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = reference_arm_baseline(args.warmup, args.steps)
    print(json.dumps(line), flush=True)
    if pg is not None:
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
