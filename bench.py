#!/usr/bin/env python
"""Benchmark of the per-step SPH interaction path on one GB300.

Workload (default): the off-axis unequal-mass collision, N = 1,000,000
(10 Msun / 4 Rsun n=3 with 600k particles + 3 Msun / 1.5 Rsun n=1.5 with 400k,
impact parameter 0.5 (R1+R2), relative speed 1.2 v_esc, ~50 neighbours),
built from seeded synthetic polytropes (no dataset is involved).

A step is one iteration of the reference's loop body — time step, predict,
density with smoothing-length iteration, EOS, tree gravity, hydro force,
correct — run by the device-resident engine as one CUDA graph.

Metric: seconds per step (lower is better), after autotuning the work shape
(n_group, item split, item order, gravity j-tile).  Beside it: pair
interactions per second counted three ways (listed in the walks' lists, also
at the reference's n_group = 256; evaluated by the kernels; inside a kernel
support), every output's error against the FP64 oracle on the same walks and
inputs, the energy drift per step, the FP64 comparator, the dominant
kernel's roofline, the end-to-end time through the C ABI with host buffers,
and the CPU oracle's time for the same step on the host cores.

    python bench.py [--gpus N --steps K --warmup W] [--impl reference]
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

# flop per pair, counted from the reference's GPU kernels (add/mul/cmp/select
# = 1, fma = 2, rsqrt/sqrt/rcp = 1): density 132 (3 x 23 + 63, four passes),
# hydro 109, gravity 29.
FLOP_PER_PAIR = {"density": 132.0, "hydro": 109.0, "gravity": 29.0}
# per evaluated pair: one density pass, the gradient pass, a hydro pair beyond
# both supports (signal-velocity terms only, hdr_hydro.hpp:348-372)
FLOP_DENS_PASS, FLOP_DENS_GRAD, FLOP_HYDRO_FAR = 23.0, 63.0, 20.0
PROFILE_TRAFFIC = os.path.join(ROOT, "profiles", "traffic.json")


def tree_lists_rate(traffic_path=PROFILE_TRAFFIC, peaks_path=os.path.join(ROOT, "MEASURED_PEAKS.json")):
    """HBM rate of the tree and list build (latency-bound traversals, climbs
    and scans): the DRAM bytes over the device time of those kernels from one
    ncu capture of a force evaluation of the benchmark workload, against the
    measured HBM copy rate (6.8 TB/s fallback).  None without a capture."""
    if not os.path.exists(traffic_path):
        return None
    t = json.load(open(traffic_path)).get("tree_lists")
    if not t or not t.get("ncu_ms"):
        return None
    hbm, src = 6800.0, "fallback 6.8 TB/s (no MEASURED_PEAKS.json)"
    if os.path.exists(peaks_path):
        pk = json.load(open(peaks_path)).get("hbm_gbs")
        if pk:
            hbm, src = float(pk), "MEASURED_PEAKS.json hbm_gbs (measured copy)"
    gbs = t["dram_bytes"] / (t["ncu_ms"] * 1e-3) / 1e9
    return {"dram_bytes": t["dram_bytes"], "ncu_ms": t["ncu_ms"], "achieved_gbs": gbs, "peak_gbs": hbm,
            "frac": gbs / hbm, "peak_source": src, "groups": t.get("groups"), "source": t.get("_source")}


def log(*a):
    print(*a, file=sys.stderr, flush=True)


# ------------------------------------------------------------------ clocks
class ClockSampler:
    """nvidia-smi samples during the timed region (sm clock, throttle reasons)."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.device = device
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 7:
                self.rows.append(parts)

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.thread.join(timeout=2)
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in self.rows for k in range(4) if r[3 + k].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


# ------------------------------------------------------------------ CPU oracle
def oracle_rates(samples, nthreads, warm=True, ksr_max=0.0):
    """Times the oracle's walk-batched functors on host-built EPI/EPJ samples.

    samples: {"density": (epi, epj, i_off, j_off), "hydro": ..., "gravity": ...}
    Returns ({phase: (pairs, seconds)}, {phase: functor outputs})."""
    from oracle import oracle as orc
    out, res = {}, {}
    for phase, (epi, epj, io, jo) in samples.items():
        pairs = int(np.sum(np.diff(io) * np.diff(jo)))
        fn = {"density": lambda: orc.density_walks(io, jo, epi, epj, eta=ETA, ksr_max=ksr_max,
                                                       nthreads=nthreads),
              "hydro": lambda: orc.hydro_walks(io, jo, epi, epj, nthreads=nthreads),
              "gravity": lambda: orc.gravity_walks(io, jo, epi, epj, nthreads=nthreads)}[phase]
        if warm:
            fn()  # warm-up (page-in, thread pool)
        t = time.perf_counter()
        res[phase] = fn()[0]
        out[phase] = (pairs, time.perf_counter() - t)
    return out, res


def field_parity(a, b, floor_frac):
    """Per-particle |a - b| / max(|b|, floor_frac x max|b|) (vector norms for
    n x 3 fields): max, p99, median and the count above 1e-5."""
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    if a.ndim > 1:
        d, s_ = np.linalg.norm(a - b, axis=1), np.linalg.norm(b, axis=1)
    else:
        d, s_ = np.abs(a - b), np.abs(b)
    r = d / np.maximum(s_, max(floor_frac * s_.max(), 1e-300))
    return {"max": float(r.max()), "p99": float(np.quantile(r, 0.99)), "median": float(np.median(r)),
            "n_above_1e-5": int((r > 1e-5).sum()), "n": int(len(r)), "floor": floor_frac}


def parity_vs_oracle(ps, idx, outs, G):
    """Every output of the evaluation against the FP64 oracle run on the same
    walks, lists and inputs (the engine's exported i-groups, j-lists, tree
    monopoles and per-particle fields: the functor-level comparison)."""
    n = ps.n
    f = {k: ps.download(k, sorted_order=True) for k in
         ("dens", "ksr", "grdh", "divv", "rotv", "np", "acch", "accg1", "accg2", "acc", "udot", "vsmx", "diffu",
          "pot")}
    par = {}
    d, i = outs["density"], idx["density"]
    one = ~d["itr"].astype(bool)   # particles that finished in the first walk (all of them when converged)
    for k in ("dens", "ksr", "grdh"):
        par[k] = field_parity(f[k][i][one], d[k][one], 1e-3)
    for k in ("divv", "rotv"):
        par[k] = field_parity(f[k][i][one], d[k][one], 1e-2)
    par["np_mismatches"] = int((f["np"][i][one].astype(np.int64) != d["np"][one]).sum())
    par["density_rewalked_not_compared"] = int((~one).sum())
    h, i = outs["hydro"], idx["hydro"]
    ref = {"acch": np.zeros((n, 3)), "accg1": np.zeros((n, 3)), "accg2": np.zeros((n, 3)), "pot": np.zeros(n)}
    ref["acch"][i], ref["accg1"][i] = h["acch"], G * h["accg"]
    par["acch"] = field_parity(f["acch"][i], h["acch"], 1e-3)
    par["accg1"] = field_parity(f["accg1"][i], G * h["accg"], 1e-3)
    par["udot"] = field_parity(f["udot"][i], h["udot"], 1e-3)
    par["vsmx"] = field_parity(f["vsmx"][i], h["vsmx"], 1e-3)
    par["diffu"] = field_parity(f["diffu"][i], h["diffu"], 1e-2)
    g, i = outs["gravity"], idx["gravity"]
    ref["accg2"][i], ref["pot"][i] = G * g["acc"], G * g["pot"]
    par["accg2"] = field_parity(f["accg2"][i], G * g["acc"], 1e-3)
    par["pot"] = field_parity(f["pot"][i], G * g["pot"], 1e-3)
    a_ref = ref["acch"] + ref["accg1"] + ref["accg2"]
    par["acc_total"] = field_parity(f["acc"], a_ref, 1e-3)
    parts = (np.linalg.norm(ref["acch"], axis=1) + np.linalg.norm(ref["accg1"], axis=1)
             + np.linalg.norm(ref["accg2"], axis=1))
    r = np.linalg.norm(f["acc"] - a_ref, axis=1) / np.maximum(parts, 1e-300)
    par["acc_total_over_parts"] = {"max": float(r.max()), "p99": float(np.quantile(r, 0.99)),
                                   "median": float(np.median(r)), "n_above_1e-5": int((r > 1e-5).sum())}
    par["note"] = ("FP32C engine vs the FP64 oracle (C restatement of the reference functors, pinned to them by "
                   "golden vectors) on the engine's own walks, lists, tree monopoles and inputs; per particle "
                   "|d| / max(|ref|, floor x max|ref|) with the floor given per field (1e-2 for div v, |rot v|, "
                   "diffu); acc_total = acch + accg1 + accg2, also relative to |acch| + |accg1| + |accg2| "
                   "(the stars are near hydrostatic equilibrium: the total is a small difference of the parts)")
    return par


def combined_rate(rates, mix):
    """Interactions/s of a step with the per-phase pair mix `mix` when each
    phase runs at the measured rate."""
    t = sum(mix[p] / (rates[p][0] / rates[p][1]) for p in mix)
    return sum(mix.values()) / t


def samples_from_engine(ps, rng, frac, ksr_first):
    """EPI/EPJ arrays of a random subset of the engine's own walks, and per
    phase the sorted-order indices of their i-particles.  ksr_first: the
    smoothing lengths the evaluation started from (upload order), the density
    functor's first guess and search radius 1.1 ksr (hdr_density.hpp:376-379);
    the other phases take the evaluation's final fields."""
    from research_codes_gb300 import abi, units, walks
    n = ps.n
    f = {k: ps.download(k, sorted_order=True) for k in
         ("pos", "vel", "mass", "id", "ksr", "pres", "grdh", "dens", "bswt", "vsnd", "alph", "alphu", "uene",
          "eta")}
    f["id"] = f["id"].astype(np.int64)
    # upload index of every sorted slot, through the (unique) particle ids
    up_id = ps.download("id").astype(np.int64)
    order = np.argsort(up_id, kind="stable")
    slot = order[np.searchsorted(up_id[order], f["id"])]
    fd = dict(f, ksr=np.asarray(ksr_first)[slot])
    fd["rs"] = 1.1 * fd["ksr"]
    out, idx = {}, {}
    for kind, phase in ((0, "density"), (1, "hydro"), (2, "gravity")):
        i_first, i_count, j_off, j_idx = ps.lists(kind)
        nw = len(i_first)
        take = np.sort(rng.choice(nw, min(nw, max(4, int(nw * frac))), replace=False))
        idx[phase] = np.concatenate([np.arange(i_first[w], i_first[w] + i_count[w]) for w in take])
        items = []
        for w in take:
            gi = np.arange(i_first[w], i_first[w] + i_count[w])
            gj = j_idx[j_off[w]:j_off[w + 1]]
            if phase == "density":
                items.append((walks.density_epi(gi, fd), walks.density_epj(gj, fd)))
            elif phase == "hydro":
                items.append((walks.hydro_epi(gi, f), walks.hydro_epj(gj, f)))
            else:
                mom, neps2 = NODES
                pj, sj = gj[gj < n], gj[gj >= n] - n
                epi = walks.gravity_epi(gi, f)
                epj = np.zeros(len(gj), abi.GravityEPJ)
                epj["mass"][:len(pj)] = f["mass"][pj]
                epj["pos"][:len(pj)] = f["pos"][pj]
                epj["eps2"][:len(pj)] = (f["ksr"][pj] / units.KSRH) ** 2
                epj["mass"][len(pj):] = mom[sj, 3]
                epj["pos"][len(pj):] = mom[sj, :3]
                epj["eps2"][len(pj):] = neps2[sj]
                items.append((epi, epj))
        out[phase] = walks.concat_walks(items)
    return out, idx


# ------------------------------------------------------------------ our arm
def run_ours(args):
    import torch

    from research_codes_gb300 import functors, ic
    from research_codes_gb300.system import ParticleSystem, state_from_ic

    from research_codes_gb300 import replicas
    world, rank, local = replicas.rank_info()
    torch.cuda.set_device(local)
    replicas.init("nccl", torch.device("cuda", local))

    global ETA
    t_ic = time.time()
    s, ETA = ic.config_system(args.config, scale=args.scale, seed=replicas.replica_seed(args.seed, rank))
    s = state_from_ic(s)
    n = len(s["mass"])
    log(f"[bench] rank {rank}: {args.config} n={n} ic {time.time() - t_ic:.1f}s")

    ctx = functors.Context(device=local, precision="fp32c", eta=ETA)
    # the large collision (c4) runs its gravity with node quadrupoles
    quad = 1 if args.config == "c4" else 0
    ps = ParticleSystem(ctx, n, n_group=args.n_group, quadrupole=quad)
    ps.upload(s)
    ps.compute_forces()
    tuned = None
    if not args.no_autotune:
        # n_group (i-group size), the gravity j-tile, the item split (lanes
        # per i-particle) and the item order, by coordinate descent on the
        # device time of force evaluations of this state
        from research_codes_gb300 import autotune
        ps.compute_forces()
        best, table = autotune.autotune(ps)
        tuned = {"chosen": best, "force_ms": [{"params": p, "ms": round(ms, 3)} for p, ms in table[:8]],
                 "evaluated": len(table)}
        log(f"[bench] autotune: {best}")
    stream = torch.cuda.ExternalStream(ctx.stream())
    for _ in range(args.warmup):
        ps.step(1)
    torch.cuda.synchronize()
    st0 = ps.stats()   # energy and clock before the timed steps

    # ---- timed region: K graph-captured steps, CUDA events on the engine's stream
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    replicas.barrier()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    ps.step(args.steps)
    e1.record(stream)
    e1.synchronize()
    torch.cuda.synchronize()
    replicas.barrier()
    ms = e0.elapsed_time(e1)
    clk = clocks.stop()
    # phases of the last timed step, from the event-record nodes of its graph
    phases_graph = ps.phase_times()
    st = ps.stats()
    pairs = {"density": st["pairs_density"], "hydro": st["pairs_hydro"], "gravity": st["pairs_gravity"]}
    # energy drift of the timed steps (FP64 sums of m (v^2/2 + u + pot/2))
    energy = {"e_start": st0["e_tot"], "e_end": st["e_tot"], "steps": args.steps,
              "time_start": st0["time"], "time_end": st["time"],
              "drift_per_step": (st["e_tot"] - st0["e_tot"]) / abs(st0["e_tot"]) / args.steps}
    inter = sum(pairs.values())
    # every rank evolves its own replica: the job's pairs over the slowest rank
    rate_listed, ms = replicas.aggregate_rate(inter, ms, args.steps, device="cuda")
    ms_step = ms / args.steps
    value = ms_step * 1e-3   # s/step, the headline
    log(f"[bench] {ms_step:.2f} ms/step, {inter:.3e} pairs/step, iters {st['density_iterations']}")

    # ---- per-kernel durations: CUDA events on the engine's stream around each
    # phase of eager force evaluations of the current state (the same
    # kernels, lists and work items as inside the captured step)
    acc_t = {}
    ps.set_graph(False)
    for _ in range(args.steps):
        ps.compute_forces()
        for k, v in ps.phase_times().items():
            acc_t[k] = acc_t.get(k, 0.0) + v
    ps.set_graph(True)
    phases = {k: v / args.steps for k, v in acc_t.items()}
    st_k = ps.stats()
    # the four pair kernels and the algorithmic work of one launch: pairs x
    # flop per pair counted from the reference's GPU kernels (density 132 per
    # listed pair of the first walk, gravity 29; the hydro signal velocity 20
    # per listed pair, hdr_hydro.hpp:368-372, taken over every j of a list;
    # the rest of the hydro pair formula, 109 per pair, on the marked pairs
    # inside a support, which the double-float pass evaluates)
    kern = {"density": phases["density_kernel"], "gravity": phases["gravity_kernel"],
            "hydro_signal": phases["hydro_signal"], "hydro_df": phases["hydro_df"]}
    dom = max(kern, key=kern.get)
    peak = ctx.probe_fp32_peak()
    work = {"density": (st_k["pairs_density_first"], FLOP_PER_PAIR["density"]),
            "gravity": (st_k["pairs_gravity"], FLOP_PER_PAIR["gravity"]),
            "hydro_signal": (st_k["pairs_hydro"], FLOP_HYDRO_FAR),
            "hydro_df": (st_k["hydro_pairs_marked"], FLOP_PER_PAIR["hydro"])}
    achieved = work[dom][0] * work[dom][1] / (kern[dom] * 1e-3) / 1e12 if work[dom][0] else None
    # work the kernels actually evaluated: the density and hydro kernels drop
    # list entries beyond every i-particle's kernel support before their pair
    # loops (those pairs contribute exactly zero); gravity evaluates all
    useful_d = float(ps.download("np").sum())
    flop_eval = {"density": st_k["evals_density_first"] * FLOP_DENS_PASS + st_k["evals_density_grad"] * FLOP_DENS_GRAD,
                 "gravity": st_k["pairs_gravity"] * FLOP_PER_PAIR["gravity"],
                 "hydro_signal": (st_k["evals_hydro_near"] + st_k["evals_hydro_far"]) * FLOP_HYDRO_FAR,
                 "hydro_df": st_k["hydro_pairs_marked"] * FLOP_PER_PAIR["hydro"]}
    per_kernel = {}
    for k in kern:
        per_kernel[k] = {"ms": round(kern[k], 4), "pairs": int(work[k][0]), "flop_per_pair": work[k][1],
                         "achieved_tflops": work[k][0] * work[k][1] / (kern[k] * 1e-3) / 1e12,
                         "achieved_evaluated_tflops": flop_eval[k] / (kern[k] * 1e-3) / 1e12}
    per_kernel["density"]["pair_evaluations"] = {"three_passes": int(st_k["evals_density_first"]),
                                                 "gradient_pass": int(st_k["evals_density_grad"]),
                                                 "useful_per_pass": int(useful_d)}
    per_kernel["hydro_signal"]["pair_evaluations"] = {"near": int(st_k["evals_hydro_near"]),
                                                      "signal_velocity_only": int(st_k["evals_hydro_far"])}
    per_kernel["hydro_df"]["rows_overflowed"] = int(st_k["hydro_rows_overflowed"])
    traffic = None
    if os.path.exists(PROFILE_TRAFFIC):
        tr = json.load(open(PROFILE_TRAFFIC))
        if dom in tr:
            traffic = tr[dom].get("bytes_per_launch")
    tree_lists = tree_lists_rate()

    # pairs per step three ways: listed (sum n_i n_j over the walks' lists at
    # n_group, the reference's work), evaluated by the kernels (list entries
    # beyond every i-particle's support are dropped before the pair loops),
    # and useful (inside a support: 4 x the neighbour counts for the density's
    # three h passes and gradient pass, the marked hydro pairs, every gravity
    # pair)
    evaluated = {"density": st["evals_density_first"] + st["evals_density_grad"],
                 "hydro": st["evals_hydro_near"] + st["evals_hydro_far"], "gravity": st["pairs_gravity"]}
    useful_d = 4.0 * float(ps.download("np").sum())
    useful = {"density": useful_d, "hydro": st["hydro_pairs_marked"], "gravity": st["pairs_gravity"]}
    listed_256 = pairs
    if ps.params.n_group != 256:
        # the listed pairs at the reference's n_group = 256 (main.cpp:380,386,394),
        # from one eager evaluation of the same state outside the timed region
        g = ps.params.n_group
        ps.set_params(n_group=256)
        ps.set_graph(False)
        ps.compute_forces()
        s256 = ps.stats()
        listed_256 = {"density": s256["pairs_density"], "hydro": s256["pairs_hydro"],
                      "gravity": s256["pairs_gravity"]}
        ps.set_params(n_group=g)
        ps.set_graph(True)
    ips = {k: world * sum(v.values()) / (ms_step * 1e-3) for k, v in
           (("listed", pairs), ("evaluated", evaluated), ("useful", useful))}
    line = {"metric": METRIC, "value": value, "unit": "s/step", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 pair math (FP32C, double-float hydro sums), "
                                                          "f64 state",
            "data": DATA, "config": workload_config(args, n),
            "interactions_per_s": ips,
            "pairs_per_step": {"listed": pairs, "listed_at_n_group_256": listed_256, "evaluated": evaluated,
                               "useful": useful, "n_group": ps.params.n_group},
            "density_walks": st["density_iterations"],
            "parallelism": "replicas" if world > 1 else "single GPU",
            "phases_ms": {k: round(v, 4) for k, v in phases.items()},
            "phases_ms_step_graph": {k: round(v, 4) for k, v in phases_graph.items()},
            "roofline": {"bound": "fp32", "kernel": dom, "achieved": achieved, "peak": peak,
                         "unit": "TFLOP/s", "frac": (achieved / peak) if achieved else None,
                         "traffic": traffic,
                         "peak_source": "FP32 FMA probe on this GPU (sph_probe_fp32_peak); "
                                        "MEASURED_PEAKS.json holds no FP32 figure",
                         "work": "achieved = pairs of one launch x flop/pair / its CUDA-event time: listed "
                                 "pairs (sum n_i*n_j) x 132 density, 29 gravity, 20 hydro signal velocity; "
                                 "marked pairs x 109 for the hydro double-float pass; per_kernel gives every "
                                 "kernel and the evaluated work",
                         "frac_evaluated": per_kernel[dom]["achieved_evaluated_tflops"] / peak,
                         "per_kernel": per_kernel},
            "tree_lists": tree_lists, "gpu_launches": None, "clocks": clk, "autotune": tuned,
            "energy": energy}

    # kernel launches in the timed region: the kernel nodes of the captured
    # step graph (CUB sort/scan kernels compiled into the library included)
    try:
        line["gpu_launches"] = args.steps * ps.graph_kernels(step=True)
    except Exception:
        # the last step re-ran eagerly (its lists outgrew the captured
        # buffers): the next step captures the graph again
        ps.step(1)
        line["gpu_launches"] = args.steps * ps.graph_kernels(step=True)

    if rank == 0 and not args.no_fp64:
        # ---- FP64 comparator: parity of one force evaluation of identical
        # state in both precisions, then the FP64 step time
        fields = ("dens", "ksr", "acch", "accg1", "accg2", "udot", "pot")
        host = {k: ps.download(k) for k in ("pos", "vel", "mass", "uene", "ksr", "alph", "alphu", "id", "istar")}
        host["id"] = host["id"].astype(np.int64)
        host["istar"] = host["istar"].astype(np.int32)
        ps.set_graph(False)
        res = {}
        for prec in ("fp32c", "fp64"):
            ctx.set_precision(prec)
            ps.upload(host)
            ps.compute_forces()
            res[prec] = {k: ps.download(k) for k in fields}
            res[prec]["stats"] = ps.stats()
        ph64 = ps.phase_times()
        ps.set_graph(True)
        f32, f64 = res["fp32c"], res["fp64"]
        ps.step(1)            # captures the FP64 graph
        torch.cuda.synchronize()
        k64 = max(1, min(args.steps, 3))
        e0.record(stream)
        ps.step(k64)
        e1.record(stream)
        e1.synchronize()
        ms64 = e0.elapsed_time(e1) / k64
        ctx.set_precision("fp32c")

        def rel(a, b, floor=1e-3):
            a, b = np.asarray(a), np.asarray(b)
            if a.ndim > 1:
                d, s_ = np.linalg.norm(a - b, axis=1), np.linalg.norm(b, axis=1)
            else:
                d, s_ = np.abs(a - b), np.abs(b)
            r = d / np.maximum(s_, floor * s_.max())
            return {"max": float(r.max()), "median": float(np.median(r)), "p99": float(np.quantile(r, 0.99))}

        line["fp64"] = {"ms_per_step": ms64, "speedup_fp32c_over_fp64": ms64 / ms_step,
                        "phases_ms": {k: round(v, 3) for k, v in ph64.items()}}
        par = {k: rel(f32[k], f64[k], 1e-2 if k == "accg1" else 1e-3) for k in fields}
        for k in fields:
            a_, b_ = np.asarray(f32[k]), np.asarray(f64[k])
            d_ = np.linalg.norm(a_ - b_, axis=1) if a_.ndim > 1 else np.abs(a_ - b_)
            s_ = np.linalg.norm(b_, axis=1) if b_.ndim > 1 else np.abs(b_)
            floor = (1e-2 if k == "accg1" else 1e-3) * s_.max()
            par[k]["n_above_1e-5"] = int((d_ / np.maximum(s_, floor) > 1e-5).sum())
            par[k]["normwise"] = float(np.linalg.norm(a_ - b_) / max(np.linalg.norm(b_), 1e-300))
        par["density_rechecked_fp64"] = int(f32["stats"]["density_rechecked"])
        par["same_density_walks"] = f32["stats"]["density_iterations"] == f64["stats"]["density_iterations"]
        par["note"] = ("per-particle |d|/max(|ref|, floor), floor 1e-3 of the field max (1e-2 for the "
                       "softening correction accg1); the total acceleration is compared by parts")
        line["parity_fp32c_vs_fp64"] = par
        log(f"[bench] fp64 {ms64:.1f} ms/step (x{ms64 / ms_step:.1f})")

    if rank == 0 and not args.no_e2e:
        # ---- end to end through the C ABI with host buffers: per step the
        # converged particle state goes up from pinned host memory, the forces
        # are evaluated (density, EOS, gravity, hydro), acc and du/dt come back.
        host = {k: ps.download(k) for k in ("pos", "vel", "mass", "uene", "ksr", "alph", "alphu", "id", "istar")}
        host["id"] = host["id"].astype(np.int64)
        host["istar"] = host["istar"].astype(np.int32)
        pin = {k: torch.from_numpy(np.ascontiguousarray(v)).pin_memory().numpy() for k, v in host.items()}
        out_acc = torch.empty((n, 3), dtype=torch.float64).pin_memory().numpy()
        out_udot = torch.empty(n, dtype=torch.float64).pin_memory().numpy()
        h2d = sum(pin[k].nbytes for k in pin)
        d2h = out_acc.nbytes + out_udot.nbytes
        ke = max(1, min(args.steps, 5))
        ps.upload(pin)
        ps.compute_forces()            # captures the force-evaluation graph
        torch.cuda.synchronize()
        t = time.perf_counter()
        for _ in range(ke):
            ps.upload(pin)
            ps.compute_forces()
            ps.download("acc", out=out_acc)
            ps.download("udot", out=out_udot)
        el = time.perf_counter() - t
        # every timed evaluation is of the same uploaded state: its pairs
        ste = ps.stats()
        pairs_e = ke * (ste["pairs_density"] + ste["pairs_hydro"] + ste["pairs_gravity"])
        line["e2e"] = {"value": el / ke, "unit": "s/step", "h2d_bytes_per_step": int(h2d),
                       "d2h_bytes_per_step": int(d2h), "ms_per_step": 1e3 * el / ke,
                       "interactions_per_s": pairs_e / el, "density_walks": ste["density_iterations"],
                       "path": "sph_system_upload -> sph_system_compute_forces -> sph_system_download "
                               "(pinned host buffers, converged state)"}

    if rank == 0 and not args.no_cpu:
        # ---- CPU oracle (port) on the host cores, bounded sample of this workload's walks
        global NODES
        ksr_first = ps.download("ksr")   # the density iteration's first guess
        ps.compute_forces()   # eager evaluation: every list is exported as used
        NODES = ps.nodes()
        rng = np.random.default_rng(1)
        smp, idx = samples_from_engine(ps, rng, args.cpu_frac, ksr_first)
        nthreads = os.cpu_count() or 1
        ksr_max = ps.stats()["ksr_max"]   # this evaluation's cap (the star separation for two stars)
        rates, outs = oracle_rates(smp, nthreads, ksr_max=ksr_max if np.isfinite(ksr_max) else 0.0)
        cpu_rate = combined_rate(rates, {k: float(v) for k, v in pairs.items()})
        cpu_s = sum(float(pairs[p]) / (rates[p][0] / rates[p][1]) for p in pairs)   # this step's pairs
        if args.cpu_frac >= 1.0:
            line["parity_vs_oracle"] = parity_vs_oracle(ps, idx, outs, ps.params.G)
        line["cpu_baseline"] = {"value": cpu_s, "unit": "s/step", "interactions_per_s": cpu_rate,
                                "cores": nthreads, "kind": "port",
                                "sample": f"{args.cpu_frac:.1%} of the walks of each phase of this step "
                                          f"({', '.join(f'{k} {v[0]:.2e} pairs in {v[1]:.1f}s' for k, v in rates.items())}); "
                                          "scalar FP64 C restatement of the reference functors, OpenMP over walks; "
                                          "tree/list construction not included"}
    ps.close()
    ctx.close()
    if rank == 0:
        print(json.dumps(line), flush=True)
    replicas.finalize()


# ------------------------------------------------------------------ reference arm
def tree_groups(keys, n_group):
    """i-groups as FDPS forms them: the cells of an octree over the Morton
    order (keys sorted) holding at most n_group particles, each a contiguous
    index range; returns a list of index arrays in key order."""
    keys = np.asarray(keys, np.uint64)
    out, stack = [], [(0, len(keys), 0)]
    while stack:
        a, b, level = stack.pop()
        if b - a <= n_group or level >= 21:
            out.append((a, b))
            continue
        shift = 3 * (20 - level)
        base = (int(keys[a]) >> (shift + 3)) << (shift + 3)
        cuts = [a] + [a + int(np.searchsorted(keys[a:b], np.uint64(base | (o << shift)))) for o in range(1, 8)] + [b]
        for o in range(7, -1, -1):
            if cuts[o + 1] > cuts[o]:
                stack.append((cuts[o], cuts[o + 1], level + 1))
    return [np.arange(a, b) for a, b in sorted(out)]


def _group_ranges(groups):
    gf = np.array([g[0] for g in groups], np.int64)
    gc = np.array([len(g) for g in groups], np.int64)
    return gf, gc


def host_walks_density(s, keys, groups, rs, active, nthreads):
    """Gather lists (hdr_density.hpp:389-397; FDPS's Gather search): for each
    group with iterating particles, every j within the largest search radius
    of those particles from the group's bounding box (host octree,
    oracle_neighbour_lists).  Returns EPI/EPJ walk arrays and the i-particle
    indices, in walk order."""
    from oracle import oracle as orc
    from research_codes_gb300 import walks
    gf, gc = _group_ranges(groups)
    owner = np.repeat(np.arange(len(groups)), gc)
    gr = np.full(len(groups), -1.0)
    np.maximum.at(gr, owner[active], rs[active])
    off, idx = orc.neighbour_lists(keys, s["pos"], s["ksr"], gf, gc, gr, 0, 8, nthreads)
    keep = gr >= 0.0
    i_idx = np.flatnonzero(active)                       # group order = index order
    i_off = np.concatenate([[0], np.cumsum(np.bincount(owner[active], minlength=len(groups))[keep])])
    j_off = np.concatenate([[0], np.cumsum(np.diff(off)[keep])])
    epi = walks.density_epi(i_idx, s, rs)
    epj = walks.density_epj(idx, s)
    return (epi, epj, i_off.astype(np.int64), j_off.astype(np.int64)), i_idx


def host_walks_hydro(s, keys, groups, nthreads):
    """Symmetric lists (main.cpp:336-344; FDPS's Symmetry search): every j
    within max(max_{i in g} h_i, h_j) of the group's bounding box."""
    from oracle import oracle as orc
    from research_codes_gb300 import walks
    gf, gc = _group_ranges(groups)
    gr = np.maximum.reduceat(s["ksr"], gf)
    off, idx = orc.neighbour_lists(keys, s["pos"], s["ksr"], gf, gc, gr, 1, 8, nthreads)
    i_off = np.concatenate([[0], np.cumsum(gc)])
    epi = walks.hydro_epi(np.arange(len(s["mass"])), s)
    return epi, walks.hydro_epj(idx, s), i_off.astype(np.int64), off.astype(np.int64)


def host_walks_gravity(s, keys, groups, theta, nthreads):
    """theta-criterion group walk of a host octree (oracle_gravity_lists; the
    role of FDPS's TreeForForceLong walk, hdr_gravity.hpp:385-402): particle
    entries as GravityEPJ, accepted nodes' monopoles as GravitySPJ (same
    layout) after them."""
    from oracle import oracle as orc
    from research_codes_gb300 import abi, units, walks
    eps2 = (s["ksr"] / units.KSRH) ** 2
    gf = np.array([g[0] for g in groups], np.int64)
    gc = np.array([len(g) for g in groups], np.int64)
    ep_off, ep_idx, sp_off, sp_idx, mom, neps2 = orc.gravity_tree_lists(keys, s["pos"], s["mass"], eps2, gf, gc,
                                                                        theta, 8, nthreads)
    items = []
    for k, g in enumerate(groups):
        e = ep_idx[ep_off[k]:ep_off[k + 1]]
        sp = sp_idx[sp_off[k]:sp_off[k + 1]]
        epj = np.zeros(len(e) + len(sp), abi.GravityEPJ)
        epj["mass"][:len(e)], epj["pos"][:len(e)], epj["eps2"][:len(e)] = s["mass"][e], s["pos"][e], eps2[e]
        epj["mass"][len(e):], epj["pos"][len(e):], epj["eps2"][len(e):] = mom[sp, 3], mom[sp, :3], neps2[sp]
        items.append((walks.gravity_epi(g, s), epj))
    return walks.concat_walks(items)


def host_force_evaluation(s, keys, groups, nthreads, theta=0.5, cache=None):
    """One calcSPHKernel (main.cpp:300-358) on the host: the density with its
    search-radius re-walks (hdr_density.hpp:372-415), EOS and Balsara switch,
    tree gravity and the hydro force, every functor the oracle's (OpenMP over
    walks), every list the host's.  Updates s in place; returns the functor
    seconds and listed pairs per phase and the density walks.  `cache`
    (a dict) keeps the walk arrays of the first call for later calls on the
    same state, which then time the functors alone."""
    from oracle import oracle as orc
    from research_codes_gb300 import units
    reuse = cache is not None and "density" in cache
    n = len(s["mass"])
    sec = {"density": 0.0, "gravity": 0.0, "hydro": 0.0}
    pairs = {"density": 0, "gravity": 0, "hydro": 0}
    h0 = s["ksr"].copy()
    rs = 1.1 * h0
    active = np.ones(n, bool)
    walks_d = 0
    while active.any():
        if reuse:
            (epi, epj, io, jo), idx = cache["density"][walks_d]
        else:
            (epi, epj, io, jo), idx = host_walks_density(dict(s, ksr=h0), keys, groups, rs, active, nthreads)
            if cache is not None:
                cache.setdefault("density_build", []).append(((epi, epj, io, jo), idx))
        t = time.perf_counter()
        out, _ = orc.density_walks(io, jo, epi, epj, eta=ETA, nthreads=nthreads)
        sec["density"] += time.perf_counter() - t
        pairs["density"] += int(np.sum(np.diff(io) * np.diff(jo)))
        walks_d += 1
        done = ~out["itr"].astype(bool)
        for k in ("dens", "divv", "rotv", "grdh", "ksr"):
            s[k][idx[done]] = out[k][done]
        active[idx[done]] = False
        rs[idx[~done]] *= 1.1
        if walks_d >= 20 or (reuse and walks_d >= len(cache["density"])):
            break
    if cache is not None and not reuse:
        cache["density"] = cache.pop("density_build", [])
    s["pres"], s["vsnd"] = orc.eos(s["dens"], s["uene"])
    s["bswt"] = orc.balsara(s["divv"], s["rotv"], s["vsnd"], s["ksr"])
    if reuse:
        epi, epj, io, jo = cache["gravity"]
    else:
        epi, epj, io, jo = host_walks_gravity(s, keys, groups, theta, nthreads)
        if cache is not None:
            cache["gravity"] = (epi, epj, io, jo)
    t = time.perf_counter()
    gout, _ = orc.gravity_walks(io, jo, epi, epj, nthreads=nthreads)
    sec["gravity"] += time.perf_counter() - t
    pairs["gravity"] = int(np.sum(np.diff(io) * np.diff(jo)))
    gi = np.concatenate(groups)
    s["eta"] = np.empty(n)
    s["eta"][gi] = s["ksr"][gi] ** 2 / units.KSRH ** 2 * s["grdh"][gi] / (3.0 * s["dens"][gi]) * gout["eta"]
    if reuse:
        epi, epj, io, jo = cache["hydro"]
    else:
        epi, epj, io, jo = host_walks_hydro(s, keys, groups, nthreads)
        if cache is not None:
            cache["hydro"] = (epi, epj, io, jo)
    t = time.perf_counter()
    orc.hydro_walks(io, jo, epi, epj, nthreads=nthreads)
    sec["hydro"] += time.perf_counter() - t
    pairs["hydro"] = int(np.sum(np.diff(io) * np.diff(jo)))
    return sec, pairs, walks_d


def run_reference(args):
    """The reference's CPU functors for this path, timed on the host cores.

    The reference tree is not available at run time and its compiled
    functors are x86-only here, so the timed code is the oracle's C
    restatement of the reference's scalar FP64 functors (kind "port"), pinned
    to them by the golden vectors.  A step is one force evaluation
    (calcSPHKernel) of the same configuration: the density with its
    search-radius re-walks over every i-group, EOS and Balsara switch, theta
    = 0.5 tree gravity and the hydro force, on lists the host builds (groups
    of n_group Morton-ordered particles, KD-tree gather and symmetric lists, a
    host octree walk for gravity).  The state is the configuration's initial
    conditions after one evaluation (so the timed one starts from converged
    smoothing lengths, as the GPU arm's steps do).  ms_per_step is the wall
    time of the functor calls of a step; FDPS's tree and list construction has
    no counterpart here and is not included."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from research_codes_gb300 import ic, walks
    from research_codes_gb300.system import state_from_ic

    global ETA
    s, ETA = ic.config_system(args.config, scale=args.scale, seed=args.seed)
    s = state_from_ic(s)
    n = len(s["mass"])
    keys = walks.morton_keys(s["pos"])
    order = np.argsort(keys, kind="stable")
    keys = keys[order]
    s = {k: (np.asarray(v)[order].copy() if np.ndim(v) > 0 and len(v) == n else v) for k, v in s.items()}
    for k in ("dens", "divv", "rotv", "grdh"):
        s[k] = np.zeros(n)
    groups = tree_groups(keys, args.n_group)
    nthreads = os.cpu_count() or 1
    t0 = time.perf_counter()
    host_force_evaluation(s, keys, groups, nthreads)   # from the initial guess of h
    # the evaluation every step repeats: lists built once (not timed), the
    # functors of every walk timed per step
    cache = {}
    host_force_evaluation({k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in s.items()}, keys, groups,
                          nthreads, cache=cache)
    log(f"[bench/ref] set-up evaluations {time.perf_counter() - t0:.1f}s")
    for _ in range(args.warmup):
        host_force_evaluation({k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in s.items()}, keys,
                              groups, nthreads, cache=cache)
    secs = []
    for _ in range(args.steps):
        st = {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in s.items()}
        sec, pairs, walks_d = host_force_evaluation(st, keys, groups, nthreads, cache=cache)
        secs.append(sum(sec.values()))
    value = float(np.mean(secs))   # s/step
    ms_step = 1e3 * value
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "s/step", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": DATA,
            "config": workload_config(args, n),
            "interactions_per_s": {"listed": float(sum(pairs.values()) / value)},
            "pairs_per_step": {"listed": pairs}, "density_walks": walks_d, "n_group": args.n_group,
            "phases_s": {k: round(v, 3) for k, v in sec.items()},
            "cpu_baseline": {"value": value, "unit": "s/step", "cores": nthreads, "kind": "port",
                             "sample": f"every walk of one force evaluation per step ({len(groups)} octree groups "
                                       f"of <= {args.n_group}; density {pairs['density']:.2e}, hydro "
                                       f"{pairs['hydro']:.2e}, gravity {pairs['gravity']:.2e} pairs); scalar FP64 C "
                                       "restatement of the reference functors, OpenMP over walks; host-built "
                                       "lists (KD-tree gather/symmetric, octree theta = 0.5); list construction "
                                       "not timed"},
            "e2e": {"value": value, "unit": "s/step", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


METRIC = "s/step of the SPH interaction path (density+EOS+gravity+hydro), N=1M collision"
DATA = "synthetic seeded polytropes (ic.config_system)"


def workload_config(args, n):
    """The config dict of both arms' lines (the workload, not the machine)."""
    big = n >= 500_000
    return {"workload": f"{args.config}: {WORKLOADS.get(args.config, args.config)}, N={n}, theta=0.5, eta={ETA}",
            "n_particles": n,
            "l2": ("inputs larger than L2 (particle state + lists ~2 kB per particle, 2 GB at N=1M)" if big else
                   "inputs smaller than L2 (a test-size configuration)")}


ETA = 1.18
NODES = None
# what each configuration of ic.config_system is
WORKLOADS = {"c0": "single n=1.5 polytrope (1 Msun, 1 Rsun)",
             "c1": "head-on collision of two n=3 polytropes (2 x 10 Msun, 4 Rsun)",
             "c2": "off-axis unequal-mass collision",
             "c3": "head-on collision of two n=3 polytropes (2 x 10 Msun, 4 Rsun)",
             "c4": "off-axis unequal-mass collision, quadrupole gravity"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="c2")
    ap.add_argument("--scale", type=float, default=1.0)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--n-group", type=int, default=256)
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--cpu-frac", type=float, default=1.0)
    args = ap.parse_args()
    if args.warmup < 3:
        log("[bench] warm-up raised to 3 steps")
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
