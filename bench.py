"""Benchmark: particle-steps/s of the GB300 DEM step engine.

Default workload: the single large system (3D bidisperse spheres,
N = 1,048,576, radii 0.5/0.7, periodic box at packing fraction 0.55,
linear spring k = 1e3, velocity Verlet, dt = 5e-4), synthetic and seeded.

  value     particle-steps/s with the state resident in HBM, CUDA events on
            the engine's stream around graph-captured 50-step chunks; L2 is
            flushed (256 MB write) between timed chunks.
  e2e       the same metric through the C ABI with host buffers: pinned host
            upload, K steps, host download inside the timed region.
  roofline  the fused force/integrate kernel: 80 B per particle-step (3D
            state record read + write) over its average launch duration,
            measured in an instrumented pass with per-launch CUDA events.
  cpu_baseline  the C/OpenMP restatement of the reference step on the host
            cores, on a bounded sample of steps of the same workload.

``--impl reference`` times that CPU restatement alone (the reference is a
JAX program that cannot be installed here).  Under torchrun with N > 1 each
rank runs an independent replica (the path has no exchange step).
"""

from __future__ import annotations

import argparse
import json
import os
import shutil
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

BYTES_PER_PARTICLE_STEP = {3: 80, 2: 56}
RESORT_RECORD_BYTES = 64  # per slot, read and written once per re-sort (k_gather)
CHUNK = 50
E2E_REPS = 5  # timed repetitions of the end-to-end call sequence (median reported)


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=200)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--workload", default="c2", choices=["c1", "c2", "c3", "c4"])
    p.add_argument("--no-batched", action="store_true", help="skip the batched mixed-size summary")
    p.add_argument("--no-served", action="store_true", help="skip the serving summary")
    p.add_argument("--no-rollout", action="store_true", help="skip the trajectory-streaming summary")
    p.add_argument("--frame-stride", type=int, default=10, help="steps between saved rollout frames")
    p.add_argument("--serve-requests", type=int, default=2000, help="window of the request stream served")
    p.add_argument("--serve-baseline", type=int, default=40,
                   help="requests of the window, evenly spaced, served one at a time (baseline)")
    p.add_argument("--no-tune", action="store_true", help="skip the skin autotuner")
    p.add_argument("--plain-sample", type=int, default=192, help="systems timed one at a time (batched baseline)")
    p.add_argument("--graph-mode", type=int, default=0, choices=[0, 1, 2],
                   help="0 conditional re-sort nodes, 1 plain graphs (profilers see every kernel), 2 no graphs")
    p.add_argument("--skin", type=float, default=None)
    p.add_argument("--prune-skin", type=float, default=0.0,
                   help="inner-list margin of the Verlet-list dynamic pruning (0: skin / 3, < 0: off)")
    p.add_argument("--brick", type=int, default=0,
                   help="particles per list-build brick (0: 240, 60 at most 32768 particles)")
    p.add_argument("--force-block", type=int, default=0, help="threads per block of k_force (0: 128)")
    p.add_argument("--small-lanes", type=int, default=0, help="lanes per slot at <= 32768 particles (0: 8)")
    p.add_argument("--n", type=int, default=None, help="override particle count (testing only)")
    p.add_argument("--cpu-seconds", type=float, default=15.0)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    return p.parse_args()


def make_workload(name, n, rank):
    from jaxdem_gb300 import workloads as W

    seed_off = 1000 * rank
    if name == "c1":
        return W.c1(**({"N": n} if n else {}), seed=1 + seed_off)
    if name == "c2":
        return W.c2(**({"N": n} if n else {}), seed=2 + seed_off)
    return W.c3(**({"N": n} if n else {}), seed=3 + seed_off)


def describe(w):
    return {
        "c1": "3D monodisperse spheres N={N} r=0.5 periodic phi=0.40 dt=1e-3",
        "c2": "3D bidisperse spheres N={N} r=0.5/0.7 periodic phi=0.55 dt=5e-4",
        "c3": "2D polydisperse disks N={N} r~U[0.4,0.6] reflect phi=0.70 gravity -y dt=5e-4",
    }[w.name].format(N=w.N)


# ------------------------------------------------------------------ clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.rows = []
        self.proc = None
        self.th = None

    def start(self):
        exe = shutil.which("nvidia-smi")
        if not exe:
            return
        self.proc = subprocess.Popen([exe, f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                                      "--format=csv,noheader,nounits", "-lms", "100"],
                                     stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)

        def rd():
            for line in self.proc.stdout:
                self.rows.append([x.strip() for x in line.split(",")])

        self.th = threading.Thread(target=rd, daemon=True)
        self.th.start()

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.th:
            self.th.join(timeout=2)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
            except (ValueError, IndexError):
                continue
            for k, nm in enumerate(names):
                if len(r) > 5 + k and r[5 + k].lower() == "active":
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------- CPU baseline
def cpu_baseline(w, seconds, max_steps=1000):
    """C/OpenMP restatement of the reference step on the host cores."""
    import oracle

    threads = oracle.max_threads()
    pos, vel, frc = w.pos.copy(), w.vel.copy(), np.zeros_like(w.pos)
    kw = dict(domain=w.domain, box=w.box_size, anchor=w.anchor, dt=w.dt, cell_size=2 * float(w.rad.max()),
              gravity=w.gravity, restitution=w.restitution, threads=threads)
    oracle.c_step(w.dim, pos, vel, frc, w.rad, w.mass, steps=1, **kw)  # warm-up
    steps, t0 = 0, time.perf_counter()
    while steps < max_steps:
        oracle.c_step(w.dim, pos, vel, frc, w.rad, w.mass, steps=1, **kw)
        steps += 1
        if time.perf_counter() - t0 > seconds:
            break
    dt = time.perf_counter() - t0
    return {"value": w.N * steps / dt, "unit": "particle-steps/s", "cores": threads, "kind": "port",
            "sample": f"{steps} steps of the same {w.N}-particle workload (C/OpenMP restatement of the "
                      f"reference step, float32), {dt:.1f} s"}


def run_reference(args, rank, world):
    if rank != 0:
        return
    w = make_workload(args.workload, args.n, 0)
    per_step = []
    for _ in range(args.warmup):
        cpu_baseline(w, seconds=0.0, max_steps=1)
    res = cpu_baseline(w, seconds=max(5.0, args.cpu_seconds), max_steps=max(args.steps, 1))
    val = res["value"]
    line = {"metric": "particle-steps/s", "value": val, "unit": "particle-steps/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": w.N / val * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "impl": "reference",
            "config": {"workload": describe(w), "N": w.N},
            "cpu_baseline": {"value": val, "unit": "particle-steps/s", "cores": res["cores"], "kind": res["kind"],
                             "sample": res["sample"]},
            "e2e": {"value": val, "unit": "particle-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# -------------------------------------------------------------- ours
def traffic_from_profile(workload, n, skin, pruning, prune_frac, prune_skin=0.0):
    """DRAM bytes per fused-kernel launch from the committed ncu captures
    (profiles/k_force_<workload>_traffic.json), when one was taken on this workload's
    size, skin (within 5 %) and pruning setting (with pruning, the capture of the
    nearest prune skin): the inner- and prune-pass figures weighted by the fraction
    of prune passes.  Returns (bytes, capture) or (None, None)."""
    p = ROOT / "profiles" / f"k_force_{workload}_traffic.json"
    try:
        d = json.loads(p.read_text())
    except Exception:
        return None, None
    if d.get("n") != n:
        return None, None
    cands = [c for c in d.get("captures", [])
             if abs(float(c["skin"]) - float(skin)) <= 0.05 * float(skin) and bool(c["pruning"]) == bool(pruning)]
    if not cands:
        return None, None
    if pruning:
        c = min(cands, key=lambda c: abs(float(c.get("prune_skin", 0.0)) - float(prune_skin)))
        return prune_frac * c["prune_pass_bytes"] + (1.0 - prune_frac) * c["inner_pass_bytes"], c
    return cands[0]["full_pass_bytes"], cands[0]


def l2_hit_from(capture, pruning, prune_frac):
    """L2 sector hit rate (lts__t_sector_hit_rate.pct) of the same capture as the traffic,
    the two passes weighted like the bytes; None when the capture did not record it."""
    if not capture:
        return None
    if pruning and "inner_pass_l2_hit_pct" in capture:
        return prune_frac * capture["prune_pass_l2_hit_pct"] + (1.0 - prune_frac) * capture["inner_pass_l2_hit_pct"]
    return capture.get("full_pass_l2_hit_pct")


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def run_ours(args, rank, world, dist):
    import torch

    from jaxdem_gb300 import replicas
    from jaxdem_gb300 import workloads as W
    from jaxdem_gb300._lib import Engine, host_register, host_unregister

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    from jaxdem_gb300 import autotune

    w = make_workload(args.workload, args.n, rank)
    young = np.array([[W.K_SPRING]], np.float32)
    rmax = float(w.rad.max())
    tuning = None
    prune_skin, brick = args.prune_skin, args.brick
    block, lanes = args.force_block, args.small_lanes
    if args.skin is not None:
        skin = args.skin
    elif args.no_tune:
        skin = autotune.default_skin(rmax)
    else:
        def mk(**shape):
            return Engine(w.dim, [w.desc()], young, chunk_steps=CHUNK, device=dev, **shape)

        best, timings = autotune.tune_shapes(mk, lambda e: e.upload(pos=w.pos, rad=w.rad, mass=w.mass, vel=w.vel),
                                             rmax, w.N, key=autotune.workload_key(w))
        skin, prune_skin, brick = best["skin"], best["prune_skin"], best["brick_particles"]
        block, lanes = best["force_block"], best["small_lanes"]
        tuning = {"skin_over_rmax": round(skin / rmax, 3),
                  "prune_skin_over_skin": round(prune_skin / skin, 3) if prune_skin > 0 else "off",
                  "brick_particles": brick, "force_block": block, "small_lanes": lanes,
                  "ms_per_step": {shape: {k: round(v * 1e3, 4) for k, v in t.items()}
                                  for shape, t in timings.items() if t}}
    shape_kw = dict(prune_skin=prune_skin, brick_particles=brick, force_block=block, small_lanes=lanes)
    eng = Engine(w.dim, [w.desc()], young, skin=skin, chunk_steps=CHUNK, device=dev, graph_mode=args.graph_mode,
                 **shape_kw)
    eng.upload(pos=w.pos, rad=w.rad, mass=w.mass, vel=w.vel)
    stream = torch.cuda.ExternalStream(eng.stream(), device=dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{dev}")

    K = args.steps
    chunks = [CHUNK] * (K // CHUNK) + ([K % CHUNK] if K % CHUNK else [])
    # warm-up steps: the first re-sort, then one call of every chunk length the timed
    # region runs, so that every CUDA graph it launches is captured and instantiated
    # before the first timing event (a call of c steps launches the graphs of c - 1
    # steps and of the final step)
    for _ in range(max(args.warmup, 1)):
        eng.step(1)
    for c in sorted(set(chunks)):
        eng.step(c)
    graphs_before = eng.stats()["graphs"]
    torch.cuda.synchronize()
    st0 = eng.stats()
    rebuilds_before, prunes_before = st0["rebuilds"], st0["prunes"]
    if dist is not None:
        dist.barrier()
    clocks = ClockSampler(dev)
    clocks.start()
    time.sleep(0.3)
    total_ms = 0.0
    for c in chunks:
        flush.fill_(float(c))
        torch.cuda.synchronize()
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record(stream)
        eng.step_async(c)
        e.record(stream)
        e.synchronize()
        total_ms += s.elapsed_time(e)
    eng.sync()
    torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    clk = clocks.stop()
    total_ms = replicas.max_over_ranks(dist, total_ms, device=f"cuda:{dev}")
    stats = eng.stats()
    # no graph may be captured inside the timed region
    graphs_captured_timed = stats["graphs"] - graphs_before

    # instrumented pass: per-launch events around the fused force kernel
    prunes0 = eng.stats()["prunes"]
    tot_ms, force_ms = eng.step_timed(CHUNK)
    prune_frac = (eng.stats()["prunes"] - prunes0) / CHUNK
    force_avg_ms = force_ms / CHUNK
    B = BYTES_PER_PARTICLE_STEP[w.dim]
    peak, peak_kind = peaks()
    achieved = B * w.N / (force_avg_ms * 1e-3) / 1e9
    pruning = stats["prunes"] > 0
    traffic, capture = traffic_from_profile(args.workload, w.N, skin, pruning, prune_frac,
                                            prune_skin if prune_skin > 0 else skin / 3.0)

    # Secondary figures: the whole step against the same roofline; the step with the re-sort
    # traffic counted (a re-sort reads and writes each slot's record: position and velocity
    # 16 B each, tag, original index and cell key 4 B each, wrapped position 16 B and image
    # 4 B, i.e. 64 B); and contact pairs evaluated per second.
    step_roof, contacts = {}, None
    try:
        pss = w.N * K / (total_ms * 1e-3)
        rs = (stats["rebuilds"] - rebuilds_before) / K
        b_incl = B + 2 * RESORT_RECORD_BYTES * rs
        step_roof = {"step_achieved": pss * B / 1e9, "step_frac": pss * B / 1e9 / peak,
                     "incl_binning": {"bytes_per_unit": b_incl, "achieved": pss * b_incl / 1e9,
                                      "frac": pss * b_incl / 1e9 / peak, "resorts_per_step": rs,
                                      "record_bytes": RESORT_RECORD_BYTES}}
        npairs = int(len(eng.contacts()))
        contacts = {"pairs": npairs, "pairs_per_s": npairs * pss / w.N,
                    "note": "contact pairs (|r_ij| < r_i + r_j) of the state after the timed steps"}
    except Exception as ex:  # secondary figures never cost the bench line
        step_roof = {"secondary_error": str(ex)[:200]}

    # end to end through the C ABI with pinned host buffers
    e2e = None
    if not args.no_e2e:
        host = {k: np.ascontiguousarray(getattr(w, k).copy()) for k in ("pos", "vel", "rad", "mass")}
        outb = {"pos_c": np.empty_like(w.pos), "vel": np.empty_like(w.vel), "force": np.empty_like(w.pos)}
        for a in list(host.values()) + list(outb.values()):
            host_register(a)
        e2e_eng = Engine(w.dim, [w.desc()], young, skin=skin, chunk_steps=CHUNK, device=dev, **shape_kw)
        e2e_eng.upload(pos=host["pos"], rad=host["rad"], mass=host["mass"], vel=host["vel"])
        e2e_eng.step(K)  # the timed call sequence once: every graph it launches is captured here
        e2e_graphs = e2e_eng.stats()["graphs"]
        torch.cuda.synchronize()
        # the whole call sequence, E2E_REPS times; the median is reported (one sample is
        # exposed to host-side jitter of a few milliseconds against a 2-3 ms sequence)
        samples = []
        for _ in range(E2E_REPS):
            t0 = time.perf_counter()
            e2e_eng.upload(pos=host["pos"], rad=host["rad"], mass=host["mass"], vel=host["vel"])
            e2e_eng.step(K)
            e2e_eng.download(outb)
            samples.append(time.perf_counter() - t0)
        e2e_s = float(np.median(samples))
        e2e_new_graphs = e2e_eng.stats()["graphs"] - e2e_graphs
        for a in list(host.values()) + list(outb.values()):
            host_unregister(a)
        e2e_eng.close()
        h2d = sum(a.nbytes for a in host.values())
        d2h = sum(a.nbytes for a in outb.values())
        e2e = {"value": world * w.N * K / e2e_s, "unit": "particle-steps/s",
               "h2d_bytes_per_step": h2d / K, "d2h_bytes_per_step": d2h / K,
               "graphs_captured_in_timed_region": e2e_new_graphs,
               "samples_s": [round(x, 6) for x in samples],
               "note": f"one C-ABI call sequence per {K} steps: upload (pinned host), step, download; "
                       f"median of {E2E_REPS} sequences"}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(w, args.cpu_seconds)

    value = replicas.aggregate_throughput([w.N * K] * world, total_ms * 1e-3)
    # per step call of c steps: k_pre + k_fin, then the graph of c - 1 steps and the graph of
    # the final step; per re-sort: the sort kernels (6, or 8 above 65,536 cells) + the list
    # build.  Per-step graphs: k_cond each, k_force + k_fin per step.  Many-step graphs (small
    # systems): k_multi_init, then per while iteration (one to start, one after each re-sort)
    # the sort kernels, the list build and k_multi.
    rebuilds_timed = stats["rebuilds"] - rebuilds_before
    # the cell scan is one kernel up to 65,536 cells, else three
    sort_k = 6 if stats["n_cells"] <= 65536 else 8
    if stats.get("many_step"):
        launches = sum(2 + 1 + (sort_k + 2) + 3 for c in chunks) + (sort_k + 2) * rebuilds_timed
    else:
        launches = sum(2 + 1 + 2 * (c - 1) + 3 for c in chunks) + (sort_k + 1) * rebuilds_timed
    line = {
        "metric": "particle-steps/s", "value": value, "unit": "particle-steps/s", "n_gpus": world,
        "steps": K, "warmup": args.warmup, "ms_per_step": total_ms / K, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": describe(w), "N": w.N, "skin": skin, "autotune": tuning, "chunk_steps": CHUNK,
                   "graph_mode": ["conditional re-sort nodes", "plain graphs", "direct launches"][args.graph_mode],
                   "l2": "flushed (256 MB write) between timed 50-step chunks",
                   "parallelism": "replicas" if world > 1 else "single",
                   "resorts_in_timed_region": rebuilds_timed,
                   "graphs_captured_in_timed_region": graphs_captured_timed,
                   "prune_skin": "off" if prune_skin < 0 else (prune_skin or skin / 3.0),
                   "brick_particles": brick or (240 if w.N > 32768 else 60),
                   "force_block": block or 128, "small_lanes": lanes or 8,
                   "prunes_in_timed_region": stats["prunes"] - prunes_before,
                   "verlet_list": {"capacity": stats["list_capacity"], "tiles": stats["list_tiles"],
                                   "regrowths": stats["list_regrowths"]}},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic, "peak_kind": peak_kind,
                     "traffic_source": (f"ncu capture at skin {capture['skin']}, pruning "
                                        f"{'on' if capture['pruning'] else 'off'}"
                                        f"{', prune skin ' + str(capture['prune_skin']) if capture['pruning'] else ''}"
                                        f", weighted by this pass's prune fraction {prune_frac:.2f} "
                                        f"({capture['source']}; kernel: {capture.get('kernel', 'unknown')})")
                     if capture else "no ncu capture at this skin and pruning setting",
                     "kernel": ("k_force_small (8 lanes a slot), timed per launch: the timed region runs the "
                                "same step inside cooperative many-step launches (k_multi)")
                     if stats.get("many_step") else "k_force (fused force + integrate)",
                     "bytes_per_unit": B,
                     "l2_hit_pct": l2_hit_from(capture, pruning, prune_frac),
                     "avg_launch_ms": force_avg_ms, **step_roof},
        "contacts": contacts,
        "cpu_baseline": cpu,
        "e2e": e2e,
        "gpu_launches": launches,
        "clocks": clk,
    }
    if stats.get("many_step"):
        # a small system is bound by launch and dependent-load latency, not by HBM: the
        # step's time beside the same step launched kernel by kernel and its force kernel
        line["latency"] = {"us_per_step": total_ms / K * 1e3,
                           "force_kernel_us": force_avg_ms * 1e3,
                           "resorts_per_step": rebuilds_timed / K,
                           "note": ("us_per_step: cooperative many-step launches (one grid barrier a "
                                    "step); force_kernel_us: the same step's force kernel launched alone "
                                    "(CUDA events around each launch), one chain of dependent loads")}
    eng.close()
    if rank == 0 and world == 1 and not args.no_rollout:
        line["rollout"] = run_rollout(args, w, young, skin, dev, torch, **shape_kw)
    if rank == 0 and world == 1 and not args.no_batched:
        line["batched"] = run_batched(args, dev, flush, torch)
    if rank == 0 and world == 1 and not args.no_served:
        line["served"] = run_served(args, dev)
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_rollout(args, w, young, skin, dev, torch, **eng_kw):
    """System.trajectory_rollout through jdem_rollout: the timed steps with a frame
    (pos_c, vel, force in caller order) saved every ``--frame-stride`` steps, into
    device memory and into fresh pageable host arrays, beside the same steps
    without frames.  Wall-clock per call, best of three."""
    from jaxdem_gb300._lib import Engine

    K, k = args.steps, max(1, args.frame_stride)
    T = max(1, K // k)
    strides = np.full(T, k, np.int64)
    eng = Engine(w.dim, [w.desc()], young, skin=skin, chunk_steps=CHUNK, device=dev, **eng_kw)
    fields = ("pos_c", "vel", "force")
    dev_out = {f: torch.empty((T, w.N, w.dim), dtype=torch.float32, device=f"cuda:{dev}") for f in fields}

    def best(fn):
        t = []
        for _ in range(3):
            eng.upload(pos=w.pos, rad=w.rad, mass=w.mass, vel=w.vel)
            eng.step(CHUNK)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            fn()
            t.append(time.perf_counter() - t0)
        return min(t)

    eng.upload(pos=w.pos, rad=w.rad, mass=w.mass, vel=w.vel)
    eng.rollout(strides[:2], fields=fields, boxes=False)  # graphs for the stride, ring allocation
    plain = best(lambda: eng.step(T * k))
    on_dev = best(lambda: eng.rollout(strides, fields=fields, out=dev_out, boxes=False))
    on_host = best(lambda: eng.rollout(strides, fields=fields, boxes=False))
    eng.close()
    frame_bytes = 3 * w.N * w.dim * 4
    rate = lambda s: w.N * T * k / s
    return {"frames": T, "frame_stride": k, "frame_bytes": frame_bytes,
            "plain_steps": rate(plain), "to_device": rate(on_dev), "to_host_pageable": rate(on_host),
            "unit": "particle-steps/s",
            "host_frame_GBps": frame_bytes * T / on_host / 1e9,
            "note": "wall clock per call (best of 3); host arrays freshly allocated each call"}


def run_batched(args, dev, flush, torch, n_systems=4096, steps=1000):
    """Mixed-size batch: 4096 periodic 3D systems, N ~ logU[64, 16384], phi ~ U[0.3, 0.6],
    1000 steps in 50-step graph chunks, against the plain kernel looped per system."""
    from jaxdem_gb300 import workloads as W
    from jaxdem_gb300._lib import Engine
    from jaxdem_gb300.batch import BatchedSystems

    from jaxdem_gb300 import autotune

    ws = W.c4(n_systems=n_systems)
    total = sum(w.N for w in ws)
    rmax = max(float(w.rad.max()) for w in ws)
    shapes, tuning = {}, None
    if args.skin is not None or args.no_tune:
        skin = args.skin if args.skin is not None else autotune.default_skin(rmax)
    else:
        from jaxdem_gb300.batch import tune_key

        key = tune_key(ws)

        def mk(skin, **shape):
            return BatchedSystems(ws, skin=skin, chunk_steps=CHUNK, device=dev, **shape).engine

        def up(eng):
            cat = lambda k: np.concatenate([getattr(w, k) for w in ws])  # noqa: E731
            eng.upload(pos=cat("pos"), rad=cat("rad"), mass=cat("mass"), vel=cat("vel"))

        best, timings = autotune.tune_shapes(mk, up, rmax, total, key=key, steps=CHUNK)
        skin = best.pop("skin")
        shapes = best
        ps = shapes["prune_skin"]
        tuning = {"skin_over_rmax": round(skin / rmax, 3),
                  "prune_skin_over_skin": round(ps / skin, 3) if ps > 0 else "off",
                  "brick_particles": shapes["brick_particles"], "force_block": shapes["force_block"],
                  "small_lanes": shapes["small_lanes"],
                  "ms_per_step": {sh: {k: round(v * 1e3, 4) for k, v in t.items()} for sh, t in timings.items() if t}}
    bs = BatchedSystems(ws, skin=skin, chunk_steps=CHUNK, device=dev, **shapes)
    bs.upload()
    bs.step(CHUNK)  # warm-up: capture, first re-sort
    stream = torch.cuda.ExternalStream(bs.engine.stream(), device=dev)
    ms = 0.0
    for _ in range(steps // CHUNK):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        bs.step_async(CHUNK)
        b.record(stream)
        b.synchronize()
        ms += a.elapsed_time(b)
    bs.engine.sync()
    batched = total * steps / (ms * 1e-3)
    bs.close()
    # plain fused kernel looped per system: every k-th system, one handle each
    k = max(1, n_systems // max(1, args.plain_sample))
    sample = ws[::k]
    p_steps = 100
    t_sum, ps_sum = 0.0, 0
    for w in sample:
        e = Engine(3, [w.desc()], np.array([[W.K_SPRING]], np.float32), skin=skin, chunk_steps=CHUNK, device=dev)
        e.upload(pos=w.pos, rad=w.rad, mass=w.mass, vel=w.vel)
        e.step(CHUNK)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e.step(p_steps)
        t_sum += time.perf_counter() - t0
        ps_sum += w.N * p_steps
        e.close()
    plain = ps_sum / t_sum
    return {"workload": f"{n_systems} periodic 3D systems, N~logU[64,16384] (total {total}), phi~U[0.3,0.6], "
                        f"r 0.5/0.7, dt=1e-3, {steps} steps in {CHUNK}-step graph chunks",
            "value": batched, "unit": "particle-steps/s", "ms_per_step": ms / steps, "autotune": tuning,
            "plain_looped": plain, "batched_over_plain": batched / plain,
            "plain_sample": f"{len(sample)} of {n_systems} systems stepped one at a time ({p_steps} steps each, "
                            f"one handle and graph per system), throughput = sum(N*steps)/sum(time)"}


def run_served(args, dev):
    """Continuous batching of the rollout-request stream (Poisson arrivals at 200/s,
    N ~ logU[256, 262144], dim 2 or 3, phi ~ U[0.3, 0.6], steps ~ U{100..10000}): the
    first ``--serve-requests`` requests at their configured arrival times, against the
    plain kernel serving requests one at a time.

    The one-at-a-time server is timed on ``--serve-baseline`` requests spread evenly over
    the window (its throughput is their particle-steps over their service time).  Its
    latency on the full window is modelled, not measured: a FIFO queue over the same
    arrivals whose service times come from a per-dimension linear fit of the measured
    times against N x steps."""
    from jaxdem_gb300 import serve
    from jaxdem_gb300 import workloads as W

    reqs = W.c5()
    head = reqs[: args.serve_requests]
    offered = sum(r.N * r.steps for r in head) / max(head[-1].arrival, 1e-9)
    res = serve.run_stream(head, device=dev)
    k = max(1, len(head) // max(1, args.serve_baseline))
    sample = head[::k][: args.serve_baseline]
    base = serve.run_one_at_a_time(sample, device=dev, paced=False)
    model = serve.fifo_model(head, sample, base["service_s"])
    return {"workload": f"first {len(head)} of 20000 requests (Poisson 200/s; N~logU[256,262144]; dim 2|3; "
                        f"phi~U[0.3,0.6]; r~U[0.4,0.6]; steps~U{{100..10000}}), periodic, 150 GB HBM budget",
            "value": res["throughput"], "unit": "particle-steps/s",
            "latency_s": res["latency_s"], "queue_wait_s": res["queue_wait_s"], "completed": res["completed"],
            "requests": len(head), "offered_load": offered, "makespan_s": res["makespan_s"],
            "arrival_window_s": head[-1].arrival, "server_stats": res["server_stats"],
            "one_at_a_time": {"requests_timed": base["completed"], "busy_throughput": base["busy_throughput"],
                              "sample": f"every {k}th request of the window, served back to back",
                              "modelled_latency_s": model["latency_s"],
                              "model": "FIFO queue over the window's arrivals; service time = a_dim + "
                                       "b_dim * N * steps fitted to the timed requests"},
            "served_over_one_at_a_time": res["throughput"] / base["busy_throughput"]}


def main():
    args = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    dist = None
    if world > 1:
        import torch
        import torch.distributed as tdist

        if args.impl == "ours":
            torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
            tdist.init_process_group("nccl")
            dist = tdist
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    import __graft_entry__ as g

    g.build()
    run_ours(args, rank, world, dist)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
