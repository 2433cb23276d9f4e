#!/usr/bin/env python3
"""Benchmark of the Solvent-Excluded Surface build on GB300.

One step = one complete SES build (bcs::Sesdf::build semantics) of the
100,000-atom assembly (20 globules of 5,000 atoms, probe 1.4 A), full surface.
`value` is atoms/s over K device-timed builds with the atoms resident in HBM
(CUDA events on the launching stream around each build; L2 flushed between
builds by writing a 256 MB buffer outside the events). `e2e` is the same metric
through the C ABI from pinned host memory: upload, build and counter read-back,
wall-clocked per call. Extra keys report the exterior-only build and the
1,000,000-atom shell.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference runs the reference's own CUDA kernels (PlathC/SESDF, compiled
from its sources into oracle/_ref/) through the restated host driver of
oracle/ref/ref_driver.cu, timed the way the reference's benchmark app times
build() (CUDA events on the default stream around each build).
For N > 1 (torchrun) every rank builds its own copy: replicas, no collective.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "SES build ms & atoms/s at 100k/1M atoms; batched+adjoint vs plain, ≤1e-4 Å"
RP = 1.4
L2_FLUSH_BYTES = 256 << 20
COUNTS_BYTES = 132  # sesgb DeviceCounts read back per build
FP32_LANES = 152 * 128  # SMs x FP32 lanes of a GB300


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), float(p.get("sm_max_mhz", 2070.0)), "measured"
    except Exception:
        return 6800.0, 2070.0, "fallback"


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_init():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    import torch
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    return rank, world, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x: float, world: int) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def workload(name: str):
    from sesdf_gb300 import synth
    if name == "assembly100k":
        return synth.assembly()
    if name == "shell1m":
        return synth.shell()
    if name == "globule2k":
        return synth.globule(2000, 1000)
    raise ValueError(name)


def time_ours(atoms, mode, steps, warmup, flush, stages=None):
    """Device-timed builds from atoms resident in HBM; returns per-step ms, launches, context.

    With `stages` (a dict), the builds also record CUDA events between their
    stages (on the build's stream) and the dict receives the per-stage
    milliseconds averaged over the timed builds."""
    import torch
    from sesdf_gb300 import SesBuild, api
    g = SesBuild(atoms, RP, mode, profile=stages is not None)
    d_atoms = torch.from_numpy(atoms).cuda()
    stream = torch.cuda.current_stream()
    for _ in range(max(warmup, 1)):
        flush.zero_()
        g.build_async(d_atoms.data_ptr(), stream.cuda_stream)
        g.finish()
    torch.cuda.synchronize()
    l0 = api.launch_count()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    for k in range(steps):
        flush.zero_()
        starts[k].record(stream)
        g.build_async(d_atoms.data_ptr(), stream.cuda_stream)
        ends[k].record(stream)
        g.finish()
        if stages is not None:
            for name, v in g.stage_times().items():
                if name:
                    stages[name] = stages.get(name, 0.0) + v / steps
    torch.cuda.synchronize()
    launches = api.launch_count() - l0
    ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    return ms, launches, g


def time_e2e(atoms, mode, steps, warmup, flush):
    """Public API from pinned host memory: upload + build + counter read-back per call."""
    import torch
    from sesdf_gb300 import SesBuild
    pinned = torch.from_numpy(atoms).pin_memory()
    g = SesBuild(atoms, RP, mode)
    g.set_host_pointer(pinned.data_ptr())
    for _ in range(max(warmup, 1)):
        flush.zero_()
        torch.cuda.synchronize()
        g.build()
    ms = []
    for _ in range(steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        g.build()
        ms.append((time.perf_counter() - t0) * 1e3)
    g.close()
    return ms


def time_plain_loop(mols, mode, repeats, flush):
    """One build per molecule through its own context (created beforehand), in sequence:
    per-step device ms for the whole loop."""
    import torch
    from sesdf_gb300 import SesBuild
    stream = torch.cuda.current_stream()
    ctxs = [SesBuild(m, RP, mode) for m in mols]
    dev = [torch.from_numpy(m).cuda() for m in mols]
    for g, d in zip(ctxs, dev):
        g.build_async(d.data_ptr(), stream.cuda_stream)
        g.finish()
    out = []
    for _ in range(repeats):
        flush.zero_()
        t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0.record(stream)
        for g, d in zip(ctxs, dev):
            g.build_async(d.data_ptr(), stream.cuda_stream)
            g.finish()
        t1.record(stream)
        torch.cuda.synchronize()
        out.append(t0.elapsed_time(t1))
    for g in ctxs:
        g.close()
    return out


def time_batched(mols, mode, repeats, flush, cap, graph, tuning=None):
    import torch
    from sesdf_gb300 import SesBatch
    stream = torch.cuda.current_stream()
    b = SesBatch(mols, RP, mode, max_neighbor_per_atom=cap, graph=graph)
    if tuning:
        b.set_tuning(**tuning)
    d = torch.from_numpy(b.atoms).cuda()
    for _ in range(2):
        b.build_async(d.data_ptr(), stream.cuda_stream)
        b.finish()
    out = []
    for _ in range(repeats):
        flush.zero_()
        t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0.record(stream)
        b.build_async(d.data_ptr(), stream.cuda_stream)
        t1.record(stream)
        b.finish()
        torch.cuda.synchronize()
        out.append(t0.elapsed_time(t1))
    c = b.counts()
    b.close()
    return out, c


def batch_extras(args, flush, rank=0, world=1):
    """Batched builds (256 molecules of log-uniform size; 64 jittered frames) against the plain loop.
    With several ranks each builds its contiguous share of the molecules (balanced by atoms); the
    slowest rank sets the time."""
    from sesdf_gb300 import synth
    from sesdf_gb300.autotune import tune_batch
    from sesdf_gb300.partition import split_by_atoms
    res = {}
    sizes = synth.batch_sizes()
    sets = {"batch256_mixed": [synth.globule(int(n), 1300 + m) for m, n in enumerate(sizes)],
            "batch64_frames": synth.frames()}
    for name, all_mols in sets.items():
        a, b = split_by_atoms([m.shape[0] for m in all_mols], world)[rank]
        mols = all_mols[a:b] if b > a else all_mols[:1]
        tuned = tune_batch(mols, RP, "full")
        bm, c = time_batched(mols, "full", 5, flush, tuned["max_neighbor_per_atom"], tuned["graph"], tuned["tuning"])
        pm = time_plain_loop(mols, "full", 3, flush)
        bmed = max_over_ranks(float(np.median(bm)), world)
        pmed = max_over_ranks(float(np.median(pm)), world)
        atoms = int(sum(m.shape[0] for m in all_mols))
        res[name] = {"molecules": len(all_mols), "atoms": atoms, "batched_ms": round(bmed, 3),
                     "plain_loop_ms": round(pmed, 3), "speedup": round(pmed / bmed, 2),
                     "batched_atoms_per_s": round(atoms / (bmed * 1e-3), 1),
                     "tuned": {k: tuned[k] for k in ("max_neighbor_per_atom", "graph", "max_neighbors", "tuning")},
                     "probes_rank0": c["probes"], "split": "molecules by atoms over ranks" if world > 1 else None}
    return res


def sdf_extra(flush):
    """SDF forward and adjoint (20,000-atom globule, 1M query points within 3 A of its vdW surface);
    SES area of the same build and its adjoint."""
    import torch
    from sesdf_gb300 import SesBuild, synth
    atoms, q = synth.sdf_workload()
    m = q.shape[0]
    stream = torch.cuda.current_stream()
    g = SesBuild(atoms, RP, "full")
    g.build()
    dq = torch.from_numpy(q).cuda()
    out = torch.empty(m, dtype=torch.float32, device="cuda")
    gs = torch.ones(m, dtype=torch.float32, device="cuda")
    ga = torch.empty((atoms.shape[0], 4), dtype=torch.float32, device="cuda")
    res = {}
    for name, fn in (("forward", lambda: g.sdf(dq.data_ptr(), m, out.data_ptr(), None, stream.cuda_stream)),
                     ("backward", lambda: g.sdf_backward(dq.data_ptr(), m, gs.data_ptr(), ga.data_ptr(),
                                                         stream.cuda_stream))):
        for _ in range(3):
            fn()
        ms = []
        for _ in range(10):
            flush.zero_()
            t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            t0.record(stream)
            fn()
            t1.record(stream)
            torch.cuda.synchronize()
            ms.append(t0.elapsed_time(t1))
        res[f"{name}_ms"] = round(float(np.median(ms)), 4)
        res[f"{name}_queries_per_s"] = round(m / (float(np.median(ms)) * 1e-3), 1)
    res["queries"] = int(m)
    res["atoms"] = int(atoms.shape[0])
    res["probes"] = int(g.counts()["probes"])
    res["band_A"] = 3.0
    # SES area of the primitives (sesgb_ses_area synchronises: host wall clock around the call)
    # and its adjoint (device events)
    per = torch.empty(atoms.shape[0], dtype=torch.float32, device="cuda")
    for _ in range(3):
        area = g.ses_area(per.data_ptr(), stream.cuda_stream)
    ms = []
    for _ in range(10):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        area = g.ses_area(per.data_ptr(), stream.cuda_stream)
        ms.append((time.perf_counter() - t0) * 1e3)
    res["area_A2"] = round(area["total"], 3)
    res["area_parts_A2"] = {k: round(area[k], 3) for k in ("convex", "toroidal", "concave")}
    res["area_ms"] = round(float(np.median(ms)), 4)
    for _ in range(3):
        g.ses_area_backward(ga.data_ptr(), (1.0, 1.0, 1.0), stream.cuda_stream)
    ms = []
    for _ in range(10):
        flush.zero_()
        t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0.record(stream)
        g.ses_area_backward(ga.data_ptr(), (1.0, 1.0, 1.0), stream.cuda_stream)
        t1.record(stream)
        torch.cuda.synchronize()
        ms.append(t0.elapsed_time(t1))
    res["area_backward_ms"] = round(float(np.median(ms)), 4)
    # headless image: 512 x 512 rays sphere-traced on the device in one launch (sesgb_render)
    from sesdf_gb300 import render
    w = h = 512
    eye, centre, up, t_near, t_far = render.framing(atoms, RP)
    f, r, u = render.camera_basis(eye, centre, up)
    cam = dict(eye=eye, forward=f, right=r, up=u, tan_half_fov=float(np.tan(np.radians(20.0))), t_near=float(t_near),
               t_far=float(t_far), eps=1e-3, normal_step=1e-2, width=w, height=h, max_steps=256)
    depth = torch.empty(w * h, dtype=torch.float32, device="cuda")
    nrm = torch.empty(3 * w * h, dtype=torch.float32, device="cuda")
    for _ in range(2):
        g.render(cam, depth.data_ptr(), nrm.data_ptr(), stream.cuda_stream)
    ms = []
    for _ in range(5):
        t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0.record(stream)
        g.render(cam, depth.data_ptr(), nrm.data_ptr(), stream.cuda_stream)
        t1.record(stream)
        torch.cuda.synchronize()
        ms.append(t0.elapsed_time(t1))
    res["render_512x512_ms"] = round(float(np.median(ms)), 4)
    res["render_hit_pixels"] = int(torch.isfinite(depth).sum().item())
    # exterior and cavities on a 0.5 A voxel grid (sesgb_cavities synchronises: host wall clock)
    g.cavities(0.5)
    ms = []
    for _ in range(5):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        info = g.cavities(0.5)
        ms.append((time.perf_counter() - t0) * 1e3)
    res["cavities_0.5A_ms"] = round(float(np.median(ms)), 4)
    res["cavities_0.5A"] = {"voxels": int(np.prod(info["dims"])), "components": info["components"],
                            "exterior": info["exterior"], "cavities": info["cavities"]}
    g.close()
    return res


def profiled(kernel: str, workload: str = "assembly100k") -> dict:
    """From the kernel's committed ncu summary (profiles/<kernel>_<workload>.txt): DRAM bytes and warp
    instructions per launch, threads per instruction, and the issue-slot, ALU-pipe and FMA-pipe
    utilisations of the same capture (fractions)."""
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "profiles", f"{kernel}_{workload}.txt")
    out = {}
    keys = {"dram_bytes_per_launch:": "traffic", "issue active %": "issue_active", "ALU pipe %": "alu_pipe",
            "FMA pipe %": "fma_pipe", "threads per instruction": "threads_per_instruction",
            "warp instructions": "warp_instructions", "duration (one launch, cold)": "duration_us"}
    try:
        with open(path) as f:
            for line in f:
                for k, name in keys.items():
                    if line.startswith(k):
                        v = float(line[len(k):].split()[0])
                        out[name] = int(v) if name in ("traffic", "warp_instructions") else (
                            round(v / 100, 3) if "%" in k else v)
    except (OSError, ValueError):
        pass
    return out


ISSUE_SLOTS = 152 * 4  # SMs x warp schedulers (one warp instruction per scheduler and cycle)


def issue_roofline(kernel: str, ms: float, sm_mhz: float, bytes_alg: float, workload: str = "assembly100k") -> dict:
    """Issue-rate roofline of a SIMT kernel that is not a dense contraction and not HBM-bound: the warp
    instructions of one launch (committed ncu summary of the same workload) over its CUDA-event time,
    against 152 SMs x 4 schedulers x the SM clock sampled during the timed builds. lane_efficiency =
    threads per instruction / 32; useful_lane_frac = frac x lane_efficiency is the fraction of the SIMT
    lanes' peak that does work. The HBM fraction (algorithmic bytes over the same time) is secondary."""
    hbm, sm_max, src = peaks()
    prof = profiled(kernel, workload)
    clk = sm_mhz or sm_max
    peak = ISSUE_SLOTS * clk * 1e6 / 1e9  # G warp instructions/s
    inst = prof.get("warp_instructions")
    achieved = inst / (ms * 1e-3) / 1e9 if inst else None
    lane = prof["threads_per_instruction"] / 32 if "threads_per_instruction" in prof else None
    frac = achieved / peak if achieved else None
    hbm_achieved = bytes_alg / (ms * 1e-3) / 1e9
    return {"kernel": kernel, "bound": "issue", "achieved": round(achieved, 1) if achieved else None, "peak": round(peak, 1),
            "unit": "G warp-instructions/s", "frac": round(frac, 4) if frac else None,
            "traffic": prof.get("traffic"), "lane_efficiency": round(lane, 4) if lane else None,
            "useful_lane_frac": round(frac * lane, 4) if frac and lane else None,
            "warp_instructions_per_launch": inst, "ms_per_launch": round(ms, 4),
            "peak_basis": f"152 SMs x 4 schedulers x {clk:.0f} MHz (SM clock sampled during the timed builds)",
            "profile": f"profiles/{kernel}_{workload}.txt",
            "hbm": {"achieved": round(hbm_achieved, 1), "peak": hbm, "unit": "GB/s", "frac": round(hbm_achieved / hbm, 4),
                    "bytes_per_launch": bytes_alg, "peak_source": src}}


def roofline(stages, counts, n_atoms, sm_mhz):
    """The dominant kernel of the build (k_visibility or k_probes, one launch per build), by its
    CUDA-event time in the timed builds."""
    P, C1, I = counts["pairs"], counts["partial_circles"], counts["probes"]
    if stages.get("probes", 0.0) > stages.get("visibility", 0.0):
        kernel, ms = "k_probes", stages["probes"]
        # staged neighbourhood (ids, atoms, statuses, neighbour counts), touch masks, staged probes and jobs
        bytes_alg = 25.0 * P + 8.0 * C1 + 64.0 * I + 36.0 * n_atoms
    else:
        kernel, ms = "k_visibility", stages["visibility"]
        bytes_alg = 21.0 * P + 32.0 * n_atoms  # neighbour ids + neighbour atoms + status + per-atom I/O
    return issue_roofline(kernel, ms, sm_mhz, bytes_alg)


def cpu_baseline(atoms, budget_s: float = 12.0):
    from oracle import oracle
    cores = os.cpu_count() or 1
    runs, total = 0, 0.0
    while total < budget_s or runs == 0:
        t0 = time.perf_counter()
        oracle.run(atoms, RP, "full", threads=cores)
        total += time.perf_counter() - t0
        runs += 1
        if runs >= 8:
            break
    return {"value": round(atoms.shape[0] * runs / total, 1), "unit": "atoms/s", "cores": cores, "kind": "port",
            "sample": f"FP64 oracle, full surface of the whole 100k-atom assembly, {runs} build(s) in {total:.1f} s"}


def bench_config(n: int, world: int) -> dict:
    """The workload both arms time (identical dicts, so that their lines compare)."""
    return {"workload": "assembly100k: 20 globules x 5,000 atoms, full SES, probe 1.4 A", "atoms": n,
            "probe_radius": RP, "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
            "l2": "flushed between builds (256 MB write outside the timed events)"}


def run_ours(args, rank, world, local):
    import torch
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    atoms = workload("assembly100k")
    n = atoms.shape[0]
    sampler = ClockSampler(local)
    barrier(world)
    torch.cuda.synchronize()
    sampler.start()
    t_wall = time.perf_counter()
    ms, launches, g = time_ours(atoms, "full", args.steps, args.warmup, flush)
    torch.cuda.synchronize()
    barrier(world)
    wall = time.perf_counter() - t_wall
    clocks = sampler.stop()
    total_ms = max_over_ranks(float(np.sum(ms)), world)
    counts = g.counts()
    g.close()
    # per-stage CUDA events (recorded inside the replayed graph) over as many builds again,
    # right after the timed ones: the timed builds carry no events
    stages = {}
    time_ours(atoms, "full", args.steps, 2, flush, stages)[2].close()
    value = n * args.steps * world / (total_ms * 1e-3)
    if args.kernels_only:
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": round(value, 1), "unit": "atoms/s", "n_gpus": world,
                              "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(total_ms / args.steps, 4),
                              "gpu_launches": int(launches), "kernels_only": True}), flush=True)
        return

    e2e_ms = time_e2e(atoms, "full", args.steps, args.warmup, flush)
    e2e_total = max_over_ranks(float(np.sum(e2e_ms)), world)

    extra = {}
    if not args.no_extras:
        xm, _, gx = time_ours(atoms, "exterior", args.steps, args.warmup, flush)
        extra["exterior_100k"] = {"ms_per_step": round(float(np.mean(xm)), 4),
                                  "atoms_per_s": round(n / (np.mean(xm) * 1e-3), 1)}
        gx.close()
        shell = workload("shell1m")
        for mode in ("full", "exterior"):
            k1m = max(3, args.steps // 4)
            sm, _, gs = time_ours(shell, mode, k1m, 2, flush)
            c = gs.counts()
            extra[f"{mode}_1m"] = {"ms_per_step": round(float(np.mean(sm)), 4),
                                   "atoms_per_s": round(shell.shape[0] / (np.mean(sm) * 1e-3), 1),
                                   "probes": c["probes"], "fp64_decisions": c["fp64_decisions"]}
            if not args.no_error_report:
                # error of the build's probes and sectors against FP64, and its band counts (after the timing)
                from sesdf_gb300 import precision
                extra[f"{mode}_1m"]["error_vs_fp64"] = precision.error_report(gs.fetch(analysis=True), RP, mode)
            gs.close()
            em = time_e2e(shell, mode, k1m, 2, flush)
            extra[f"{mode}_1m"]["e2e"] = {"ms_per_step": round(float(np.mean(em)), 4),
                                          "atoms_per_s": round(shell.shape[0] / (np.mean(em) * 1e-3), 1),
                                          "h2d_bytes_per_step": shell.shape[0] * 16,
                                          "d2h_bytes_per_step": COUNTS_BYTES}
        del shell
        extra.update(batch_extras(args, flush, rank, world))
        extra["sdf_20k_1m"] = sdf_extra(flush)
        sx = extra["sdf_20k_1m"]
        # issue-rate rooflines of the on-demand kernels (their ncu summaries: profiles/<kernel>_<workload>.txt);
        # the SDF call's time is k_sdf's to within its sort of the query keys, the area call's is the sum of
        # k_area_atoms and k_area_probes (split by the launch list's shares)
        n20, m = sx["atoms"], sx["queries"]
        extra["rooflines"] = {
            "k_sdf": issue_roofline("k_sdf", sx["forward_ms"], clocks.get("sm_mhz"), 16.0 * m + 16.0 * n20,
                                    "globule20k_1m"),
        }
        # the image: 16 bytes (depth + normal) per pixel out; the build it traces is L2-resident
        extra["rooflines"]["k_trace"] = issue_roofline("k_trace", sx["render_512x512_ms"], clocks.get("sm_mhz"),
                                                       16.0 * 512 * 512, "globule20k_512")
        prof_a, prof_p = profiled("k_area_atoms", "globule20k"), profiled("k_area_probes", "globule20k")
        if prof_a.get("duration_us") and prof_p.get("duration_us"):
            share = prof_a["duration_us"] / (prof_a["duration_us"] + prof_p["duration_us"])
            extra["rooflines"]["k_area_atoms"] = issue_roofline("k_area_atoms", sx["area_ms"] * share, clocks.get("sm_mhz"),
                                                                16.0 * n20, "globule20k")
            extra["rooflines"]["k_area_probes"] = issue_roofline("k_area_probes", sx["area_ms"] * (1 - share),
                                                                 clocks.get("sm_mhz"), 64.0 * sx.get("probes", 0),
                                                                 "globule20k")

    roof = roofline(stages, counts, n, clocks.get("sm_mhz"))
    line = {
        "metric": METRIC, "value": round(value, 1), "unit": "atoms/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(total_ms / args.steps, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 (f64 triplet solve and band re-evaluation)",
        "data": "synthetic (seeded protein-like globules; no PDB files)",
        "config": bench_config(n, world),
        "e2e": {"value": round(n * args.steps * world / (e2e_total * 1e-3), 1), "unit": "atoms/s",
                "h2d_bytes_per_step": n * 16, "d2h_bytes_per_step": COUNTS_BYTES,
                "ms_per_step": round(e2e_total / args.steps, 4)},
        "gpu_launches": int(launches),
        "launches_per_build": int(launches // max(args.steps, 1)),
        "roofline": roof,
        "stages_ms": {k: round(v, 4) for k, v in stages.items()},
        "counts": {k: counts[k] for k in ("pairs", "sectors", "partial_circles", "probes", "singular_probes",
                                          "segments", "full_circles")},
        "fp64_decisions": counts["fp64_decisions"],
        "clocks": clocks,
        "timed_wall_s": round(wall, 3),
        "extra": extra,
    }
    if rank == 0:
        line["cpu_baseline"] = cpu_baseline(atoms)
        print(json.dumps(line), flush=True)


# read-backs inside one reference build (oracle/ref/ref_driver.cu, as sesdf/src/sesdf/sesdf.cu:172-264 does
# them): five blocking 4-byte counter reads, plus the 8-byte results of one thrust::count_if and two
# thrust::copy_if calls
REF_D2H_BYTES_FULL = 5 * 4 + 3 * 8
# exterior build (sesdf/src/ssesdf/ssesdf.cu:133-187): one 4-byte counter read, the results of four
# thrust::count_if calls and one thrust::copy_if
REF_D2H_BYTES_EXTERIOR = 4 + 5 * 8


def run_profile_case(args):
    """One on-demand workload of the 20,000-atom globule, args.steps times after args.warmup, for
    profiler runs (no JSON line): sdf (forward and adjoint at 200,000 of the 1M queries), area
    (SES area and its adjoint), render (512 x 512 depth and normal image, as timed), cavities (0.5 A voxels)."""
    import torch
    from sesdf_gb300 import SesBuild, render, synth
    atoms, q = synth.sdf_workload()
    q = np.ascontiguousarray(q[:200_000])
    stream = torch.cuda.current_stream()
    g = SesBuild(atoms, RP, "full")
    g.build()
    m = q.shape[0]
    dq = torch.from_numpy(q).cuda()
    out = torch.empty(m, dtype=torch.float32, device="cuda")
    gs = torch.ones(m, dtype=torch.float32, device="cuda")
    ga = torch.empty((atoms.shape[0], 4), dtype=torch.float32, device="cuda")
    depth = torch.empty(512 * 512, dtype=torch.float32, device="cuda")
    nrm = torch.empty(3 * 512 * 512, dtype=torch.float32, device="cuda")
    eye, centre, up, t_near, t_far = render.framing(atoms, RP)
    f, r, u = render.camera_basis(eye, centre, up)
    cam = dict(eye=eye, forward=f, right=r, up=u, tan_half_fov=float(np.tan(np.radians(20.0))), t_near=float(t_near),
               t_far=float(t_far), eps=1e-3, normal_step=1e-2, width=512, height=512, max_steps=256)

    def once():
        if args.profile_case == "sdf":
            g.sdf(dq.data_ptr(), m, out.data_ptr(), None, stream.cuda_stream)
            g.sdf_backward(dq.data_ptr(), m, gs.data_ptr(), ga.data_ptr(), stream.cuda_stream)
        elif args.profile_case == "area":
            g.ses_area(None, stream.cuda_stream)
            g.ses_area_backward(ga.data_ptr(), (1.0, 1.0, 1.0), stream.cuda_stream)
        elif args.profile_case == "render":
            g.render(cam, depth.data_ptr(), nrm.data_ptr(), stream.cuda_stream)
        elif args.profile_case == "cavities":
            g.cavities(0.5)
    for _ in range(args.warmup + args.steps):
        once()
    torch.cuda.synchronize()
    g.close()


def run_reference(args, rank, world, local):
    """The reference's own kernels under its restated host orchestration. This process maps only the
    reference harness (oracle/_ref/libsesref.so, which also carries the synthetic-input generator):
    nothing of sesdf_gb300's native code is built or loaded here."""
    if rank != 0:
        return
    import torch
    from oracle import refharness
    if not refharness.available():
        print(json.dumps({"impl": "reference", "unavailable": "reference kernels not built (oracle/_ref missing)"}))
        return
    from sesdf_gb300 import synth
    synth.use_library(refharness.build_driver())
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    atoms = workload("assembly100k")
    n = atoms.shape[0]
    r = refharness.RefBuild(atoms, RP, "full")
    for _ in range(max(args.warmup, 1)):
        r.build()
    torch.cuda.synchronize()
    sampler = ClockSampler(local)
    sampler.start()
    ms = []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        ms.append(float(r.time(1)[0]))
    clocks = sampler.stop()
    counts = r.counts()
    r.close()
    total = float(np.sum(ms))
    value = n * args.steps / (total * 1e-3)
    extra = {}
    if not args.no_extras:
        rx = refharness.RefBuild(atoms, RP, "exterior")
        rx.build()
        xm = [float(rx.time(1)[0]) for _ in range(args.steps)]
        rx.close()
        extra["exterior_100k"] = {"ms_per_step": round(float(np.mean(xm)), 4),
                                  "atoms_per_s": round(n / (np.mean(xm) * 1e-3), 1)}
        shell = workload("shell1m")
        for mode in ("full", "exterior"):
            rs = refharness.RefBuild(shell, RP, mode)
            rs.build()
            sm = [float(rs.time(1)[0]) for _ in range(max(3, args.steps // 4))]
            rs.close()
            # the reference's build() uploads the atoms itself: its time is end to end
            extra[f"{mode}_1m"] = {"ms_per_step": round(float(np.mean(sm)), 4),
                                   "atoms_per_s": round(shell.shape[0] / (np.mean(sm) * 1e-3), 1),
                                   "e2e": {"ms_per_step": round(float(np.mean(sm)), 4),
                                           "atoms_per_s": round(shell.shape[0] / (np.mean(sm) * 1e-3), 1),
                                           "h2d_bytes_per_step": shell.shape[0] * 16,
                                           "d2h_bytes_per_step": REF_D2H_BYTES_FULL if mode == "full"
                                           else REF_D2H_BYTES_EXTERIOR}}
        del shell
        # the reference's per-molecule loop over the same 256-molecule batch (context for the batched build)
        mols = [synth.globule(int(nm), 1300 + k) for k, nm in enumerate(synth.batch_sizes())]
        refs = [refharness.RefBuild(m, RP, "full") for m in mols]
        for rr in refs:
            rr.build()
        loops = []
        for _ in range(2):
            flush.zero_()
            torch.cuda.synchronize()
            loops.append(float(sum(float(rr.time(1)[0]) for rr in refs)))
        for rr in refs:
            rr.close()
        extra["batch256_mixed_loop"] = {"molecules": len(mols), "atoms": int(sum(m.shape[0] for m in mols)),
                                        "loop_ms": round(float(np.median(loops)), 3)}
        # and over the 64 jittered frames of the 20,000-atom globule (the oracle finds at most 26 probes
        # owned by one atom in any frame, far inside the reference's unchecked 128-entry block buffer)
        frames = synth.frames()
        refs = [refharness.RefBuild(m, RP, "full") for m in frames]
        for rr in refs:
            rr.build()
        loops = []
        for _ in range(2):
            flush.zero_()
            torch.cuda.synchronize()
            loops.append(float(sum(float(rr.time(1)[0]) for rr in refs)))
        for rr in refs:
            rr.close()
        extra["batch64_frames_loop"] = {"molecules": len(frames), "atoms": int(sum(m.shape[0] for m in frames)),
                                        "loop_ms": round(float(np.median(loops)), 3)}
    line = {
        "metric": METRIC, "value": round(value, 1), "unit": "atoms/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(total / args.steps, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 (--use_fast_math)", "impl": "reference",
        "data": "synthetic (seeded protein-like globules; no PDB files)",
        "config": bench_config(n, world),
        # the timed build() uploads the atoms from host memory (pageable cudaMemcpy, sesdf/src/sesdf/sesdf.cu:212-213)
        # and reads its counters back: the device-timed value is already end to end
        "e2e": {"value": round(value, 1), "unit": "atoms/s", "h2d_bytes_per_step": n * 16,
                "d2h_bytes_per_step": REF_D2H_BYTES_FULL, "ms_per_step": round(total / args.steps, 4)},
        "cpu_baseline": {"value": round(value, 1), "unit": "atoms/s", "cores": 1, "kind": "reference",
                         "sample": "the reference's own implementation of this path is CUDA: its kernels (built from "
                                   "its sources) run on the GPU under its restated host orchestration, one host thread"},
        "counts": counts, "clocks": clocks, "extra": extra,
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-extras", action="store_true")
    ap.add_argument("--no-error-report", action="store_true", help="skip the FP64 error report of the 1M builds")
    ap.add_argument("--profile-case", choices=["sdf", "area", "render", "cavities"], default=None,
                    help="run one on-demand workload of the 20k-atom globule for a profiler (no JSON line)")
    ap.add_argument("--kernels-only", action="store_true",
                    help="only the device-timed builds (for profiler runs): no e2e, extras, stage profile or CPU baseline")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    rank, world, local = dist_init()
    if args.impl == "ours" and (rank == 0 or world == 1):
        import __graft_entry__
        __graft_entry__.build()
    elif args.impl == "reference" and rank == 0:
        # the reference harness only (its cubin from the checkout where present, else the prebuilt one)
        from oracle import refharness
        refharness.build_cubin()
    barrier(world)
    if args.profile_case:
        run_profile_case(args)
    elif args.impl == "reference":
        run_reference(args, rank, world, local)
    else:
        run_ours(args, rank, world, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
