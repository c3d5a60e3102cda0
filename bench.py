"""Benchmark of the SPH-erosion simulation step on one GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--workload plain_1m]

A step is one simulation step (sort, density, forces, integration, terrain
contact, erosion) of every particle of the workload.  The default workload
is the plain scene at scale: 1,048,576 particles over a 1024 x 1024 fBm
terrain (see sph-erosion_gb300/workloads.py).  `value` is particle-steps/s
with the state resident in HBM, each timed step bracketed by CUDA events on
the library's stream and preceded by an L2 flush; `e2e` is the same metric
through the C ABI with a parameter upload and a positions readback to host
memory inside every timed step.  The same line carries, measured in the same
run, the batched form (256 seeded scenes in one system against each scene in
a system of its own) and the served form (a seeded Poisson request trace
through the continuous-batching server, with p50/p99 latency).
`--impl reference` times the reference's algorithm (the oracle's FP32
restatement of FluidSystemSPH::Run, all-pairs) on the host cores over a
bounded sample of the same workload.

With --gpus N > 1 and no launcher around it, bench.py starts N ranks itself
(torch.distributed.run, one process per GPU); the plain scene runs as
replicas, batched scenes and served requests shard across the ranks.
"""
from __future__ import annotations

import argparse
import csv
import hashlib
import json
import os
import socket
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "sph-erosion_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

METRIC = "particle-steps/s"


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def port_calibration():
    """How fast the oracle's FP32 port runs against the reference's own
    FluidSystemSPH::Run on the same host (oracle/port_calibration.json,
    written by oracle/calibrate.py where the reference sources exist): the
    CPU baseline times the port, which is the faster of the two, so the
    reported baseline flatters the reference by this factor."""
    try:
        with open(os.path.join(ROOT, "oracle", "port_calibration.json")) as f:
            return json.load(f)
    except Exception:
        return None


COUNTERS = os.path.join(ROOT, "profiles", "ncu_counters.json")
KERNEL_SOURCES = ("sph_kernels.cu", "sph_kernels.h", "sph_types.h")


def source_digest() -> str:
    """Digest of the kernels' source files: counters captured from another
    build of the kernels are not reported as the current kernels'."""
    h = hashlib.sha256()
    for f in KERNEL_SOURCES:
        with open(os.path.join(ROOT, "sph-erosion_gb300", "csrc", f), "rb") as fh:
            h.update(fh.read())
    return h.hexdigest()[:16]


# The variant bits that select the force kernel (4 register budget, 8 lists,
# 16 list walk loaded ahead, 128 packed records, 256 cooperative pass with
# 512/1024 its group size, 32768 dynamically scheduled warp slices, 131072
# fast arithmetic); the others change only the density pass.
FORCE_BITS = 4 | 8 | 16 | 128 | 256 | 512 | 1024 | 32768 | 131072 | 262144


def variant_bits(kernel, variant):
    """The bits of `variant` that select `kernel`'s code: FORCE_BITS for the
    force pass, all of them for the density pass."""
    return variant & FORCE_BITS if kernel == "k_force" else variant


def ncu_counters(workload, variant, cm, kernel="k_force"):
    """A neighbour kernel's DRAM bytes and warp instructions per launch from
    the committed ncu capture of the same workload, kernel variant, cell
    size and kernel sources; (None, reason) when no capture matches."""
    try:
        with open(COUNTERS) as f:
            entries = json.load(f)["entries"]
    except Exception:
        return None, "no ncu capture committed"
    dig = source_digest()
    want = dict(kernel=kernel, workload=workload, variant_bits=variant_bits(kernel, variant), cell_mult=cm)
    for e in entries:
        if all(e.get(k) == v for k, v in want.items()):
            if e.get("source_digest") != dig:
                return None, f"ncu capture is of other kernel sources ({e.get('source_digest')} vs {dig})"
            return e, None
    return None, f"no ncu capture of {want}"


def ingest_ncu(raw_csv, workload, variant, cm, command, kernel="k_force"):
    """Reads `ncu -i <report> --page raw --csv` output, takes the launches of
    `kernel` (per launch: DRAM bytes read + written, warp instructions,
    duration) and records their mean as the counters of this workload,
    kernel variant, cell size and kernel sources in profiles/."""
    with open(raw_csv, newline="") as f:
        rows = list(csv.reader(f))
    head = rows[0]
    units = rows[1]
    col = {name: i for i, name in enumerate(head)}
    scale = {"byte": 1.0, "Kbyte": 1e3, "Mbyte": 1e6, "Gbyte": 1e9, "KB": 1e3, "MB": 1e6, "GB": 1e9,
             "nsecond": 1e-9, "usecond": 1e-6, "msecond": 1e-3, "second": 1.0, "ns": 1e-9, "us": 1e-6, "ms": 1e-3,
             "s": 1.0, "inst": 1.0, "": 1.0}

    def val(r, name):
        i = col[name]
        u = units[i].strip()
        return float(r[i].replace(",", "")) * scale.get(u, 1.0)

    launches = [r for r in rows[2:] if len(r) == len(head) and kernel in r[col["Kernel Name"]]]
    if not launches:
        raise SystemExit(f"no {kernel} launch in {raw_csv}")
    rd = float(np.mean([val(r, "dram__bytes_read.sum") for r in launches]))
    wr = float(np.mean([val(r, "dram__bytes_write.sum") for r in launches]))
    inst = float(np.mean([val(r, "smsp__inst_executed.sum") for r in launches]))
    dur = float(np.mean([val(r, "gpu__time_duration.sum") for r in launches]))
    try:
        commit = subprocess.run(["git", "-C", ROOT, "rev-parse", "--short", "HEAD"], capture_output=True,
                                text=True).stdout.strip() or None
    except Exception:
        commit = None
    entry = dict(kernel=kernel, workload=workload, variant_bits=variant_bits(kernel, variant), cell_mult=cm,
                 variant=variant, source_digest=source_digest(), git_commit=commit, launches=len(launches),
                 dram_bytes_read=rd, dram_bytes_write=wr, dram_bytes=rd + wr, warp_instructions=inst,
                 ncu_duration_s=dur, command=command)
    try:
        with open(COUNTERS) as f:
            data = json.load(f)
    except Exception:
        data = {"about": "ncu counters of the neighbour kernels per launch (mean over the captured launches), "
                         "read by bench.py for roofline.traffic and issue_roofline; variant_bits are the variant "
                         "bits that select the kernel's code, source_digest identifies the kernel sources "
                         "captured, git_commit the checkout at ingestion", "entries": []}
    key = ("kernel", "workload", "variant_bits", "cell_mult")
    data["entries"] = [e for e in data["entries"] if any(e.get(k) != entry[k] for k in key)] + [entry]
    with open(COUNTERS, "w") as f:
        json.dump(data, f, indent=1)
        f.write("\n")
    print(json.dumps(entry))


class Clocks:
    """Samples nvidia-smi clocks and throttle reasons during the timed region.
    The sampler is started and seen running before the region starts (its
    start-up takes longer than a short region), and the summary covers the
    samples from the region's start through the first one after its end."""

    def __init__(self):
        self.samples = []
        self.proc = None
        self.first = 0

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", os.environ.get("LOCAL_RANK", "0"),
                                          f"--query-gpu={q}", "--format=csv,noheader,nounits", "-lms", "25"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            t0 = time.perf_counter()
            while not self.samples and time.perf_counter() - t0 < 5.0:
                time.sleep(0.01)
            self.first = len(self.samples)
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 7:
                self.samples.append(parts)

    def __exit__(self, *exc):
        if self.proc:
            end = len(self.samples)
            t0 = time.perf_counter()
            while len(self.samples) <= end and time.perf_counter() - t0 < 1.0:
                time.sleep(0.005)
            self.samples = self.samples[self.first:]
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if s[3 + i].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def barrier_max(value, ws):
    """Barrier and max over ranks (replicas only: no data-path collective)."""
    if ws == 1:
        return value
    import torch
    import torch.distributed as dist

    t = torch.tensor([value], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def cpu_sample(spec, budget_s=12.0, nthreads=0):
    """The reference's algorithm (all-pairs FP32, the oracle's restatement of
    FluidSystemSPH::Run) on a bounded sample: the three passes and the
    integration for m particles against all n.  Returns particle-steps/s."""
    import oracle as O

    p = spec["params"]
    bh = p["box_half"]
    prm = O.make_params(g=p["gravity"], dt=p["dt"], p0=p["rest_density"], mass=p["mass"], visc=p["viscosity"],
                        surf_tens=p["surface_tension"], k=p["gas_stiffness"], cr=p["restitution"],
                        h=p["smoothing_radius"], box_l=bh)
    pos = spec["pos"]
    vel = np.zeros_like(pos)
    n = len(pos)
    cores = nthreads if nthreads > 0 else (os.cpu_count() or 1)
    m = min(n, 64)
    t0 = time.perf_counter()
    O.time_sample(prm, pos, vel, n // 2, m, nthreads)
    t = time.perf_counter() - t0
    m2 = int(min(n, max(m, m * budget_s / max(t, 1e-6))))
    i0 = max(0, n // 2 - m2 // 2)
    t0 = time.perf_counter()
    O.time_sample(prm, pos, vel, i0, m2, nthreads)
    t = time.perf_counter() - t0
    return m2 / t, cores, m2, t


def run_reference(args, spec, config):
    """The reference arm: the reference's algorithm on the host cores.  Each
    step is a bounded sample of the workload (the three all-pairs passes and
    the integration of m particles against all n), sized so that the whole
    run, warm-up included, takes about 150 s; `ms_per_step` is that sample
    step's measured time, and the time a step of the whole workload would
    take is reported beside it as an extrapolation.  Rank 0 alone runs."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    import oracle as O

    O.build()
    budget = min(args.ref_seconds, max(0.5, 150.0 / max(args.steps + args.warmup, 1)))
    sizes, times = [], []
    cores = m = 0
    for _ in range(args.warmup):
        cpu_sample(spec, budget_s=budget)
    for _ in range(args.steps):
        _v, cores, m, t = cpu_sample(spec, budget_s=budget)
        sizes.append(m)
        times.append(t)
    val = float(np.sum(sizes) / np.sum(times)) if times else 0.0
    sample = f"{m} of {spec['n']} particles x 3 all-pairs passes + integration per step"
    line = {"metric": METRIC, "value": val, "unit": "particle-steps/s", "impl": "reference", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": float(np.mean(times)) * 1e3,
            "ms_per_step_kind": "measured per sample step (" + sample + ")",
            "ms_per_step_full_workload": spec["n"] / val * 1e3 if val else None,
            "ms_per_step_full_workload_kind": "extrapolated: the whole workload at the sampled rate",
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded lattice + fBm terrain)", "config": config,
            "cpu_baseline": dict({"value": val, "unit": "particle-steps/s", "cores": cores, "kind": "port",
                                  "sample": sample}, **calibration_keys()),
            "e2e": {"value": val, "unit": "particle-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def calibration_keys():
    c = port_calibration()
    if not c:
        return {}
    return {"port_vs_reference": c["port_speed_over_reference"],
            "port_vs_reference_note": c["note"]}


def traversal(scene, step_ms):
    """Neighbour-search counters at the end of the run: per particle, the
    candidates each of the two neighbour passes tests and the in-range pairs
    it evaluates; pair tests per second over the whole step; the spread of
    in-range neighbour counts and the share of particles whose list
    (the library's capacity, self included) overflows, and of
    32-particle warps holding one."""
    import sph_gb300 as S
    cap = S.neighbour_list_capacity()
    t = scene.traversal_stats()
    n = max(t["particles"], 1)
    cnt = scene.neighbour_counts()  # by id; warps hold sorted order
    _, order = scene.debug_sort()
    c = cnt[order] + 1
    over = c > cap
    warps = over[: len(over) // 32 * 32].reshape(-1, 32).any(axis=1) if len(over) >= 32 else over
    return {"candidates_per_particle": t["candidates"] / n, "in_range_per_particle": t["in_range"] / n,
            "rows_per_particle": t["rows"] / n, "pair_tests_per_s": 2 * t["candidates"] / (step_ms * 1e-3),
            "in_range_pairs_per_s": 2 * t["in_range"] / (step_ms * 1e-3),
            "in_range_percentiles": {str(q): int(np.percentile(c, q)) for q in (50, 90, 99, 99.9, 100)},
            "list_capacity": cap, "list_overflow_frac": float(over.mean()),
            "warps_with_overflow_frac": float(warps.mean()),
            "reference_pair_tests_per_step": 3 * n * n}


SPINUP = {"plain_1m": 1000, "plain_small": 500, "skew": 2000, "batched": 500}


def spinup_steps(args, workload=None):
    """Untimed steps before the warm-up: --spinup for the workload the
    command names, the workload's mid-run default otherwise."""
    w = workload or args.workload
    if args.spinup is not None and w == args.workload:
        return args.spinup
    return SPINUP.get(w, 0)


def flush_l2(buf):
    buf.zero_()


def init_dist(ws):
    """Gloo process group for the barrier and the max over ranks (the data
    path has no collective)."""
    if ws > 1:
        import torch.distributed as dist

        if not dist.is_initialized():
            dist.init_process_group("gloo")


def run_long(args, spec, config):
    """The configured run of a plain workload from its first step: --steps
    steps in chunks of --mass-every (16-step graphs, no flush: the rainfall
    state is far larger than L2), each chunk timed with CUDA events and
    followed (untimed) by the exact-mass check of the diagnostics.  One
    line: steps over the summed chunk times, and every check's units."""
    import torch

    import sph_gb300 as S
    import workloads as W

    torch.cuda.set_device(0)
    n = spec["n"]
    with S.System(particle_capacity=n, key_capacity=1 << 20, terrain_capacity=1 << 21, tile=args.tile,
                  graph_steps=16, variant=args.variant) as sysm:
        sc = W.build_scene(sysm, dict(spec, params=dict(spec["params"], cell_mult=args.cell_mult)))
        d0 = sc.diag()
        ms, checks, done = 0.0, [], 0
        with Clocks() as clk:
            while done < args.steps:
                k = min(args.mass_every, args.steps - done)
                ms += sysm.time_steps(k)
                done += k
                d = sc.diag()
                checks.append(int(d["total_units"]))
        line = {"metric": "particle-steps/s of the configured run", "value": n * done / (ms * 1e-3),
                "unit": "particle-steps/s", "n_gpus": 1, "steps": done, "ms_per_step": ms / done,
                "wall_gpu_s": ms / 1e3, "config": dict(config, window=f"steps 1..{done}", l2="state larger than L2",
                                                       variant=args.variant, tile=args.tile, cell_mult=args.cell_mult),
                "mass_checks": {"every": args.mass_every, "total_units": checks,
                                "exact": all(c == 0 for c in checks) and d0["total_units"] == 0},
                "nan_particles": int(d["nan_particles"]), "clocks": clk.summary()}
    print(json.dumps(line), flush=True)


def run_ours(args, spec, config):
    import torch

    import sph_gb300 as S
    import workloads as W

    ws, rank, local = dist_env()
    init_dist(ws)
    torch.cuda.set_device(local)
    n = spec["n"]
    sysm = S.System(particle_capacity=n, key_capacity=1 << 20, terrain_capacity=1 << 21, tile=args.tile,
                    graph_steps=16, device=local, variant=args.variant)
    spec = dict(spec, params=dict(spec["params"], cell_mult=args.cell_mult))
    sc = W.build_scene(sysm, spec)
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=f"cuda:{local}")
    # spin-up to the middle of the configured run (untimed: the flow has
    # collapsed and compressed by then, which is what most of the run's steps
    # look like), warm-up, then the autotuner picks tile, cell size and
    # variant from this state (each trial restarts from a snapshot; the
    # state is restored after)
    spin = spinup_steps(args)
    if args.load_state:
        sc.load(args.load_state)  # a spun-up state saved by --save-state
    elif spin:
        sysm.step(spin)
    if args.save_state:
        sc.save(args.save_state)
    for _ in range(args.warmup):
        sysm.step(1)
    sysm.sync()
    tuned = sysm.autotune(8) if args.autotune else None
    # the state the timed steps start from: the e2e loops below restart from
    # it, so that all three time the same K steps of the flow
    if not args.kernels_only:
        snap_dir = tempfile.mkdtemp(prefix="sph_bench_")
        snap = os.path.join(snap_dir, "timed_start.sphe")
        sc.save(snap)
    torch.cuda.synchronize()
    # timed: K steps, each bracketed by CUDA events on the library stream,
    # an L2 flush before each
    with Clocks() as clk:
        tot = 0.0
        for _ in range(args.steps):
            flush_l2(flush)
            torch.cuda.synchronize()
            tot += sysm.time_steps(1)
        tot_s = barrier_max(tot / 1e3, ws)
    value = ws * n * args.steps / tot_s
    if args.kernels_only:
        sysm.sync()
        return
    # per-stage device times of the same steps (events on the launching stream)
    stages = sysm.profile_stages(max(3, min(args.steps, 10)))
    # e2e: through the C ABI with host buffers, copies inside the timed
    # region.  Each step uploads the parameter block (as the front end
    # re-uploads its edits every frame), runs, and reads the positions back
    # into pinned host memory with the asynchronous readback, whose copies
    # overlap the next step; the clock stops when the last copy is done.
    prm = sc.params()
    host = [S.pinned_empty((n, 3)) for _ in range(2)]
    sc.load(snap)
    sysm.sync()
    t0 = time.perf_counter()
    for k in range(args.steps):
        sc.set_params(prm)
        sysm.step(1)
        sc.get_positions_async(host[k % 2])
    sysm.sync()
    e2e_t = barrier_max(time.perf_counter() - t0, ws)
    e2e = ws * n * args.steps / e2e_t
    # the same with a blocking readback into pageable memory every step
    host_pos = np.zeros((n, 3), np.float32)
    sc.load(snap)
    sysm.sync()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        sc.set_params(prm)
        sysm.step(1)
        sc.get_positions(host_pos)
    e2e_sync = ws * n * args.steps / barrier_max(time.perf_counter() - t0, ws)
    os.remove(snap)
    os.rmdir(snap_dir)
    d = sc.diag()
    dev_bytes = int(sysm.memory())
    trav = traversal(sc, tot / args.steps) if rank == 0 else None
    grid_cells = int(np.prod(sc.grid_dims()[:3]))
    sysm.close()
    del flush
    torch.cuda.empty_cache()
    # the batched and served forms, in the same run
    extras = {}
    if args.extras and spec["name"] == "plain_1m":
        # the served arm runs the kernels the plain scene's tuning picked (the
        # server has no tuner of its own); the batched arm tunes itself
        args.serve_variant = tuned["variant"] if tuned else args.variant
        base_cfg = {"h": W.H, "dt": W.PHYS["dt"], "erosion": True, "tile": args.tile, "cell_mult": args.cell_mult}
        extras["batched"] = run_batched(args, base_cfg, embedded=True)
        extras["serving"] = run_serving(args, base_cfg, embedded=True)
    if rank != 0:
        return
    # rooflines of the two neighbour kernels; the line's `roofline` is the
    # one with the longer measured stage time.  Algorithmic bytes: density
    # pass 16 B read (sorted position) + 16 B written (density factors) per
    # particle; force pass 48 B read (sorted position, velocity, density
    # factors) + 32 B written (position, velocity) per particle + 4 B per
    # terrain height read
    hbm, kind = peaks()
    t = spec.get("terrain")
    texels = t["w"] * t["d"] if t else 0
    step_ms = tot / args.steps
    step_bytes = 88.0 * n + 16.0 * grid_cells + 20.0 * texels
    cpu_v, cores, m, _ = cpu_sample(spec, budget_s=args.ref_seconds)
    variant = tuned["variant"] if tuned else args.variant if args.variant is not None else 88
    cm = tuned["cell_mult"] if tuned else args.cell_mult
    clk_sum = clk.summary()
    roofs, issues = {}, {}
    for kernel, ms, alg in (("k_density", float(stages[4]), 32.0 * n), ("k_force", float(stages[5]), 80.0 * n + 4.0 * texels)):
        cnt, why = ncu_counters(config["workload"], variant, cm, kernel)
        achieved = alg / (ms * 1e-3) / 1e9
        roofs[kernel] = {"bound": "hbm", "kernel": kernel, "achieved": achieved, "peak": hbm, "unit": "GB/s",
                         "frac": achieved / hbm, "traffic": cnt["dram_bytes"] if cnt else None,
                         "traffic_source": (f"ncu capture {cnt['source_digest']} ({cnt['command']})" if cnt else why),
                         "algorithmic_bytes": alg, "peak_kind": kind, "stage_ms": ms}
        issues[kernel] = issue_roofline(cnt, ms, clk_sum, kernel)
    dominant = max(roofs, key=lambda k: roofs[k]["stage_ms"])
    line = {
        "metric": METRIC, "value": value, "unit": "particle-steps/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": step_ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded lattice + fBm terrain)",
        "config": config,
        "roofline": dict(roofs[dominant], step_bytes_frac=step_bytes / (step_ms * 1e-3) / 1e9 / hbm),
        "issue_roofline": issues[dominant],
        "rooflines": {k: {"hbm": roofs[k], "issue": issues[k]} for k in roofs},
        "cpu_baseline": dict({"value": cpu_v, "unit": "particle-steps/s", "cores": cores, "kind": "port",
                              "sample": f"{m} of {n} particles x 3 all-pairs passes + integration per step"},
                             **calibration_keys()),
        "e2e": {"value": e2e, "unit": "particle-steps/s", "h2d_bytes_per_step": int(C_PARAMS_BYTES),
                "d2h_bytes_per_step": int(n * 12), "readback": "asynchronous into pinned memory, overlapped"},
        "e2e_sync": {"value": e2e_sync, "unit": "particle-steps/s", "h2d_bytes_per_step": int(C_PARAMS_BYTES),
                     "d2h_bytes_per_step": int(n * 12), "readback": "blocking into pageable memory"},
        "gpu_launches": int(args.steps * (7 if t else 6)),
        "stages_ms": {name: float(v) for name, v in zip(S.STAGES, stages)},
        "clocks": clk_sum,
        "device_bytes": dev_bytes,
        "mass_units_total": int(d["total_units"]),
        "diag_fp64": {"kinetic": d["kinetic"], "potential": d["potential"], "momentum": d["momentum"],
                      "nan_particles": d["nan_particles"]},
        "tuned": tuned,
        "traversal": trav,
    }
    line.update(extras)
    if extras:
        line["config"] = dict(config, batched=extras["batched"]["config"]["scenes_desc"],
                              serving=extras["serving"]["config"]["trace_desc"])
    print(json.dumps(line), flush=True)


# Host-to-device bytes of a parameter upload: the scene descriptor (248 B)
# and its step budget (4 B) that set_params copies to the device.
C_PARAMS_BYTES = 248 + 4


def issue_roofline(cnt, ms, clocks, kernel):
    """A neighbour kernel against the instruction-issue peak: warp
    instructions per launch (the ncu capture of the same workload, kernel
    variant, cell size and sources) over the live CUDA-event time, against 4
    per cycle per SM at the sampled SM clock."""
    inst = cnt["warp_instructions"] if cnt else None
    if inst is None or not ms:
        return None
    import torch

    sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    mhz = clocks.get("sm_mhz") or clocks.get("sm_max_mhz") or 2070.0
    peak = 4.0 * sms * mhz * 1e6
    achieved = inst / (ms * 1e-3)
    return {"kernel": kernel, "achieved": achieved, "peak": peak, "unit": "warp-instructions/s",
            "frac": achieved / peak, "warp_instructions_per_launch": inst, "source": "ncu smsp__inst_executed.sum"}


def _init_ranks():
    """Rank setup of the batched and served modes: scenes shard across ranks
    (no data-path collective), gloo carries the final metric reduction."""
    import torch

    ws, rank, local = dist_env()
    init_dist(ws)
    torch.cuda.set_device(local)
    return ws, rank, local


def _gather(value, ws):
    if ws == 1:
        return [value]
    import torch.distributed as dist

    out = [None] * ws
    dist.all_gather_object(out, value)
    return out


def run_batched(args, config, embedded=False):
    """Batched form vs plain form on the same seeded scenes: all scenes in one
    system (one launch per stage for all of them, 16-step CUDA graphs) against
    each scene alone in its own system, timed scene after scene.  With N ranks
    each rank runs its cost-balanced share of the scenes.  Returns the
    result on rank 0 (embedded) or prints it as a line of its own."""
    import shard
    import sph_gb300 as S
    import workloads as W

    ws, rank, local = _init_ranks()
    all_reqs = W.batched_requests(args.scenes)
    reqs = shard.shard_requests(all_reqs, ws, rank)
    total = sum(r["particles"] for r in reqs)
    total_all = sum(r["particles"] for r in all_reqs)
    base = W.base_params(args.cell_mult)
    sysm = S.System(particle_capacity=total + 512 * len(reqs), key_capacity=1 << 24, terrain_capacity=1 << 24,
                    tile=args.tile, graph_steps=16, device=local, variant=args.variant)
    scenes = [sysm.scene_from_request(base, r) for r in reqs]
    # spin-up (untimed), the autotuner's pick (it restores the state it
    # started from), then each scene's state is checkpointed so that the
    # plain form starts every scene from the same state and runs the same
    # warm-up and timed steps with the same kernels
    spin = spinup_steps(args, "batched")
    tmp = tempfile.mkdtemp(prefix="sph_bench_")
    if spin:
        sysm.step(spin)
    sysm.sync()
    tuned = sysm.autotune(4) if args.autotune else None
    paths = []
    for k, sc in enumerate(scenes):
        paths.append(os.path.join(tmp, f"scene{k}.sphe"))
        sc.save(paths[-1])
    sysm.step(args.warmup)
    sysm.sync()
    if args.kernels_only:
        sysm.step(args.steps)
        sysm.sync()
        sysm.close()
        for path in paths:
            os.remove(path)
        os.rmdir(tmp)
        return None
    d0 = sysm.diag_many(scenes)
    with Clocks() as clk:
        ms = barrier_max(sysm.time_steps(args.steps), ws)
    d1 = sysm.diag_many(scenes)
    batched = total_all * args.steps / (ms * 1e-3)
    bad = sum(1 for d in d1 if d["total_units"] != 0 or d["nan_particles"] != 0)
    # per-stage CUDA-event times of a few more steps (after the fingerprints)
    stages = sysm.profile_stages(max(3, min(args.steps, 10)))
    sysm.close()
    # plain form: one system per scene, same steps, same tuned tile and cell
    tile = tuned["tile"] if tuned else args.tile
    cm = tuned["cell_mult"] if tuned else args.cell_mult
    variant = tuned["variant"] if tuned else args.variant
    plain_ms = 0.0
    same = 0
    for r, path, a in zip(reqs, paths, d1):
        with S.System(particle_capacity=r["particles"], tile=tile, graph_steps=16, device=local,
                      variant=variant) as one:
            sc1 = one.scene_from_request(W.base_params(cm), r)
            sc1.load(path)
            os.remove(path)
            one.step(args.warmup)
            one.sync()
            plain_ms += one.time_steps(args.steps)
            # the scene alone ends where it ended in the batch, bit for bit
            same += int(sc1.diag()["state_hash"] == a["state_hash"])
    os.rmdir(tmp)
    plain_ms = barrier_max(plain_ms, ws)
    plain = total_all * args.steps / (plain_ms * 1e-3)
    same = sum(_gather(same, ws))
    bad = sum(_gather(bad, ws))
    if rank != 0:
        return None
    window = (f"steps {spin + args.warmup + 1}..{spin + args.warmup + args.steps} after {spin} untimed spin-up "
              f"steps")
    desc = (f"{len(all_reqs)} seeded scenes, {total_all} particles (2,048-131,072 each, log-uniform), "
            f"terrain sides 64-512, {window}")
    res = {"metric": METRIC, "value": batched, "unit": "particle-steps/s", "n_gpus": ws, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
           "scaling": "strong", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded scenes)",
           "config": dict(config, workload="batched", scenes=len(all_reqs), particles=total_all, window=window,
                          parallelism=f"scenes sharded over {ws} rank(s)", scenes_desc=desc,
                          l2="inputs larger than L2 (%.0f MB of particle state)" % (total_all * 100 / 1e6)),
           "plain_value": plain, "batched_over_plain": batched / plain, "plain_ms_per_step": plain_ms / args.steps,
           "alone_equals_batched": f"{same} of {len(all_reqs)} scenes (state fingerprint after the timed steps)",
           "mass_violations": bad, "tuned": tuned, "clocks": clk.summary(),
           "stages_ms": {name: float(v) for name, v in zip(S.STAGES, stages)}}
    if embedded:
        return {k: res[k] for k in ("value", "unit", "ms_per_step", "plain_value", "plain_ms_per_step",
                                    "batched_over_plain", "alone_equals_batched", "mass_violations", "tuned",
                                    "clocks", "config", "stages_ms")}
    print(json.dumps(res), flush=True)
    return None


def run_serving(args, config, embedded=False):
    """Served form: a Poisson request trace replayed in real time through the
    continuous-batching server.  With N ranks each rank serves its
    cost-balanced share of the trace; throughput is the job's particle-steps
    over the slowest rank's wall time, latencies are pooled.  Returns the
    result on rank 0 (embedded) or prints it as a line of its own."""
    import shard
    import sph_gb300 as S
    import workloads as W

    ws, rank, local = _init_ranks()
    full = W.serving_trace(args.requests, rate=args.rate)
    trace = shard.shard_requests(full, ws, rank)
    variant = getattr(args, "serve_variant", None) or args.variant or 0
    with Clocks() as clk, S.Server(W.base_params(args.cell_mult), tile=args.tile, chunk_steps=16,
                                    hbm_budget=120 << 30, device=local, policy=1 if args.policy == "work" else 0,
                                    max_active_particles=args.max_active, variant=variant) as srv:
        res, st = srv.run_trace(trace)
    lat = [r.done_s - r.arrival_s for r in res]
    bad = sum(1 for r in res if r.total_units != 0 or r.nan_particles != 0)
    parts = _gather(dict(lat=lat, bad=bad, ps=st["particle_steps"], wall=st["wall_s"], peak=st["peak_active"],
                         peak_p=st["peak_particles"], peak_b=st["peak_bytes"], chunks=st["chunks"],
                         phases={k: st[k] for k in ("admit_s", "prepare_s", "gpu_wait_s", "retire_s")}), ws)
    if rank != 0:
        return None
    lat = np.sort(np.concatenate([np.asarray(q["lat"]) for q in parts]))

    def pct(q):
        return float(lat[min(len(lat) - 1, max(0, int(np.ceil(q * len(lat))) - 1))])

    wall = max(q["wall"] for q in parts)
    ps = sum(q["ps"] for q in parts)
    desc = (f"{len(full)} seeded requests, Poisson at {args.rate:g}/s, 4,096-262,144 particles, "
            f"100-2,000 steps, 120 GB budget, admission {args.policy}")
    out = {"metric": METRIC, "value": ps / wall, "unit": "particle-steps/s", "n_gpus": ws,
           "steps": int(sum(r["steps"] for r in full)), "warmup": 0, "ms_per_step": None,
           "higher_is_better": True, "scaling": "strong", "vs_baseline": None, "dtype": "f32",
           "data": "synthetic (seeded Poisson request trace)",
           "config": dict(config, workload="serving", requests=len(full), rate_per_s=args.rate,
                          hbm_budget_gb=120, parallelism=f"requests sharded over {ws} rank(s)",
                          policy=args.policy, max_active_particles=args.max_active, variant=variant,
                          trace_desc=desc),
           "p50_latency_s": pct(0.50), "p99_latency_s": pct(0.99), "max_latency_s": float(lat[-1]),
           "requests": int(len(lat)), "wall_s": wall, "peak_active": max(q["peak"] for q in parts),
           "peak_particles": max(q["peak_p"] for q in parts), "peak_bytes": max(q["peak_b"] for q in parts),
           "chunks": sum(q["chunks"] for q in parts), "mass_violations": sum(q["bad"] for q in parts),
           "host_phases_s": parts[0]["phases"],
           "clocks": clk.summary()}
    if embedded:
        return {k: out[k] for k in ("value", "unit", "p50_latency_s", "p99_latency_s", "max_latency_s", "requests",
                                    "wall_s", "peak_active", "peak_particles", "mass_violations", "host_phases_s",
                                    "clocks", "config")}
    print(json.dumps(out), flush=True)
    return None


def free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def launch_ranks(n):
    """Re-executes this command as n ranks, one process per GPU, through
    torch.distributed.run; returns its exit status."""
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={n}",
           "--master-addr", "127.0.0.1", "--master-port", str(free_port()), os.path.abspath(__file__),
           *sys.argv[1:]]
    return subprocess.run(cmd).returncode


def dry_run(args):
    """The rank plumbing without CUDA: every rank takes part in the barrier
    and the max over ranks; rank 0 prints what the real line's rank fields
    would hold."""
    ws, rank, _ = dist_env()
    init_dist(ws)
    t = barrier_max(0.001 * (rank + 1), ws)
    if rank == 0:
        print(json.dumps({"dry_run": True, "impl": args.impl, "n_gpus": ws, "steps": args.steps,
                          "warmup": args.warmup, "max_over_ranks_s": t, "workload": args.workload}), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="plain_1m",
                    choices=["plain_1m", "plain_small", "batched", "serving", "skew"])
    ap.add_argument("--no-autotune", dest="autotune", action="store_false",
                    help="keep --tile/--cell-mult instead of autotuning them")
    ap.add_argument("--tile", type=int, default=256)
    ap.add_argument("--variant", type=int, default=None,
                    help="kernel variant bits of the plain workloads (before autotuning)")
    ap.add_argument("--cell-mult", type=float, default=0.5)
    ap.add_argument("--ref-seconds", type=float, default=12.0)
    ap.add_argument("--scenes", type=int, default=256, help="batched: number of scenes")
    ap.add_argument("--requests", type=int, default=400, help="serving: requests in the trace")
    ap.add_argument("--long", action="store_true",
                    help="plain workloads: the configured run from step 1 (--steps steps, no spin-up), in timed "
                         "chunks with an exact-mass check after each (e.g. --workload skew --steps 10000)")
    ap.add_argument("--mass-every", type=int, default=500, help="with --long: steps between mass checks")
    ap.add_argument("--rate", type=float, default=200.0, help="serving: mean arrivals per second")
    ap.add_argument("--policy", default="work", choices=["arrival", "work"],
                    help="serving: admission order among arrived requests (least work first by default)")
    ap.add_argument("--max-active", type=int, default=40_000_000,
                    help="serving: cap on resident particles (0 = none; the budget alone)")
    ap.add_argument("--particles", type=int, default=8388608, help="skew: particles (the box floor scales with them)")
    ap.add_argument("--spinup", type=int, default=None,
                    help="untimed steps before the warm-up (default: to mid-run; plain_1m 1000 of its 2000 steps, "
                         "skew 2000, batched 500, plain_small 500)")
    ap.add_argument("--save-state", default=None, help="plain workloads: checkpoint the scene after the spin-up")
    ap.add_argument("--load-state", default=None,
                    help="plain workloads: start from a checkpoint instead of the spin-up (short profiler runs)")
    ap.add_argument("--kernels-only", action="store_true",
                    help="warm-up and timed steps only (for profiler captures); prints nothing")
    ap.add_argument("--no-extras", dest="extras", action="store_false",
                    help="plain_1m: leave out the batched and served forms measured in the same run")
    ap.add_argument("--dry-run", action="store_true",
                    help="rank plumbing only, without CUDA: each rank joins the barrier, rank 0 prints n_gpus")
    ap.add_argument("--ingest-ncu", default=None, metavar="RAW_CSV",
                    help="record a neighbour kernel's counters from `ncu -i REPORT --page raw --csv` output for "
                         "--workload/--variant/--cell-mult into profiles/ncu_counters.json")
    ap.add_argument("--ingest-command", default="", help="with --ingest-ncu: the capture command, as run")
    ap.add_argument("--ingest-kernel", default="k_force", choices=("k_force", "k_density"),
                    help="with --ingest-ncu: the kernel whose launches to record")
    args = ap.parse_args()
    if args.ingest_ncu:
        ingest_ncu(args.ingest_ncu, args.workload, args.variant if args.variant is not None else 88, args.cell_mult,
                   args.ingest_command, args.ingest_kernel)
        return
    if "WORLD_SIZE" not in os.environ and args.gpus > 1:
        sys.exit(launch_ranks(args.gpus))
    ws = dist_env()[0]
    if "WORLD_SIZE" in os.environ and ws != args.gpus:
        print(f"bench: --gpus {args.gpus} but WORLD_SIZE={ws}; n_gpus reports the ranks running", file=sys.stderr)
    if args.dry_run:
        dry_run(args)
        return
    import workloads as W

    if args.workload in ("batched", "serving") and args.impl == "ours":
        cfg = {"h": W.H, "dt": W.PHYS["dt"], "erosion": True, "tile": args.tile, "cell_mult": args.cell_mult}
        (run_batched if args.workload == "batched" else run_serving)(args, cfg)
        return
    spec = {"plain_small": W.plain_small, "skew": lambda: W.skew_rain(args.particles)}.get(args.workload, W.plain_1m)()
    t = spec.get("terrain")
    config = {"workload": spec["name"], "particles": spec["n"],
              "terrain": f"{t['w']}x{t['d']} fBm {t['octaves']} oct amp {t['amplitude']}" if t else None,
              "box": "x".join(str(2 * b) for b in spec["params"]["box_half"]), "h": spec["params"]["smoothing_radius"],
              "dt": spec["params"]["dt"], "erosion": bool(spec["params"]["erosion"]), "resort": "every step",
              "l2": "flushed (512 MiB write) before every timed step",
              "window": f"steps {spinup_steps(args) + args.warmup + 1}..{spinup_steps(args) + args.warmup + args.steps} "
                        f"after {spinup_steps(args)} untimed spin-up steps"}
    if args.impl == "reference":
        run_reference(args, spec, config)
    elif args.long:
        run_long(args, spec, config)
    else:
        run_ours(args, spec, config)


if __name__ == "__main__":
    main()
