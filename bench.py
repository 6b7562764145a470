#!/usr/bin/env python3
"""World-step benchmark (one JSON line on rank 0).

Workload: the plain drop-in world step at full size -- a 2048x2048 world
with a 2048x2048 fluid grid, multigrid pressure on 8 levels down to 16x16
with 4 V-cycles of 3+3 red-black Gauss-Seidel sweeps (30 sweeps on the
coarsest level), monomer transport and the exact-mass ledger every step,
on seeded synthetic inputs (value-noise velocity, 10% rock, Poisson(4)
monomers in 8 fields).  A step is one full world step (fluid + pressure +
transport + ledger) of one world.

  value  world-steps/s, device time (CUDA events on the world's stream),
         state resident in HBM (~0.7 GB, larger than L2: every step
         streams it, so no L2 flush is needed between steps)
  e2e    the same metric through the public API with host buffers: per
         step, SimParams go host->device and the step's ledger comes back
         device->host and is checked against the seeded counts
  --impl reference   the CPU restatement of the reference's passes (the
         reference itself is Rust + WGSL on wgpu and cannot run here),
         all host threads, bounded sample of the same workload
  batched  (N = 1) 64 worlds of uneven sizes as one ribo_batch vs the same
         worlds stepped one after another: world-steps/s and p50/p99 step
         latency of each form
  serving  (N = 1) the continuous-batching server fed by a Poisson request
         stream (200 req/s for 60 s, 150 GB budget), and again at a rate the
         GPU sustains: world-steps/s, p50/p99 step and job latency
  mixed_precision  (N = 1) the same step with the pressure solved to a
         relative residual of 1e-5 every step; residual re-checked in FP64
  --ncu-case   seed the world and run --steps steps with nothing else (a
         short program for ncu captures; prints nothing)
  --ncu-terrain  the same with the terrain block on (10% rubble, grains
         settling), for captures of the terrain kernels
N > 1 GPUs run independent replicas (one world per rank, no collective).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "ribossome-v2_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

METRIC = "world-steps/s at 2048^2"
UNIT = "world-steps/s"
FALLBACK_HBM_GBS = 6800.0


def workload_config(n):
    return {
        "workload": f"plain world step {n}x{n} (fluid {n}x{n}), multigrid 8 levels to 16x16, 4 V-cycles of 3+3 "
                    "red-black GS sweeps, 30 coarse sweeps, transport + exact ledger every step",
        "grid": [n, n], "fluid": [n, n], "mg_min_size": 16, "mg_cycles": 4, "mg_pre": 3, "mg_post": 3,
        "mg_coarse": 30, "fluid_substep": 1, "transport_every": 1, "dt": 1.0,
        "inputs": "seeded synthetic: 4-octave value-noise velocity (max 0.5 cells/step), 10% rock, "
                  "Poisson(4) monomers x 8 fields",
        "l2": "inputs larger than L2: ~0.7 GB of resident world state streamed every step",
    }


def reference_pass_bytes(n, cycles=4, pre=3, post=3):
    """Bytes per step of the reference's pass structure (every smoother sweep
    a full read/write pass), per fluid cell F and env cell G at F = G = n:
    non-multigrid fluid 237, multigrid 18 + 8 + cycles * 4/3 * (13 (pre + post)
    + 11.25 + 10), transport 28 + 57 + 16 (ledger)."""
    cells = float(n) * n
    mg = 18.0 + 8.0 + cycles * (4.0 / 3.0) * (13.0 * (pre + post) + 11.25 + 10.0)
    return cells * (237.0 + mg) + cells * (28.0 + 57.0 + 16.0)


def read_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


def profile_traffic(kernel):
    """dram bytes per launch of `kernel` from the committed ncu summaries."""
    pdir = os.path.join(ROOT, "profiles")
    if not os.path.isdir(pdir):
        return None
    for name in sorted(os.listdir(pdir)):
        if not name.endswith((".txt", ".md")):
            continue
        for line in open(os.path.join(pdir, name)):
            parts = line.split()
            if len(parts) >= 3 and parts[0] == "traffic_bytes_per_launch:" and parts[1] == kernel:
                try:
                    return float(parts[2])
                except ValueError:
                    pass
    return None


class Clocks:
    """nvidia-smi sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for k, name in enumerate(names):
                if f[5 + k].lower().startswith("active"):
                    reasons.add(name)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def loaded_native_libraries():
    """The repository's shared libraries mapped into this process (Linux)."""
    out = set()
    try:
        for line in open("/proc/self/maps"):
            path = line.split()[-1]
            if path.endswith(".so") and path.startswith(ROOT):
                out.add(os.path.relpath(path, ROOT))
    except OSError:
        pass
    return sorted(out)


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist

        dist.barrier()


def max_over_ranks(ws, v):
    if ws == 1:
        return v
    import torch
    import torch.distributed as dist

    t = torch.tensor([v], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(ws, v):
    if ws == 1:
        return v
    import torch
    import torch.distributed as dist

    t = torch.tensor([v], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def oracle_world(n):
    """The CPU restatement seeded with the workload's inputs and SimParams.

    Its parameters come from the restatement's own table of the reference
    defaults (ribo_oracle.default_params), so a CPU-only run never loads
    the CUDA library; ribo_world supplies only the ABI struct layouts,
    which it reads from the C header."""
    import ribo_oracle
    import synth

    o = ribo_oracle.OracleWorld(n, seed=1000, mg_min_size=16, mg_pre=3, mg_post=3)
    o.seed_inputs(synth.make_world_inputs(n, seed=1000))
    o.params = synth.bench_params(1000, defaults=ribo_oracle.default_params)
    o.settings.fluid_substep = 1
    o.settings.mg_cycles = 4
    return o


def cpu_sample(n, seconds_budget=15.0, max_steps=20):
    """The oracle (CPU restatement) on the host cores: a bounded sample of the workload."""
    import ribo_oracle

    threads = os.cpu_count() or 1
    ribo_oracle.set_threads(threads)
    o = oracle_world(n)
    o.encode_steps(1)  # warm-up
    t = time.perf_counter()
    o.encode_steps(1)
    one = time.perf_counter() - t
    steps = int(max(1, min(max_steps, seconds_budget / max(one, 1e-6))))
    t = time.perf_counter()
    done = 0
    while done < steps:
        k = min(64, steps - done)
        o.encode_steps(k)
        done += k
    el = time.perf_counter() - t
    return {"value": steps / el, "unit": UNIT, "cores": ribo_oracle.get_threads(), "kind": "port",
            "sample": f"{steps} full world steps of the {n}x{n} workload after 2 untimed steps ({el:.1f} s)"}


def run_reference(args):
    ws, rank, _ = int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")), 0
    if rank != 0:
        return
    import ribo_oracle

    n = args.size
    threads = os.cpu_count() or 1
    ribo_oracle.set_threads(threads)
    o = oracle_world(n)
    warm = max(args.warmup, 4)
    for _ in range(warm):
        o.encode_steps(1)
    t = time.perf_counter()
    o.encode_steps(1)
    one = time.perf_counter() - t
    steps = int(max(1, min(args.steps - 1, args.reference_seconds / max(one, 1e-6))))
    t = time.perf_counter()
    done = 0
    while done < steps:
        k = min(64, steps - done)
        o.encode_steps(k)
        done += k
    el = time.perf_counter() - t + one
    steps += 1
    value = steps / el
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": steps,
        "warmup": warm, "ms_per_step": 1000.0 * el / steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+u32", "data": "synthetic", "config": dict(workload_config(n), parallelism=f"replicas x{ws}" if ws > 1 else "single world"),
        "native_libraries": loaded_native_libraries(),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": ribo_oracle.get_threads(), "kind": "port",
                         "sample": f"{steps} of the {args.steps} requested full world steps ({el:.1f} s); the "
                                   "reference (Rust + WGSL via wgpu) cannot run without a graphics stack, so its "
                                   "passes run as the C++ restatement"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_ours(args):
    ws, rank, local = dist_setup()
    import ribo_world as rw
    import synth

    n = args.size
    seed = 1000 + rank
    inputs = synth.make_world_inputs(n, seed=seed)
    w = rw.World(n, seed=seed, mg_min_size=16, mg_pre=3, mg_post=3, device=local)
    w.settings.fluid_substep = 1
    w.settings.mg_cycles = 4
    w.settings.ledger_each_step = 1

    def reset():
        """Every measured phase starts from the same seeded state at epoch 0."""
        w.seed_inputs(inputs)
        w.params = synth.bench_params(seed)

    reset()
    seeded_led = rw.Ledger.from_cells(inputs[rw.CHEM])
    seeded = [seeded_led.channel(c) for c in range(4)]

    def conserved(led):
        return [led.channel(c) for c in range(4)] == seeded

    def run_steps(k, timing=False, acc=None):
        done = 0
        while done < k:
            c = min(rw.MAX_STEPS_PER_FRAME, k - done)
            w.encode_steps(c)
            done += c
            if timing:
                for name, launches, ms, b in w.read_kernel_timing():
                    e = acc.setdefault(name, [0, 0.0, 0.0])
                    e[0] += launches
                    e[1] += ms
                    e[2] += b
            ledgers = w.step_ledgers(c)
            if not all(conserved(l) for l in ledgers):
                raise RuntimeError("matter not conserved")

    # Steady state: the warm-up and the timed region issue one step per call,
    # the call shape of the end-to-end loop below.  A call shape is captured
    # into a CUDA graph the second time it is seen (the key holds the
    # parameter slot and the chem ping-pong side, which alternate), so from
    # the fifth warm-up call on every call replays a graph.
    warm = max(args.warmup, 4)
    for _ in range(warm):
        w.encode_steps(1)
    w.sync()
    barrier(ws)

    # ---- device-timed region: K one-step calls, no host sync inside ----
    clocks = Clocks(local)
    clocks.start()
    launches0 = rw.kernel_launch_count()
    w.mark(0)
    for _ in range(args.steps):
        w.encode_steps(1)
    w.mark(1)
    ms = w.elapsed_ms(0, 1)
    launches = rw.kernel_launch_count() - launches0
    clk = clocks.stop()
    # the ledger kernel ran every step; the last one must hold the seeded counts
    if not conserved(w.step_ledgers(1)[0]):
        raise RuntimeError("matter not conserved (timed region)")
    barrier(ws)
    ms_max = max_over_ranks(ws, ms)
    value = args.steps * ws / (ms_max / 1000.0)

    # ---- per-kernel CUDA events (a separate pass: events between launches
    # would perturb the timed region above) ----
    prof_steps = max(1, min(args.steps, args.profile_steps))
    reset()
    run_steps(max(args.warmup, 3))
    w.enable_kernel_timing(True)
    kern = {}
    run_steps(prof_steps, timing=True, acc=kern)
    w.enable_kernel_timing(False)

    # ---- end to end through the public API, host buffers ----
    e2e_steps = max(1, min(args.steps, args.e2e_steps))
    reset()
    for _ in range(warm):
        w.encode_steps(1)
        w.step_ledgers(1)
    w.sync()
    barrier(ws)
    t = time.perf_counter()
    for _ in range(e2e_steps):
        w.encode_steps(1)
        led = w.step_ledgers(1)[0]
        if not conserved(led):
            raise RuntimeError("matter not conserved (e2e)")
    el = time.perf_counter() - t
    el = max_over_ranks(ws, el)
    e2e = {"value": e2e_steps * ws / el, "unit": UNIT, "h2d_bytes_per_step": 464, "d2h_bytes_per_step": 48,
           "note": "per step: SimParams host->device (encode_steps), then the step's ledger device->host and "
                   "checked against the seeded per-channel counts; wall clock"}

    # ---- roofline of the dominant kernel ----
    peak, peak_kind = read_peaks()
    top = max(kern.items(), key=lambda kv: kv[1][1])
    name, (nl, tms, tb) = top
    avg_ms = tms / nl
    bpl = tb / nl
    achieved = bpl / (avg_ms * 1e-3) / 1e9
    traffic = profile_traffic(name)
    step_bytes = sum(v[2] for v in kern.values()) / prof_steps
    roofline = {"bound": "hbm", "kernel": name, "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "traffic": traffic, "peak_source": f"{peak_kind} hbm_gbs (copy)",
                "bytes_per_launch": bpl, "avg_launch_ms": avg_ms,
                "share_of_step": tms / max(sum(v[1] for v in kern.values()), 1e-9)}
    step_s = ms / args.steps * 1e-3
    ref_bytes = reference_pass_bytes(n)
    step_rl = {"bytes_per_step": step_bytes, "achieved": step_bytes / step_s / 1e9,
               "frac": step_bytes / step_s / 1e9 / peak,
               "note": "compulsory bytes of this implementation's passes (fused smoothers move a box once per 3 sweeps)",
               "reference_pass_bytes_per_step": ref_bytes,
               "reference_pass_achieved": ref_bytes / step_s / 1e9,
               "reference_pass_frac": ref_bytes / step_s / 1e9 / peak}
    # [pass, ms per step, launches per step, algorithmic GB/s], every pass
    breakdown = sorted(((k, v[1] / prof_steps, v[0] // prof_steps, v[2] / max(v[1], 1e-9) / 1e6) for k, v in kern.items()),
                       key=lambda x: -x[1])

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": warm, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+u32", "data": "synthetic",
        "config": dict(workload_config(n), parallelism=f"replicas x{ws}" if ws > 1 else "single world"),
        "e2e": e2e, "gpu_launches": launches, "roofline": roofline, "step_roofline": step_rl,
        "kernels_ms_per_step": [[k, round(t, 4), c, round(g, 1)] for k, t, c, g in breakdown],
        "clocks": clk,
    }
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_sample(n)
    # batched and served forms: single-GPU runs only (replicas would repeat them per rank)
    if ws == 1 and not args.no_extras:
        line["next_rows"] = run_extras(args, w)
    if ws == 1 and not args.no_mixed:
        w.close()
        line["mixed_precision"] = run_mixed(args, local)
    if ws == 1 and not args.no_batched:
        w.close()
        line["batched"] = run_batched(args, local)
        if not args.no_mixed and args.batched_mixed_steps > 0:
            line["batched"]["mixed"] = run_batched(args, local, precision_mode=1, steps=args.batched_mixed_steps)
    if ws == 1 and not args.no_serving:
        line["serving"] = run_serving(args, local, args.serve_rate, args.serve_seconds, args.serve_drain_seconds)
        if args.serve_sustainable_rate > 0:
            line["serving_sustainable"] = run_serving(args, local, args.serve_sustainable_rate,
                                                      args.serve_sustainable_seconds, args.serve_sustainable_seconds)
    line["headlines"] = headlines(line)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


def headlines(line):
    """The figures of every section in a few keys, printed last on the line
    so that a reader of only its tail sees them."""
    def r(v, k=4):
        return None if v is None else round(float(v), k)

    h = {"plain_world_steps_per_s": r(line["value"], 1), "plain_e2e_world_steps_per_s": r(line["e2e"]["value"], 1),
         "plain_ms_per_step": r(line["ms_per_step"]), "dominant_kernel": line["roofline"].get("kernel"),
         "dominant_kernel_hbm_frac": r(line["roofline"]["frac"]),
         "step_hbm_frac_reference_pass_bytes": r(line["step_roofline"]["reference_pass_frac"])}
    cpu = line.get("cpu_baseline")
    if cpu:
        h["cpu_baseline_world_steps_per_s"] = r(cpu["value"], 3)
    mp = line.get("mixed_precision")
    if mp:
        h["mixed_world_steps_per_s"] = r(mp["world_steps_per_s"], 1)
        h["mixed_rel_residual_fp64_host"] = mp["rel_residual_fp64_host"]
        h["mixed_tolerance"] = mp["tolerance"]
    bt = line.get("batched")
    if bt:
        h["batched_world_steps_per_s"] = r(bt["batched"]["world_steps_per_s"], 1)
        h["plain_loop_world_steps_per_s"] = r(bt["plain"]["world_steps_per_s"], 1)
        h["batched_speedup"] = r(bt["speedup"], 3)
        h["batched_step_ms_p50_p99"] = [r(bt["batched"]["step_latency_ms_p50"], 3), r(bt["batched"]["step_latency_ms_p99"], 3)]
        h["plain_step_ms_p50_p99"] = [r(bt["plain"]["step_latency_ms_p50"], 3), r(bt["plain"]["step_latency_ms_p99"], 3)]
        if bt.get("mixed"):
            h["batched_mixed_speedup"] = r(bt["mixed"].get("speedup"), 3)
            h["batched_mixed_world_steps_per_s"] = r(bt["mixed"]["batched"]["world_steps_per_s"], 1)
    for key in ("serving", "serving_sustainable"):
        sv = line.get(key)
        if sv:
            h[key] = {"world_steps_per_s": r(sv["world_steps_per_s"], 1), "step_ms_p50": r(sv["step_latency_ms_p50"], 3),
                      "step_ms_p99": r(sv["step_latency_ms_p99"], 3), "completed": sv["completed"]}
    return h


def percentile(xs, q):
    s = sorted(xs)
    if not s:
        return None
    k = (len(s) - 1) * q / 100.0
    lo = int(k)
    hi = min(lo + 1, len(s) - 1)
    return s[lo] + (s[hi] - s[lo]) * (k - lo)


def run_batched(args, local, precision_mode=0, steps=None):
    """Batched worlds vs the plain per-world loop on the same GPU.

    64 worlds of uneven sizes (synth.batch_specs: squares 128..1024 and the
    rectangles 512x2048, 2048x256, fluid grid = env grid), the solver of the
    full-size workload (4 V-cycles of 3+3 sweeps to 16x16, transport every
    step).  Plain: one world after another through its own World API, each
    stepped `steps` times.  Batched: all worlds as one ribo_batch, every pass
    one launch over all of them, steps replayed from CUDA graphs.
    Throughput = world-steps / device time; latency = device time of one
    step as its caller sees it (one world's step alone, or one batched step
    that advances every world).  precision_mode 1: every world solves every
    step's pressure to a relative residual of 1e-5 (mixed precision); the
    batch runs those solves one world at a time inside its step, and every
    world's last residual is checked against the tolerance.
    """
    import ribo_world as rw
    import synth

    specs = synth.batch_specs(args.batched_worlds)
    worlds = []
    total_cells = 0
    for (gw, gh), seed, rock, mean in specs:
        # the FP64 dense coarsest solve takes at most 1024 cells: the mixed
        # hierarchy goes down to 8 (2048x256 would stop at 128x16 with 16)
        w = rw.World((gw, gh), seed=seed, mg_min_size=8 if precision_mode else 16, mg_pre=3, mg_post=3,
                     device=local, precision_mode=precision_mode)
        w.settings.fluid_substep = 1
        w.settings.mg_cycles = 4
        w.seed_inputs(synth.make_world_inputs((gw, gh), seed=seed, rock_frac=rock, monomer_mean=mean))
        w.params = synth.bench_params(seed)
        worlds.append(w)
        total_cells += gw * gh
    seeded = [w.ledger_blocking().total() for w in worlds]
    steps = steps or args.batched_steps
    warm = max(args.warmup, 3)

    # ---- plain per-world loop ----
    for w in worlds:
        w.run(warm)
    for w in worlds:
        w.sync()
    plain_ms = 0.0
    t = time.perf_counter()
    for w in worlds:
        w.mark(0)
        w.run(steps)
        w.mark(1)
        plain_ms += w.elapsed_ms(0, 1)
    plain_wall = time.perf_counter() - t
    plain_lat = []
    for w in worlds:
        for _ in range(args.latency_samples):
            w.mark(2)
            w.encode_steps(1)
            w.mark(3)
            plain_lat.append(w.elapsed_ms(2, 3))

    # ---- the same worlds as one batch ----
    b = rw.Batch(worlds, device=local)
    modes = b.autotune()
    b.run(warm)
    b.sync()
    launches0 = rw.kernel_launch_count()
    t = time.perf_counter()
    b.mark(0)
    b.run(steps)
    b.mark(1)
    batch_ms = b.elapsed_ms(0, 1)
    batch_wall = time.perf_counter() - t
    launches = rw.kernel_launch_count() - launches0
    batch_lat = []
    for _ in range(args.latency_samples * 4):
        b.mark(2)
        b.encode_steps(1)
        b.mark(3)
        batch_lat.append(b.elapsed_ms(2, 3))
    b.sync()
    b.close()
    for w, s0 in zip(worlds, seeded):
        if w.ledger_blocking().total() != s0:
            raise RuntimeError("matter not conserved (batched)")
    worst = None
    if precision_mode:
        worst = max(w.solve_info()[2] for w in worlds)
        if not worst <= 1e-5:
            raise RuntimeError(f"batched mixed-precision solve above tolerance: {worst}")
    n = len(worlds)
    plain = {"world_steps_per_s": n * steps / (plain_ms / 1000.0), "wall_world_steps_per_s": n * steps / plain_wall,
             "step_latency_ms_p50": percentile(plain_lat, 50), "step_latency_ms_p99": percentile(plain_lat, 99)}
    batched = {"world_steps_per_s": n * steps / (batch_ms / 1000.0), "wall_world_steps_per_s": n * steps / batch_wall,
               "step_latency_ms_p50": percentile(batch_lat, 50), "step_latency_ms_p99": percentile(batch_lat, 99),
               "gpu_launches": launches, "tile_modes": modes}
    for w in worlds:
        w.close()
    solver = ("every pressure solved to relative residual 1e-5 (mixed precision, 3+3 V-cycles to 8x8 as "
              "the preconditioner)" if precision_mode else "4 V-cycles 3+3 to 16x16")
    out = {
        "workload": f"{n} worlds of uneven sizes (seeded draw from squares 128..1024 and 512x2048, 2048x256; "
                    f"{total_cells / 1e6:.1f} M cells), {solver}, transport every step, "
                    f"{steps} steps each",
        "worlds": n, "steps": steps, "cells": total_cells, "plain": plain, "batched": batched,
        "speedup": batched["world_steps_per_s"] / plain["world_steps_per_s"],
        "latency_note": "plain: one world's step alone; batched: one batched step (advances every world)",
    }
    if precision_mode:
        out["worst_rel_residual_device"] = worst
    return out


def run_extras(args, w):
    """The widened rows on the benchmark world (2048^2): the light block
    (light_mode 1: one propagation round, and a full sweep, device time per
    call), scene files (save and load of the whole world, wall time, through
    the public API) and the asynchronous ledger (wall time from request to
    availability, polling)."""
    import ribo_world as rw

    out = {}
    saved_bytes = bytes(w.settings)
    # light block: propagation rounds, then sweeps (a gamma upload marks the light dirty)
    w.settings.light_mode = 1
    w.settings.light_rows_per_step = 1
    w.run(2)
    w.sync()
    k = 20
    w.enable_kernel_timing(True)
    kern = {}
    for _ in range(k):
        w.encode_steps(1)
        for name, launches, kms, b in w.read_kernel_timing():
            e = kern.setdefault(name, [0, 0.0, 0.0])
            e[0] += launches
            e[1] += kms
            e[2] += b
    w.enable_kernel_timing(False)
    prop = kern.get("light_propagate", [1, 0.0, 0.0])
    comm = kern.get("light_commit", [1, 0.0, 0.0])
    w.settings.light_rows_per_step = 0
    w.settings.light_interval = 1
    w.enable_kernel_timing(True)
    sweep = [0, 0.0, 0.0]
    for _ in range(3):
        w.encode_steps(1)
        for name, launches, kms, b in w.read_kernel_timing():
            if name in ("light_transmit", "uv_light"):
                sweep[0] += 1 if name == "uv_light" else 0
                sweep[1] += kms
                sweep[2] += b
    w.enable_kernel_timing(False)
    out["light_block"] = {
        "workload": "2048^2 world, light grid 1024^2 x 2 bands",
        "propagate_round_ms": (prop[1] + comm[1]) / max(prop[0], 1),
        "propagate_round_gbs": (prop[2] + comm[2]) / max(prop[1] + comm[1], 1e-9) / 1e6,
        "full_sweep_ms": sweep[1] / max(sweep[0], 1),
    }
    import ctypes as _ct
    _ct.memmove(_ct.byref(w.settings), saved_bytes, len(saved_bytes))
    # scene files
    import tempfile

    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "bench.ribo")
        w.sync()
        t = time.perf_counter()
        w.save_scene(path)
        t_save = time.perf_counter() - t
        size = os.path.getsize(path)
        raw = sum(w.read(f).nbytes for f in (rw.CHEM, rw.GAMMA, rw.VELOCITY, rw.PRESSURE, rw.TEMP, rw.REDOX,
                                              rw.HEAT, rw.LIGHT, rw.SHADE))
        t = time.perf_counter()
        w.load_scene(path)
        t_load = time.perf_counter() - t
    _ct.memmove(_ct.byref(w.settings), saved_bytes, len(saved_bytes))
    out["scene_io"] = {"raw_mb": raw / 1e6, "file_mb": size / 1e6, "save_s": t_save, "load_s": t_load,
                       "save_mb_per_s": raw / 1e6 / t_save, "load_mb_per_s": raw / 1e6 / t_load,
                       "note": "host LZ4 block coding, single thread; includes the device copies"}
    # asynchronous ledger
    lat = []
    for _ in range(20):
        w.encode_steps(1)
        t = time.perf_counter()
        w.request_ledger()
        got = None
        while got is None:
            got = w.poll_ledger()
        lat.append((time.perf_counter() - t) * 1e3)
    w.sync()
    out["async_ledger"] = {"request_to_ready_ms_p50": percentile(lat, 50), "request_to_ready_ms_p99": percentile(lat, 99),
                           "note": "requested right after one step was recorded: includes that step's device time"}
    out["terrain_block"] = run_terrain(args)
    return out


def run_terrain(args):
    """The terrain grains (terrain_mode 1) on a world of the benchmark's size
    with 10 % rubble next to the 10 % rock, reference defaults and grains
    settling (sediment_settle 0.5: grain_fall on one step in four): the step
    rate with the terrain block against the same world with the terrain
    frozen, and the device time per step of each terrain kernel."""
    import numpy as np
    import ribo_world as rw
    import synth

    n = args.size
    inputs = synth.make_world_inputs(n, seed=1001, rubble_frac=0.1)
    w = rw.World(n, seed=1001, mg_min_size=16, mg_pre=3, mg_post=3)
    w.seed_inputs(inputs)
    w.params = synth.bench_params(1001)
    w.params.sediment_settle = 0.5
    w.settings.fluid_substep = 1
    w.settings.mg_cycles = 4
    rate = {}
    k = 64
    for mode in (1, 0, 1):
        w.settings.terrain_mode = mode
        w.run(8)
        w.sync()
        w.mark(0)
        w.run(k)
        w.mark(1)
        rate[mode] = k / (w.elapsed_ms(0, 1) / 1000.0)
    w.settings.terrain_mode = 1
    w.enable_kernel_timing(True)
    kern = {}
    steps = 8
    for _ in range(steps):
        w.encode_steps(1)
        for name, launches, kms, b in w.read_kernel_timing():
            if name in ("relax_a", "relax_b", "relax_apply", "terrain_evict", "grain_fall", "compute_gamma_slope",
                        "build_solid_mask", "wall_normals"):
                e = kern.setdefault(name, [0, 0.0, 0.0])
                e[0] += launches
                e[1] += kms
                e[2] += b
    w.enable_kernel_timing(False)
    gam = w.read(rw.GAMMA)
    moved = int((gam != inputs[rw.GAMMA]).sum())
    grains_ok = int(gam.sum(dtype=np.uint64)) == int(inputs[rw.GAMMA].sum(dtype=np.uint64))
    seeded = rw.Ledger.from_cells(inputs[rw.CHEM])
    led = w.ledger_blocking()
    terrain_ms = sum(e[1] for e in kern.values()) / steps
    out = {
        "workload": f"{n}^2 world, 10% rock + 10% rubble (1-2 grains), reference defaults, sediment_settle 0.5",
        "world_steps_per_s_terrain": rate[1],
        "world_steps_per_s_frozen": rate[0],
        "terrain_ms_per_step": terrain_ms,
        "per_kernel_ms_per_step": {name: e[1] / steps for name, e in sorted(kern.items())},
        "cells_changed": moved,
        "grains_conserved": grains_ok,
        "matter_conserved": [led.channel(c) for c in range(4)] == [seeded.channel(c) for c in range(4)],
    }
    del w
    if not args.no_cpu_baseline:
        out["cpu_baseline"] = terrain_cpu_sample(n)
    return out


def terrain_cpu_sample(n, m=512, passes=8):
    """The oracle's terrain passes (relax a, relax b, grain_fall) on the host
    cores: a bounded sample on an m x m world of the same inputs, scaled to
    the n x n world by cells."""
    import ribo_oracle
    import ribo_world as rw
    import synth

    ribo_oracle.set_threads(os.cpu_count() or 1)
    o = ribo_oracle.OracleWorld(m, seed=1001)
    o.seed_inputs(synth.make_world_inputs(m, seed=1001, rubble_frac=0.1))
    bp = synth.bench_params(1001)
    for k, _ in rw.SimParams._fields_:
        setattr(o.params, k, getattr(bp, k))
    o.params.sediment_settle = 0.5
    o.settings.terrain_mode = 1
    t = time.perf_counter()
    for e in range(passes):
        o.params.epoch = e
        for which in (16, 17, 18):
            o.run_pass(o.params, which)
    el = time.perf_counter() - t
    return {"terrain_ms_per_step": el / passes * 1e3 * (n * n) / (m * m), "cores": ribo_oracle.get_threads(),
            "kind": "port", "sample": f"{passes} terrain blocks of a {m}x{m} world ({el:.2f} s), scaled by cells"}


def host_rel_residual(p, rhs, water, eps0=float(1e-4)):
    """||rhs - L p|| / ||rhs|| over the water cells in FP64, L the level-0
    pressure operator of the reference's multigrid (sum over water neighbours
    of p_j - p_i, minus eps0 p_i; shaders/world/multigrid.wgsl:29-77)."""
    import numpy as np

    eps0 = float(np.float32(eps0))
    p = np.where(water, np.asarray(p, np.float64), 0.0)
    s = np.zeros_like(p)
    both_x, both_y = water[:, :-1] & water[:, 1:], water[:-1, :] & water[1:, :]
    s[:, 1:] += np.where(both_x, p[:, :-1] - p[:, 1:], 0.0)
    s[:, :-1] += np.where(both_x, p[:, 1:] - p[:, :-1], 0.0)
    s[1:, :] += np.where(both_y, p[:-1, :] - p[1:, :], 0.0)
    s[:-1, :] += np.where(both_y, p[1:, :] - p[:-1, :], 0.0)
    lp = np.where(water, s - eps0 * p, 0.0)
    b = np.where(water, np.asarray(rhs, np.float64), 0.0)
    bn = np.linalg.norm(b)
    return float(np.linalg.norm(b - lp) / bn) if bn > 0 else 0.0


def run_mixed(args, local):
    """The full-size step with the mixed-precision pressure solve: every solve
    iterated to a relative residual of 1e-5 (FP32-pair defect correction,
    FP32 flexible CG, FP16-storage V-cycle levels 0-3, FP64 coarsest solve and
    per-region mean removal).  The last solve's residual is re-evaluated on the
    host in FP64 (host_rel_residual)."""
    import numpy as np
    import ribo_world as rw
    import synth

    n = args.size
    w = rw.World(n, seed=1000, mg_min_size=16, mg_pre=3, mg_post=3, precision_mode=1, device=local)
    w.seed_inputs(synth.make_world_inputs(n, seed=1000))
    w.params = synth.bench_params(1000)
    w.settings.fluid_substep = 1
    warm = max(args.warmup, 3)
    w.run(warm)
    w.sync()
    steps = args.mixed_steps
    iters = []
    w.mark(0)
    done = 0
    while done < steps:
        k = min(rw.MAX_STEPS_PER_FRAME, steps - done)
        w.encode_steps(k)
        done += k
    w.mark(1)
    ms = w.elapsed_ms(0, 1)
    for _ in range(4):  # per-solve iteration counts of a few more steps
        w.encode_steps(1)
        iters.append(w.solve_info())
    # per-kernel device time of two steps (the solve then runs its loops from
    # the host, one launch per kernel)
    w.enable_kernel_timing(True)
    kern = {}
    for _ in range(2):
        w.encode_steps(1)
        for name, launches, kms, b in w.read_kernel_timing():
            e = kern.setdefault(name, [0, 0.0])
            e[0] += launches
            e[1] += kms
    w.enable_kernel_timing(False)
    top = sorted(kern.items(), key=lambda kv: -kv[1][1])[:16]
    water = w.read(rw.SOLID_MASK) == 0
    p = w.read(rw.PRESSURE).astype(np.float64) + w.read(rw.PRESSURE_LO).astype(np.float64)
    rho = host_rel_residual(p, w.read(rw.DIVERGENCE), water)
    w.close()
    return {
        "workload": f"{n}x{n} full world step, pressure solved to relative residual 1e-5 every step (mixed precision)",
        "world_steps_per_s": steps / (ms / 1000.0), "ms_per_step": ms / steps, "steps": steps,
        "solves": [{"outer": o, "cg_iterations": i, "rel_residual_device": r} for o, i, r in iters],
        "rel_residual_fp64_host": rho, "tolerance": 1e-5,
        "kernels_ms_per_step": [[k, round(v[1] / 2, 4), v[0] // 2] for k, v in top],
    }


def serving_trace(rate, seconds, seed=11):
    """Poisson arrivals; each request: a world of log-uniform side 128..2048
    with aspect ratio up to 4:1 (sides rounded to multiples of 32) and a
    log-uniform step count in 10..1000."""
    import numpy as np

    rng = np.random.default_rng(seed)
    t, out = 0.0, []
    while True:
        t += float(rng.exponential(1.0 / rate))
        if t >= seconds:
            return out
        side = float(np.exp(rng.uniform(np.log(128), np.log(2048))))
        aspect = float(np.exp(rng.uniform(-np.log(4), np.log(4))))
        w = int(min(2048, max(128, round(side * np.sqrt(aspect) / 32) * 32)))
        h = int(min(2048, max(128, round(side / np.sqrt(aspect) / 32) * 32)))
        steps = int(round(float(np.exp(rng.uniform(np.log(10), np.log(1000))))))
        out.append((t, (w, h), steps, len(out)))


def run_serving(args, local, rate, seconds, drain_seconds):
    """Continuous-batching server fed by a Poisson request stream in real time.

    Each request's fields are a seeded crop of one of two pre-generated
    2048x2048 input sets (same generators and distributions as the plain
    workload: value-noise velocity, 10% rock, Poisson(4) monomers); the
    request becomes a job (materialised, copied, queued on the server) when
    the server's own queue is short, and its latency counts from its arrival.
    The server admits jobs in arrival order against the HBM budget, keeps
    their state resident and advances all resident jobs together each
    iteration.  The run stops taking arrivals after `serve_seconds`, then
    runs the iterations it has time for within `drain_seconds`.
    """
    import numpy as np
    import ribo_world as rw
    import synth

    trace = serving_trace(rate, seconds)
    templates = [synth.make_world_inputs(2048, seed=5000 + k) for k in range(2)]
    fields = (rw.GAMMA, rw.CHEM, rw.VELOCITY, rw.LIGHT)

    def job_inputs(i, w, h):
        rng = np.random.default_rng(90000 + i)
        tp = templates[i % len(templates)]
        x0 = int(rng.integers(0, 2048 - w + 1)) // 2 * 2
        y0 = int(rng.integers(0, 2048 - h + 1)) // 2 * 2
        return {
            rw.GAMMA: tp[rw.GAMMA][y0:y0 + h, x0:x0 + w],
            rw.CHEM: tp[rw.CHEM][y0:y0 + h, x0:x0 + w],
            rw.VELOCITY: tp[rw.VELOCITY][y0:y0 + h, x0:x0 + w],
            rw.LIGHT: tp[rw.LIGHT][:, y0 // 2:(y0 + h) // 2, x0 // 2:(x0 + w) // 2],
        }

    settings = rw.default_settings()
    settings.fluid_substep = 1
    settings.mg_cycles = 4
    budget = int(args.serve_budget_gb * 1e9)
    srv = rw.Server(budget, max_chunk_steps=args.serve_chunk, device=local)
    t0 = time.perf_counter()
    arrival = {}
    nxt = 0
    it_records = []
    while True:
        now = time.perf_counter() - t0
        if now > seconds + drain_seconds:
            break
        st = srv.stats()
        while nxt < len(trace) and trace[nxt][0] <= min(now, seconds) and st.pending < args.serve_queue:
            ta, (w, h), steps, i = trace[nxt]
            jid = srv.submit((w, h), steps=steps, params=synth.bench_params(7000 + i), settings=settings,
                             inputs=job_inputs(i, w, h), mg_min_size=16, mg_pre=3, mg_post=3, user_tag=i)
            arrival[jid] = ta
            nxt += 1
            st = srv.stats()
        if st.active == 0 and st.pending == 0:
            if nxt >= len(trace):
                break
            time.sleep(min(0.01, max(0.0, trace[nxt][0] - now)))
            continue
        srv.iterate()
        it_records += srv.iterations()
    wall = time.perf_counter() - t0
    results = srv.results()
    it_records += srv.iterations()
    st = srv.stats()
    done = [r for r, _ in results if r.status == 0]
    job_lat = [(r.t_done_ms / 1000.0 - arrival[r.id]) * 1000.0 for r in done]
    job_step_lat = [l / r.steps for l, r in zip(job_lat, done)]
    per_step = []
    for ms, steps, active in it_records:
        per_step += [ms / max(steps, 1)] * max(active, 1)  # one sample per resident job-step
    srv.close()
    return {
        "workload": f"Poisson arrivals at {rate:g} req/s for {seconds:g} s; world side "
                    f"log-uniform 128..2048, aspect up to 4:1, steps log-uniform 10..1000; "
                    f"{args.serve_budget_gb:g} GB HBM budget; chunks of {args.serve_chunk} steps",
        "requests_arrived": len(trace), "submitted": st.submitted, "admitted": st.admitted,
        "completed": st.completed, "resident_at_end": st.active, "queued_at_end": st.pending,
        "not_yet_submitted": len(trace) - nxt,
        "world_steps": st.world_steps, "gpu_ms": st.gpu_ms, "wall_s": wall,
        "world_steps_per_s": st.world_steps / wall, "world_steps_per_gpu_s": st.world_steps / max(st.gpu_ms / 1000.0, 1e-9),
        "step_latency_ms_p50": percentile(per_step, 50), "step_latency_ms_p99": percentile(per_step, 99),
        "job_latency_ms_p50": percentile(job_lat, 50), "job_latency_ms_p99": percentile(job_lat, 99),
        "job_ms_per_step_p50": percentile(job_step_lat, 50), "job_ms_per_step_p99": percentile(job_step_lat, 99),
        "iterations": st.iterations,
        "note": "offered load ~= rate x E[cells x steps]; latencies of completed jobs count from arrival",
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--size", type=int, default=2048)
    ap.add_argument("--e2e-steps", type=int, default=256)
    ap.add_argument("--profile-steps", type=int, default=16)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--reference-seconds", type=float, default=60.0)
    ap.add_argument("--batched-worlds", type=int, default=64)
    ap.add_argument("--batched-steps", type=int, default=200)
    ap.add_argument("--batched-mixed-steps", type=int, default=24)
    ap.add_argument("--latency-samples", type=int, default=5)
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--no-serving", action="store_true")
    ap.add_argument("--no-mixed", action="store_true")
    ap.add_argument("--no-extras", action="store_true")
    ap.add_argument("--mixed-steps", type=int, default=32)
    ap.add_argument("--serve-rate", type=float, default=200.0)
    ap.add_argument("--serve-seconds", type=float, default=60.0)
    ap.add_argument("--serve-drain-seconds", type=float, default=0.0)
    ap.add_argument("--serve-budget-gb", type=float, default=150.0)
    ap.add_argument("--serve-chunk", type=int, default=16)
    ap.add_argument("--serve-queue", type=int, default=4)
    ap.add_argument("--serve-sustainable-rate", type=float, default=6.0)
    ap.add_argument("--serve-sustainable-seconds", type=float, default=40.0)
    ap.add_argument("--ncu-case", action="store_true")
    ap.add_argument("--ncu-terrain", action="store_true")
    ap.add_argument("--ncu-mixed", action="store_true")
    args = ap.parse_args()
    if args.ncu_case or args.ncu_terrain:
        import ribo_world as rw
        import synth

        w = rw.World(args.size, seed=1000, mg_min_size=16, mg_pre=3, mg_post=3, no_graphs=1,
                     precision_mode=1 if args.ncu_mixed else 0)
        w.settings.fluid_substep = 1
        w.settings.mg_cycles = 4
        w.seed_inputs(synth.make_world_inputs(args.size, seed=1000 if not args.ncu_terrain else 1001,
                                              rubble_frac=0.1 if args.ncu_terrain else 0.0))
        w.params = synth.bench_params(1000)
        if args.ncu_terrain:
            w.settings.terrain_mode = 1
            w.params.sediment_settle = 0.5
        w.run(args.steps)
        w.sync()
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
