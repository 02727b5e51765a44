"""Benchmark of the 3D dexel dilation path on GB300.

One step = one dilation (radius 32 dexels) of the 2048 x 2048 synthetic volume
"spheres_cyl2048" (16384 spheres, lognormal radii with median 12 clipped to
[2, 80], plus 2000 random-axis cylinders of radius 1-4; seeded), the
configuration the headline metric is quoted on. The input (~345 MB of FP64
pairs) is larger than L2 (129 MB), so no flush is needed between steps.

  value : Mcolumns/s with the input resident in HBM (device-timed, CUDA events
          on the library's stream), whole job = all ranks. The default method
          is the batch plan (vo_batch_*) with the learned sizer: one step is a
          replay of the captured graph plus the conversion of the output slots
          to CSR. The plan is built once before the warm-up.
  arms  : the plain GPU method (the separable scheme's envelope sweeps in
          FP64), its painter form (FP64, count then fill) and the
          single-volume FP32-guarded method on the same volume, for the
          "plain vs batched+learned" comparison.
  e2e   : the same metric through the C ABI from pinned host buffers: upload,
          vo_morph_batched (plan, replay, outputs) and download of the result
          inside the timed region, the copies on the context's copy stream so
          that they overlap the neighbouring steps' dilations.
  cpu_baseline : the reference's own `ours` (oracle/_ref, multithreaded) or,
          where the reference could not be built, the oracle restatement, timed
          on a bounded slab of the same workload (rank 0, N=1).

python bench.py [--gpus N --steps K --warmup W] [--impl reference]
Under torchrun each rank dilates its own replica (seed + rank): the path has
no data exchange, so scaling is weak and replicas only.
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

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = "spheres_cyl2048"
RADIUS = 32.0
METRIC = "Mcolumns/s, 3D dilation 2048² r=32: plain vs batched+learned GPU, exact topology"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--method", default="batched", choices=["batched", "separable", "brute", "fast", "envelope"],
                    help="batched: a captured batch plan with the learned sizer (the headline)")
    ap.add_argument("--no-sizer", action="store_true", help="batched plan without the learned sizer")
    ap.add_argument("--no-arms", action="store_true", help="skip the plain / single-volume comparison arms")
    ap.add_argument("--no-learned-arm", action="store_true", help="skip the 4096^2 learned-sizing arm")
    ap.add_argument("--workload", default=WORKLOAD)
    ap.add_argument("--radius", type=float, default=RADIUS)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=15.0, help="target CPU work of the baseline sample")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        self.lines = []
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        sms, maxs, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sms.append(float(p[1]))
                maxs.append(float(p[2]))
            except ValueError:
                continue
            for n, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sms:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": float(np.median(sms)), "sm_max_mhz": float(max(maxs)), "reasons": sorted(reasons),
                "samples": len(sms)}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            p = json.load(fh)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def kernel_counters(kernel: str, workload: str, radius: float) -> dict:
    """Per-output-column ncu counters of a kernel on this workload and radius from the committed
    summary (DRAM bytes, warp and thread instructions), or {} when none was captured."""
    path = os.path.join(ROOT, "profiles", "kernel_counters.json")
    try:
        with open(path) as fh:
            e = json.load(fh).get(f"{kernel}@r{int(radius)}")
        return e if e and str(e.get("workload", "")).startswith(workload + " ") else {}
    except Exception:
        return {}


def cpu_sample(grid, offs, z, radius, target_s, step_rows=None, gpu_out=None):
    """Times the CPU reference (or its restatement) on a slab of rows. Returns a dict.

    The slab is a band of `rows` interior rows from the middle of the volume plus a halo of
    floor(radius) rows on each side; the halo is computed (the interior columns' discs need it) but
    only the interior columns are counted. With gpu_out = (offs, z) of the GPU's output for the whole
    volume, the interior columns of the CPU result are also compared with it (`precision`)."""
    from oracle import oracle as O
    kind = "reference" if O.ref_available() else "port"
    cores = os.cpu_count() or 1
    R = int(np.floor(radius))
    nx, ny = grid.nx, grid.ny

    def run(rows):
        rows = min(rows, ny)
        yi0 = max(0, ny // 2 - rows // 2)
        yi1 = min(ny, yi0 + rows)
        y0, y1 = max(0, yi0 - R), min(ny, yi1 + R)
        sub_offs = offs[y0 * nx:y1 * nx + 1] - offs[y0 * nx]
        sub_z = z[2 * offs[y0 * nx]:2 * offs[y1 * nx]]
        g = O.Grid(nx, y1 - y0, (0.0, 0.0, 0.0), (nx, y1 - y0, grid.extent[2]), 1.0, 0)
        t0 = time.perf_counter()
        if kind == "reference":
            oo, oz = O.ref_morph(g, sub_offs, sub_z, radius, "dilation", "ours", threads=cores)[:2]
        else:
            oo, oz = O.dilate_timed(g, sub_offs, sub_z, radius, threads=cores)[:2]
        dt = time.perf_counter() - t0
        return dt, nx * (yi1 - yi0), (yi0, yi1, y0, y1), (oo, oz)

    if step_rows is None:
        rows = 16
        dt, inner, span, res = run(rows)
        while dt < target_s / 4 and rows < ny:
            rows = min(ny, int(rows * max(2.0, 0.5 * target_s / max(dt, 1e-3))))
            dt, inner, span, res = run(rows)
    else:
        rows = step_rows
        dt, inner, span, res = run(rows)
    yi0, yi1, y0, y1 = span
    val = inner / dt / 1e6
    sample = (f"dilation r={radius:g} of rows {yi0}-{yi1 - 1} ({yi1 - yi0} x {nx} columns counted) from the "
              f"middle of the volume, computed with a {yi0 - y0}+{y1 - yi1}-row halo that is not counted")
    out = {"value": val, "unit": "Mcolumns/s", "cores": cores, "kind": kind, "sample": sample,
           "seconds": dt, "rows": rows}
    if gpu_out is not None:
        go, gz = gpu_out
        c0, c1 = yi0 * nx, yi1 * nx  # interior columns in the whole volume
        s0 = (yi0 - y0) * nx          # ... and in the slab
        wo, wz = res
        a_off = go[c0:c1 + 1] - go[c0]
        a_z = gz[2 * go[c0]:2 * go[c1]]
        b_off = wo[s0:s0 + (c1 - c0) + 1] - wo[s0]
        b_z = wz[2 * wo[s0]:2 * wo[s0 + (c1 - c0)]]
        cmp = O.compare((a_off, a_z), (b_off, b_z))
        out["precision"] = {"max_endpoint_error": cmp["max_err"], "topology_mismatches": cmp["count_mismatch"],
                            "columns_checked": int(c1 - c0),
                            "checked_against": "the reference build (oracle/_ref)" if kind == "reference"
                            else "the FP64 oracle restatement"}
    return out


def bench_config(args, grid, offs):
    """The workload, identical in both arms (method, launch shape and the like go to `run`)."""
    # the FP64 input (16 B per segment) and its FP32 copy exceed the 129 MB L2 at the benchmark sizes, so
    # timed steps run back to back without an L2 flush
    in_bytes = 16 * int(offs[-1]) + 4 * (grid.nx * grid.ny + 1)
    l2 = "inputs larger than L2 (no flush)" if in_bytes > 129 * 2**20 else "inputs smaller than L2 (no flush)"
    return {"workload": f"{args.workload} dilation r={args.radius:g}", "grid": [grid.nx, grid.ny],
            "in_segments": int(offs[-1]), "radius": args.radius, "l2": l2}


def reference_arm(args, rank, world):
    if rank != 0:
        return 0
    import voroffset_gb300 as V  # parameters only: no product library is loaded by this arm
    from oracle import oracle as O
    grid, offs, z = V.workload(args.workload, seed=1, synth=O.SYNTH_SO)
    # calibrate a slab that takes a few seconds per step
    cal = cpu_sample(grid, offs, z, args.radius, target_s=min(args.cpu_seconds, 8.0))
    rows = cal["rows"]
    vals = []
    for i in range(args.warmup + args.steps):
        r = cpu_sample(grid, offs, z, args.radius, 0, step_rows=rows)
        if i >= args.warmup:
            vals.append(r)
    secs = sum(r["seconds"] for r in vals)
    cols = sum(r["value"] * r["seconds"] * 1e6 for r in vals)
    value = cols / secs / 1e6
    line = {"metric": METRIC, "value": value, "unit": "Mcolumns/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * secs / len(vals), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "impl": "reference",
            "config": bench_config(args, grid, offs), "run": {"parallelism": "host threads"},
            "cpu_baseline": {"value": value, "unit": "Mcolumns/s", "cores": vals[0]["cores"],
                             "kind": vals[0]["kind"], "sample": vals[0]["sample"]},
            "e2e": {"value": value, "unit": "Mcolumns/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def batch_volumes(V, n, seed):
    """The batched workload: n seeded volumes, grid side in {64, 128, 256, 512, 1024}, each a union of
    64-2048 spheres with radii 2-30, radius r uniform in [2, 64] (multiples of 0.25), mixed operations."""
    rng = np.random.default_rng(seed)
    items = []
    for _ in range(n):
        side = int(rng.choice([64, 128, 256, 512, 1024]))
        spec = V.SynthSpec(side, n_spheres=int(rng.integers(64, 2049)), s_rmin=2, s_rmax=30,
                           seed=int(rng.integers(1, 1 << 40)))
        g, o, z = V.synth_volume(spec)
        items.append((g, o, z, float(np.round(rng.uniform(2, 64) * 4) / 4),
                      ["dilation", "erosion", "opening", "closing"][int(rng.integers(0, 4))]))
    return items


def batch_main(args, rank, world, local):
    """`--workload batch256`: one step = every volume of the batch through one replay of its plan plus
    the conversion of all outputs to CSR; value = output columns per second. Arms: the same volumes one
    by one through vo_morph (FP32 method, and the plain FP64 method on a subset)."""
    import torch
    import voroffset_gb300 as V

    torch.cuda.set_device(local)
    n = int(args.workload[len("batch"):] or 256)
    items = batch_volumes(V, n, seed=7 + rank)
    ctx = V.Context(local)
    stream = torch.cuda.ExternalStream(ctx.stream, device=torch.device("cuda", local))
    sizer = None
    if not args.no_sizer:
        from voroffset_gb300.train_sizer import WEIGHTS, load
        if os.path.exists(WEIGHTS):
            sizer = load(ctx)
            ctx.set_sizer(sizer)
    vols = [ctx.upload(g, o, z) for g, o, z, _, _ in items]
    ops = [it[4] for it in items]
    radii = [it[3] for it in items]
    cols = sum(g.ncols for g, _, _, _, _ in items)
    meta = [(g.nx, op, r) for g, _, _, r, op in items]
    items = None  # host copies are no longer needed

    def progress(what):
        import resource
        free, total = torch.cuda.mem_get_info(local)
        print(f"[batch] {what}: device {(total - free) / 2**30:.1f} GiB used, host rss "
              f"{resource.getrusage(resource.RUSAGE_SELF).ru_maxrss / 2**20:.1f} GiB", file=sys.stderr, flush=True)

    progress("volumes uploaded")
    plan = ctx.batch(vols, ops, radii, "fast")
    st = plan.stats()
    progress("plan built")
    acc = {"launches": 0, "reruns": 0}

    def step():
        t = plan.run()
        acc["launches"] += t["kernel_launches"]
        acc["reruns"] += t["overflow_columns"]
        for o in plan.outputs():
            o.free()

    barrier, maxreduce = sync_helpers(world)

    def timed(f, steps, warmup):
        for _ in range(warmup):
            f()
        barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            f()
        e1.record(stream)
        barrier()
        return maxreduce(e0.elapsed_time(e1))

    clocks = ClockSampler(local)
    clocks.start()
    ms = timed(step, args.steps, args.warmup)
    clk = clocks.stop()
    value = job_rate(world, cols * args.steps, ms / 1e3)
    progress("batched steps timed")

    def loop_step():
        for v, op, r in zip(vols, ops, radii):
            o, _ = ctx.morph(v, op, r, "fast")
            o.free()

    loop_ms = timed(loop_step, 1, 1)
    arms = {"one_by_one_fast": {"value": job_rate(world, cols, loop_ms / 1e3), "unit": "Mcolumns/s",
                                "ms_per_step": loop_ms}}
    arms["batched_vs_one_by_one"] = value / arms["one_by_one_fast"]["value"]
    st_run = plan.stats()
    rerun = None
    if st_run["rerun_first"] >= 0:
        side, op, r = meta[st_run["rerun_first"]]
        rerun = {"volumes": st_run["reruns"], "first": {"side": side, "op": op, "radius": r},
                 "cause": st_run["rerun_cause"]}
    line = {"metric": METRIC, "value": value, "unit": "Mcolumns/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
            "config": {"workload": f"{n} volumes, sides 64-1024, 64-2048 spheres, r in [2, 64], mixed ops",
                       "rerun": rerun,
                       "columns": cols, "method": "batched+learned" if sizer else "batched",
                       "ops": {o: ops.count(o) for o in set(ops)},
                       "plan": {k: st[k] for k in ("slot_bytes", "tiles", "tile_rows", "union_cap", "persistent", "regs", "graph_nodes",
                                                   "graph_kernels", "learned", "plan_ms", "tune_ms")},
                       "reruns_per_step": acc["reruns"] / (args.steps + args.warmup)},
            "gpu_launches": int(acc["launches"] * args.steps / (args.steps + args.warmup)),
            "clocks": clk, "arms": arms}
    plan.free()
    for v in vols:
        v.free()
    if sizer is not None:
        ctx.set_sizer(None)
        sizer.free()
    ctx.close()
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


def learned_sizing_arm(ctx, sizer, rank, world, timed):
    """The learned-sizing configuration: dilation r=16 of the 4096^2 volume of 20000 cylinders (radius
    1.5-3, ~20 segments per column). One step each through a batch plan sized by the learned sizer, a
    batch plan with fixed-capacity slots, and the single-volume FP32 method; a plan's step is a graph
    replay (plus the re-run of a volume whose slots overflowed) and the conversion to CSR."""
    import voroffset_gb300 as V
    grid, offs, z = V.workload("cyl4096", seed=1 + rank)
    v = ctx.upload(grid, offs, z)
    ncols = grid.ncols
    del offs, z
    out = {"workload": "cyl4096 dilation r=16", "grid": [grid.nx, grid.ny]}
    for name, sz in (("learned", sizer), ("fixed_capacity", None)):
        if name == "learned" and sz is None:
            continue
        ctx.set_sizer(sz)
        plan = ctx.batch([v], ["dilation"], [16.0], "fast")
        st0 = plan.stats()

        def step():
            plan.run()
            for o in plan.outputs():
                o.free()

        ms = timed(step, 1, 1)
        st = plan.stats()
        out[name] = {"value": job_rate(world, ncols, ms / 1e3), "unit": "Mcolumns/s", "ms_per_step": ms,
                     "slot_bytes": st0["slot_bytes"], "volumes_rerun": st["reruns"], "plan_ms": st0["plan_ms"]}
        plan.free()
    ctx.set_sizer(sizer)

    def single():
        o, _ = ctx.morph(v, "dilation", 16.0, "fast")
        o.free()

    ms = timed(single, 1, 1)
    out["single_volume"] = {"value": job_rate(world, ncols, ms / 1e3), "unit": "Mcolumns/s", "ms_per_step": ms}
    if "learned" in out:
        out["learned_vs_fixed"] = out["learned"]["value"] / out["fixed_capacity"]["value"]
        out["learned_vs_single"] = out["learned"]["value"] / out["single_volume"]["value"]
    v.free()
    return out


def sync_helpers(world: int, cuda: bool = True):
    """barrier(): device sync, then a barrier over the ranks; maxreduce(x): the
    largest x over the ranks (the job's time is its slowest rank's)."""
    import torch

    def barrier():
        if cuda:
            torch.cuda.synchronize()
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    def maxreduce(x):
        if world == 1:
            return x
        import torch.distributed as dist
        t = torch.tensor([x], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    return barrier, maxreduce


def job_rate(world: int, units_per_rank: float, seconds: float) -> float:
    """Whole-job throughput in millions of units per second: every rank
    processes units_per_rank in the (slowest rank's) time `seconds`."""
    return world * units_per_rank / seconds / 1e6


def main():
    args = parse()
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    if args.workload.startswith("batch") and args.impl != "reference":
        rc = batch_main(args, rank, world, local)
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()
        return rc
    if args.impl == "reference":
        rc = reference_arm(args, rank, world)
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()
        return rc

    import torch
    import voroffset_gb300 as V

    torch.cuda.set_device(local)
    grid, offs, z = V.workload(args.workload, seed=1 + rank)
    ncols = grid.ncols
    in_bytes = offs.nbytes + z.nbytes
    ctx = V.Context(local)
    stream = torch.cuda.ExternalStream(ctx.stream, device=torch.device("cuda", local))

    barrier, maxreduce = sync_helpers(world)

    # ---------------- learned sizer (batched arms)
    sizer = None
    if args.method == "batched" and not args.no_sizer:
        from voroffset_gb300.train_sizer import WEIGHTS, load
        if os.path.exists(WEIGHTS):
            sizer = load(ctx)
            ctx.set_sizer(sizer)

    vin = ctx.upload(grid, offs, z)
    ctx.sync()

    def timed(step, steps, warmup, after_warmup=None):
        """Device time (CUDA events on the library stream) of `steps` calls of step()."""
        for _ in range(warmup):
            step()
        if after_warmup is not None:
            after_warmup()
        barrier()
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        for _ in range(steps):
            step()
        ev1.record(stream)
        barrier()
        return maxreduce(ev0.elapsed_time(ev1))

    acc = {"launches": 0, "kernel_ms": 0.0, "out_segs": 0, "mid": 0}

    def single_step(method):
        def f():
            out, t = ctx.morph(vin, "dilation", args.radius, method)
            acc["launches"] += t["kernel_launches"]
            acc["kernel_ms"] += max(t["kernel_ms"])
            acc["pass1_ms"] = acc.get("pass1_ms", 0.0) + t["pass1_ms"]
            acc["pass2_ms"] = acc.get("pass2_ms", 0.0) + t["pass2_ms"]
            acc["out_segs"] = out.nseg
            acc["mid"] = t["mid_pieces"]
            out.free()
        return f

    plan = None
    plan_stats = None
    if args.method == "batched":
        plan = ctx.batch([vin], ["dilation"], [args.radius], "fast")
        plan_stats = plan.stats()

        def step():
            t = plan.run()
            outs = plan.outputs()
            acc["launches"] += t["kernel_launches"] + 5  # graph kernels + slot -> CSR (counts, 3 scan, compact)
            acc["kernel_ms"] += t["pass2_ms"]
            acc["out_segs"] = outs[0].nseg
            outs[0].free()
    else:
        step = single_step(args.method)

    # ---------------- device-resident arm (value)
    clocks = ClockSampler(local)
    clocks.start()
    # launches and kernel time are counted over the timed steps only
    dev_ms = timed(step, args.steps, args.warmup, after_warmup=lambda: acc.update(launches=0, kernel_ms=0.0))
    clk = clocks.stop()
    launches, kernel_ms, out_segs, mid = acc["launches"], acc["kernel_ms"], acc["out_segs"], acc["mid"]
    value = job_rate(world, ncols * args.steps, dev_ms / 1e3)

    # ---------------- end-to-end arm (pinned host buffers through the C ABI), right after the
    # device-resident arm and before the FP64 comparison arms, which hold the GPU busy for tens of seconds
    pin_offs = torch.empty(offs.size, dtype=torch.int32, pin_memory=True).numpy()
    pin_z = torch.empty(max(z.size, 2), dtype=torch.float64, pin_memory=True).numpy()
    pin_offs[:] = offs
    pin_z[:z.size] = z
    out_offs = torch.empty(ncols + 1, dtype=torch.int32, pin_memory=True).numpy()
    out_z = torch.empty(max(2 * out_segs, 2), dtype=torch.float64, pin_memory=True).numpy()

    # Steps are pipelined through the copy stream of the context: the upload of step i + 1 is queued
    # (vo_volume_upload_async) before the dilation of step i and the download of step i
    # (vo_volume_download_async) after it, so both copies overlap a dilation; every step still moves
    # its input in and its result out inside the timed region, which ends when the last download has
    # landed (vo_sync). Host-clock split per step: the upload call (offsets checked while the copy
    # runs), the morphology call and its own total_ms (plan, replay, outputs), the download call and
    # the frees; `drain_ms` is the final wait for the last download.
    parts = {"upload_ms": 0.0, "morph_ms": 0.0, "morph_call_ms": 0.0, "download_ms": 0.0, "free_ms": 0.0,
             "drain_ms": 0.0}
    pin_zv = pin_z[:z.size]

    def e2e_run(steps):
        d2h = 0
        nxt = ctx.upload_async(grid, pin_offs, pin_zv)
        for i in range(steps):
            t0 = time.perf_counter()
            cur = nxt
            if i + 1 < steps:
                nxt = ctx.upload_async(grid, pin_offs, pin_zv)
            t1 = time.perf_counter()
            if args.method == "batched":
                outs, tm = ctx.morph_batched([cur], ["dilation"], [args.radius], "fast")
                o = outs[0]
            else:
                o, tm = ctx.morph(cur, "dilation", args.radius, args.method)
            t2 = time.perf_counter()
            n_o, n_z = ctx.download_async(o, out_offs, out_z)
            t3 = time.perf_counter()
            o.free()
            cur.free()
            t4 = time.perf_counter()
            for k, dt in (("upload_ms", t1 - t0), ("morph_call_ms", t2 - t1), ("download_ms", t3 - t2),
                          ("free_ms", t4 - t3)):
                parts[k] += dt * 1e3
            parts["morph_ms"] += tm["total_ms"]
            d2h = 4 * n_o + 8 * n_z
        t5 = time.perf_counter()
        ctx.sync()
        parts["drain_ms"] += (time.perf_counter() - t5) * 1e3
        return d2h

    e2e_run(max(1, args.warmup))
    barrier()
    parts.update({k: 0.0 for k in parts})
    clocks.start()
    t0 = time.perf_counter()
    d2h = e2e_run(args.steps)
    barrier()
    e2e_s = maxreduce(time.perf_counter() - t0)
    e2e_clk = clocks.stop()
    e2e = job_rate(world, ncols * args.steps, e2e_s)

    # ---------------- comparison arms on the same volume: the plain GPU method (FP64 envelope
    # sweeps), its painter form (FP64) and the single-volume FP32-guarded method
    arms = {}
    if args.method == "batched" and not args.no_arms:
        # the plain method is the separable scheme's sweeping envelope form in FP64; the painter form
        # (per-column pass-1 pieces, then their union) is the other FP64 arm
        # (the FP64 arms take seconds per step: two timed steps each keep the run within minutes)
        for name, method, k in (("plain_envelope_fp64", "envelope", min(2, args.steps)),
                                ("painter_separable_fp64", "separable", min(2, args.steps)),
                                ("fast_single_volume", "fast", args.steps)):
            ms = timed(single_step(method), k, 1, after_warmup=lambda: acc.update(pass1_ms=0.0, pass2_ms=0.0))
            arms[name] = {"value": world * ncols * k / (ms / 1e3) / 1e6, "unit": "Mcolumns/s",
                          "ms_per_step": ms / k, "steps": k}
            if method == "envelope":
                arms[name]["pass1_ms"] = acc.get("pass1_ms", 0.0) / k
                arms[name]["pass2_ms"] = acc.get("pass2_ms", 0.0) / k
        arms["batched_vs_plain"] = value / arms["plain_envelope_fp64"]["value"]
        arms["batched_vs_painter"] = value / arms["painter_separable_fp64"]["value"]
        if not args.no_learned_arm:
            arms["learned_sizing_cyl4096"] = learned_sizing_arm(ctx, sizer, rank, world, timed)

    # ---------------- roofline of the dominant kernel
    kname = {"batched": "k_fast_batched", "fast": "k_fast", "separable": "k_pass2", "brute": "k_brute",
             "envelope": "k_env2"}[args.method]
    per_launch = kernel_ms / args.steps
    alg_bytes = 4 * (ncols + 1) + 16 * int(offs[-1]) + 4 * (ncols + 1) + 16 * int(out_segs)
    peak, peak_kind = peaks()
    achieved = alg_bytes / (per_launch / 1e3) / 1e9 if per_launch > 0 else 0.0
    kc = kernel_counters(kname, args.workload, args.radius)
    tpc = kc.get("bytes_per_column")
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "traffic": None if tpc is None else tpc * ncols,
                "kernel": kname, "kernel_ms": per_launch, "peak_source": peak_kind,
                "algorithmic_bytes": alg_bytes,
                "op_achieved": alg_bytes / (dev_ms / args.steps / 1e3) / 1e9}
    # the compute side: the kernel's instruction issue against the SMs' issue slots (4 schedulers per
    # SM, one warp instruction per cycle each, at the median SM clock seen in the timed region), from
    # the instruction counts of the committed ncu capture of this workload and the live kernel time
    issue = None
    wpc = kc.get("warp_instructions_per_column")
    if wpc and per_launch > 0 and clk.get("sm_mhz"):
        import torch
        sms = torch.cuda.get_device_properties(local).multi_processor_count
        ach = wpc * ncols / (per_launch / 1e3) / 1e9
        pk = sms * 4 * clk["sm_mhz"] * 1e6 / 1e9
        lanes = kc["thread_instructions_per_column"] / wpc
        issue = {"bound": "issue", "achieved": ach, "peak": pk, "unit": "Gwarp-inst/s", "frac": ach / pk,
                 "lanes_per_inst": lanes, "lane_weighted_frac": ach / pk * lanes / 32,
                 "warp_inst_per_launch": wpc * ncols, "sms": sms, "source": kc.get("source")}

    dtype = "f64" if args.method in ("separable", "brute", "envelope") else "f32+f64"
    cfg = bench_config(args, grid, offs)
    run = {"method": args.method if args.method != "batched" else "batched+learned" if sizer else "batched",
           "out_segments": int(out_segs), "mid_pieces": int(mid),
           "l2": "inputs larger than L2 (no flush)", "parallelism": "replicas" if world > 1 else "single GPU"}
    if plan_stats is not None:
        run["plan"] = {k: plan_stats[k] for k in ("slot_bytes", "tiles", "tile_rows", "union_cap", "persistent", "regs", "graph_nodes",
                                                  "graph_kernels", "learned", "plan_ms", "tune_ms")}
    line = {"metric": METRIC, "value": value, "unit": "Mcolumns/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dev_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": dtype, "data": "synthetic", "config": cfg, "run": run,
            "e2e": {"value": e2e, "unit": "Mcolumns/s", "h2d_bytes_per_step": int(in_bytes),
                    "d2h_bytes_per_step": int(d2h), "ms_per_step": e2e_s * 1e3 / args.steps,
                    "sm_mhz": e2e_clk.get("sm_mhz"), "split": {k: v / args.steps for k, v in parts.items()}},
            "gpu_launches": int(launches),
            "roofline": roofline, "issue_roofline": issue, "clocks": clk, "arms": arms,
            "gsegments_per_s": world * (int(offs[-1]) + int(out_segs)) * args.steps / (dev_ms / 1e3) / 1e9}
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        try:
            cb = cpu_sample(grid, offs, z, args.radius, args.cpu_seconds, gpu_out=(out_offs, out_z[:2 * out_segs]))
            line["precision"] = cb.pop("precision")
            line["cpu_baseline"] = {k: v for k, v in cb.items() if k != "rows"}
        except Exception as exc:  # the baseline is reported, never required
            line["cpu_baseline"] = {"value": None, "error": str(exc)}
    if plan is not None:
        plan.free()
    if sizer is not None:
        ctx.set_sizer(None)
        sizer.free()
    vin.free()
    ctx.close()
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
