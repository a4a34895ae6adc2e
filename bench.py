#!/usr/bin/env python3
"""Benchmark: Gpixels/s of bit-exact reconstruction by dilation on GB300.

Workload (one "step"): the six plain 4096x4096 uint8 reconstructions of the
4096^2 configuration -- connectivity {4, 8} x h-dome h {10, 40, 100} on one
seeded smoothed-noise-plus-discs mask -- each through the C ABI with the
unique queue.  Every reconstruction restores its marker from a pristine
device copy first (in place).

  value : device-resident throughput (inputs already in HBM), CUDA events
          around K steps on the launching stream, max over ranks.
  e2e   : the same six reconstructions through the reference-facing
          synchronous call with pinned HOST buffers, H2D of marker + mask and
          D2H of the result inside the timed region.
  roofline : the persistent engine kernel; algorithmic bytes = 3 * W * H *
          bytes/pixel per reconstruction (read mask, read marker, write
          result) over the kernel's event-timed duration, against the
          measured HBM copy bandwidth.
  cpu_baseline : the CPU oracle (Vincent 1993 hybrid, single thread) on the
          same six images, also used to check the GPU output bit for bit.

--impl reference times the reference's CPU path for the same workload.  The
reference has no CPU implementation, so that is the oracle port, one host
thread per image (6), on the same metric and config.

Multi-GPU (torchrun, N > 1): replicas only -- every rank reconstructs its own
copy of the workload, no collective on the data path; value = all ranks'
pixels / max time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

REPO = os.path.dirname(os.path.abspath(__file__))
for p in (os.path.join(REPO, "iwpp-mp_gb300"), REPO):
    if p not in sys.path:
        sys.path.insert(0, p)

METRIC = "Gpixels/s bit-exact reconstruction (plain vs batched); served p50/p99 latency"
UNIT = "Gpixels/s"
WORKLOAD = ("4096x4096 uint8 plain reconstruction, seed 1, sigma 8, 2000 discs, h-dome h in {10,40,100} x "
            "connectivity {4,8} (6 images per step), unique queue")


def _dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, FileNotFoundError):
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "samples": len(sm),
                "reasons": sorted(reasons)}


def load_workload():
    from iwpp import synth

    mask = synth.config1_mask()
    cases = []
    for conn, h in synth.CONFIG1_CASES:
        cases.append((conn, h, synth.hdome_marker(mask, h)))
    return mask, cases


def cpu_oracle_cases(mask, cases, threads: int):
    """Runs the oracle on every case; returns (results, seconds)."""
    import oracle
    from concurrent.futures import ThreadPoolExecutor

    t0 = time.perf_counter()
    if threads <= 1:
        res = [oracle.reconstruct(m, mask, conn) for conn, _, m in cases]
    else:
        with ThreadPoolExecutor(max_workers=threads) as ex:  # ctypes releases the GIL
            res = list(ex.map(lambda c: oracle.reconstruct(c[2], mask, c[0]), cases))
    return res, time.perf_counter() - t0


def traffic_from_profile():
    path = os.path.join(REPO, "profiles", "engine_traffic.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return d.get("bytes_per_launch")
    except (OSError, ValueError):
        return None


def peak_hbm():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, ValueError, KeyError):
        return 6800.0, "fallback"


def run_reference(args):
    world, rank, _ = _dist_env()
    if rank != 0:
        return 0
    mask, cases = load_workload()
    px = sum(m.size for _, _, m in cases)
    threads = min(len(cases), os.cpu_count() or 1)
    for _ in range(args.warmup):
        cpu_oracle_cases(mask, cases, threads)
    t_total = 0.0
    for _ in range(args.steps):
        _, dt = cpu_oracle_cases(mask, cases, threads)
        t_total += dt
    value = px * args.steps / t_total / 1e9
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_total / args.steps * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u8", "data": "synthetic",
        "config": {"workload": WORKLOAD, "l2": "n/a (host)"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": "the full step: six 4096x4096 uint8 reconstructions, one host thread each "
                                   "(the reference has no CPU path; this is the oracle restatement)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_ours(args):
    import numpy as np
    import torch

    import iwpp

    world, rank, local = _dist_env()
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", init_method="env://")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    variant = args.variant
    mask_np, cases = load_workload()
    H, W = mask_np.shape
    px_step = W * H * len(cases)
    bytes_per_recon = 3 * W * H * 1

    # device-resident inputs: one mask, pristine markers, working markers
    mask = torch.from_numpy(mask_np).to(dev)
    pristine = [torch.from_numpy(m).to(dev) for _, _, m in cases]
    work = [p.clone() for p in pristine]
    conns = [c for c, _, _ in cases]
    handle = iwpp.Handle(local)
    lib = iwpp.load()
    stream = torch.cuda.Stream(dev)
    sptr = stream.cuda_stream
    vcode = iwpp._variant(variant)
    cfg = iwpp.Config.make(tile_rows=args.tile_rows) if args.tile_rows else None
    cfgp = __import__("ctypes").byref(cfg) if cfg is not None else None

    def step(ev_pairs=None):
        for i in range(len(cases)):
            work[i].copy_(pristine[i], non_blocking=True)
            if ev_pairs is not None:
                ev_pairs[i][0].record(stream)
            st = lib.iwpp_reconstruct_async(handle.ptr, work[i].data_ptr(), mask.data_ptr(), W, W, W, H, 0, conns[i],
                                            vcode, cfgp, sptr)
            if st != 0:
                raise iwpp.IwppError(st, "iwpp_reconstruct_async")
            if ev_pairs is not None:
                ev_pairs[i][1].record(stream)

    with torch.cuda.stream(stream):
        for _ in range(max(args.warmup, 3)):
            step()
        stream.synchronize()
        # bit-exact check of the warm-up results against the oracle
        results = [w.cpu().numpy() for w in work]
    cpu_res, cpu_secs = (None, None)
    if rank == 0 and not args.no_cpu:
        cpu_res, cpu_secs = cpu_oracle_cases(mask_np, cases, 1)
    bitexact = None
    if cpu_res is not None:
        bitexact = all(np.array_equal(a, b) for a, b in zip(results, cpu_res))

    # ---- device-resident timed region
    clocks = ClockSampler(local)
    ev = [[(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in cases]
          for _ in range(args.steps)]
    t_start, t_end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks.start()
    with torch.cuda.stream(stream):
        t_start.record(stream)
        for k in range(args.steps):
            step(ev[k])
        t_end.record(stream)
    torch.cuda.synchronize()
    clock_info = clocks.stop()
    elapsed_ms = t_start.elapsed_time(t_end)
    recon_ms = [a.elapsed_time(b) for row in ev for (a, b) in row]
    if world > 1:
        t = torch.tensor([elapsed_ms], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        elapsed_ms = float(t.item())
        torch.distributed.barrier()
    value = world * px_step * args.steps / (elapsed_ms / 1e3) / 1e9

    # ---- end to end: host buffers, reference-facing synchronous call
    e2e = None
    if rank == 0 or world > 1:
        host_m = [torch.from_numpy(m).pin_memory() for _, _, m in cases]
        host_k = torch.from_numpy(mask_np).pin_memory()
        host_out = [torch.empty_like(h) for h in host_m]
        dm = torch.empty((H, W), dtype=torch.uint8, device=dev)
        dk = torch.empty((H, W), dtype=torch.uint8, device=dev)

        def e2e_step():
            for i in range(len(cases)):
                dm.copy_(host_m[i], non_blocking=True)
                dk.copy_(host_k, non_blocking=True)
                iwpp.reconstruct(dm, dk, connectivity=conns[i], variant=variant, config=cfg, handle=handle)
                host_out[i].copy_(dm, non_blocking=True)
            torch.cuda.current_stream().synchronize()

        for _ in range(max(args.warmup, 3)):
            e2e_step()
        e2e_ok = all(np.array_equal(host_out[i].numpy(), results[i]) for i in range(len(cases)))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            e2e_step()
        e2e_s = time.perf_counter() - t0
        e2e = {"value": world * px_step * args.steps / e2e_s / 1e9, "unit": UNIT,
               "h2d_bytes_per_step": len(cases) * 2 * W * H, "d2h_bytes_per_step": len(cases) * W * H,
               "bitexact_vs_device_path": e2e_ok}

    if rank != 0:
        if world > 1:
            torch.distributed.destroy_process_group()
        return 0
    peak, peak_kind = peak_hbm()
    mean_recon_ms = sum(recon_ms) / len(recon_ms)
    achieved = bytes_per_recon / (mean_recon_ms / 1e3) / 1e9
    traffic = traffic_from_profile()
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": max(args.warmup, 3), "ms_per_step": elapsed_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u8", "data": "synthetic",
        "config": {"workload": WORKLOAD, "variant": variant, "tile_rows": args.tile_rows or "default",
                   "l2": "inputs larger than L2: 6 working + 6 pristine markers + mask = 218 MB per step",
                   "parallelism": f"replicas x{world}" if world > 1 else "single GPU"},
        "bitexact": bitexact,
        "e2e": e2e,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic, "peak_source": peak_kind,
                     "kernel": "iwpp::engine_kernel (persistent tile engine) + its init kernel",
                     "algorithmic_bytes_per_launch": bytes_per_recon, "mean_launch_ms": mean_recon_ms},
        "cpu_baseline": None if cpu_secs is None else {
            "value": px_step / cpu_secs / 1e9, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": "the same six 4096x4096 uint8 reconstructions, oracle (Vincent 1993 hybrid), one thread"},
        "clocks": clock_info,
        "gpu_launches": args.steps * len(cases) * 2,
    }
    print(json.dumps(line), flush=True)
    handle.close()
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--variant", default="unique", choices=["mutex", "double", "unique"])
    ap.add_argument("--tile-rows", type=int, default=0)
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline / bit-exact check")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    import __graft_entry__ as ge

    ge.build()
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
