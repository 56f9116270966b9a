#!/usr/bin/env python3
"""Benchmark: Voronoi cells per second on the periodic 4M-particle box.

Workload (the configuration the headline metric is quoted on): a
container_periodic cube of side L = 100 with 4,000,000 particles i.i.d.
uniform (seed 1002), the reference's block grid 93^3 (about 5 particles per
block).  A step is one full compute_all_cells(): binning (put() into blocks)
plus every cell, with per-cell volume, face count and neighbour IDs kept.

  value  cells/s with the particles already resident in HBM (device-timed with
         CUDA events around each compute on the engine's stream; the L2 is
         flushed between steps by writing a 512 MiB buffer, outside the timing)
  e2e    cells/s through the public API with host buffers: put() from pinned
         host memory, compute, and a device->host read of the volumes, face
         counts and neighbour lists, all inside the timed region

``--impl reference`` times the reference's CPU path on the host cores instead
(the CPU oracle port built from oracle/port, all host threads, a bounded
sample of the same workload).  Under torchrun with N > 1 every rank computes
its own independent container (weak scaling, no collective on the data path).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

ALGO_BYTES_PER_CELL = 136.0  # 32 B position+radius in, 4 B id, ~100 B out (vol, centroid, counts, 15.5 ids)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--mode", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--n", type=int, default=4_000_000)
    ap.add_argument("--density", type=float, default=0.0, help="engine particles per block (0 = default)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-tune", action="store_true", help="skip the density autotuner (library default)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--workload", default="periodic", choices=["periodic", "batched"],
                    help="periodic: the 4M periodic box (the headline); batched: many containers")
    ap.add_argument("--count", type=int, default=4096, help="batched: number of containers")
    ap.add_argument("--nmax", type=int, default=100_000, help="batched: largest container")
    ap.add_argument("--no-fp64", action="store_true", help="skip the plain FP64 engine on the same box")
    ap.add_argument("--no-c4", action="store_true", help="skip the jittered-FCC (near-degenerate) leg")
    ap.add_argument("--no-batched", action="store_true", help="skip the batched-containers leg")
    ap.add_argument("--batch-count", type=int, default=1024, help="containers of the batched leg")
    ap.add_argument("--batch-nmax", type=int, default=100_000, help="largest container of the batched leg")
    ap.add_argument("--cpu-one-core-seconds", type=float, default=8.0)
    ap.add_argument("--fp64-fallback", type=float, default=0.0,
                    help="mixed engine's FP64 fallback fraction (0: the library default; >= 1: never sample)")
    return ap.parse_args()


def workload(n):
    from voro_gb300 import workloads as W
    L = 100.0 * (n / 4_000_000) ** (1.0 / 3.0)
    g = max(1, int(round((n / 5.0) ** (1.0 / 3.0))))
    return W.periodic_cube(n=n, L=L, seed=1002, grid=(g, g, g))


def workload_name(w):
    """The workload as both arms name it (GPU and reference: same input)."""
    n = len(w["ids"])
    return (f"container_periodic L={w['geom'][0]:.4g}, {n} particles uniform (seed 1002), "
            f"blocks {w['grid'][0]}^3")


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(x, ws, device=None):
    """The maximum of a per-rank time over all ranks (every rank gets it);
    identity for one process.  Replicas compute independent containers, so
    this timing reduction is the only collective."""
    if ws <= 1:
        return float(x)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(cells_per_rank, ws, ms_max):
    """Whole-job cells/s: every rank's cells over the slowest rank's time."""
    return ws * cells_per_rank / (ms_max / 1000.0)


class Clocks:
    """Samples SM clocks and throttle reasons with nvidia-smi while running."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        # the raw samples go to VORO_BENCH_CLOCKS_DIR if set, else a temporary file
        out_dir = os.environ.get("VORO_BENCH_CLOCKS_DIR") or tempfile.gettempdir()
        self.path = os.path.join(out_dir, f"clocks_rank{index}.csv")

    def __enter__(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if self.proc is None or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def load_profile_summary():
    p = os.path.join(ROOT, "profiles", "clip_kernel_periodic_400k.json")
    if os.path.exists(p):
        try:
            return json.load(open(p))
        except Exception:
            return None
    return None


def issue_roof(prof, n, clip_ms, sms, sm_mhz):
    """The clipping kernel against the warp-instruction issue rate, the roof
    that binds it (four warp instructions per cycle per SM): the first
    pass's warp instructions per cell from the ncu capture in profiles/,
    times the cells, over the clipping time of both passes (CUDA events)."""
    ipc = prof.get("warp_instructions_per_cell")
    if ipc is None:
        return None
    peak = sms * 4 * sm_mhz * 1e6 / 1e12
    achieved = ipc * n / (clip_ms / 1000.0) / 1e12
    return {"unit": "T warp instructions/s", "achieved": achieved, "peak": peak, "frac": achieved / peak,
            "instructions_per_cell": ipc, "peak_kind": f"nominal issue ({sms} SMs x 4 x {sm_mhz:.0f} MHz)",
            "capture_issue_active": prof.get("issue_active")}


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d.get("hbm_gbs", 6790.0), "measured"
    return 6800.0, "fallback"


def cpu_baseline(w, seconds, threads=None):
    """Times the CPU oracle port (the reference's algorithm) on a bounded
    sample: the first cells of the same container, all host threads."""
    try:
        from oracle import PortLib, build_port
        build_port()
        port = PortLib()
    except Exception as e:  # noqa: BLE001
        return None, f"port unavailable: {e}"
    threads = threads or os.cpu_count() or 1
    # calibrate: a small sample, then size the real one to `seconds`
    n_total = len(w["ids"])
    t, m = port.time_cells(w, first=0, count=min(20000, n_total), threads=threads)
    rate = m / max(t, 1e-9)
    count = int(min(n_total, max(m, rate * seconds)))
    t, m = port.time_cells(w, first=0, count=count, threads=threads)
    return {"value": m / t, "unit": "cells/s", "cores": threads, "kind": "port",
            "sample": f"first {m} cells (loop order) of the {n_total}-particle container, "
                      f"{threads} threads, {t:.2f} s"}, None


def cpu_one_core(w, seconds):
    """The same CPU port on one thread (bounded sample of the same container)."""
    try:
        from oracle import PortLib, build_port
        build_port()
        port = PortLib()
    except Exception as e:  # noqa: BLE001
        return {"value": None, "unavailable": f"port unavailable: {e}"}
    n_total = len(w["ids"])
    t, m = port.time_cells(w, first=0, count=min(5000, n_total), threads=1)
    count = int(min(n_total, max(m, m / max(t, 1e-9) * seconds)))
    t, m = port.time_cells(w, first=0, count=count, threads=1)
    return {"value": m / t, "unit": "cells/s", "cores": 1, "kind": "port",
            "sample": f"first {m} cells (loop order) of the {n_total}-particle container, 1 thread, {t:.2f} s"}


def fp64_leg(con, n, flush, mixed):
    """The plain FP64 engine (every side test, vertex and reduction in FP64)
    on the same container, device-timed like the headline; its topology is
    compared with the mixed engine's (``mixed``: that compute's results)."""
    import torch
    con.compute_all_cells(mode="fp64")   # warm-up (sizes the FP64 record store)
    ms, clip, fin = [], [], []
    for _ in range(2):
        flush.zero_()
        torch.cuda.synchronize()
        con.compute_all_cells(mode="fp64")
        st = con.stats()
        ms.append(st["step_ms"])
        clip.append(st["clip_ms"])
        fin.append(st["finish_ms"])
    f = con.cells()
    topo = (np.array_equal(f.nf, mixed.nf) and np.array_equal(f.nv, mixed.nv)
            and np.array_equal(f.nb_off, mixed.nb_off) and np.array_equal(f.nb, mixed.nb))
    ok = f.vol > 0
    rel = np.abs(mixed.vol[ok] - f.vol[ok]) / f.vol[ok]
    t = statistics.mean(ms)
    return {"value": n / (t / 1000.0), "unit": "cells/s", "ms_per_step": t, "clip_ms": statistics.mean(clip),
            "finish_ms": statistics.mean(fin), "topology_equal_to_mixed": bool(topo),
            "max_rel_volume_diff_mixed_vs_fp64": float(rel.max()) if len(rel) else 0.0}


def c4_leg():
    """Near-degenerate lattice: 64^3 FCC (a = 1, periodic), every coordinate
    jittered by N(0, (1e-7)^2).  The mixed compute as it runs by default (its
    sample of the first pass hands the container to the FP64 engine), the
    FP32 engine forced through every cell (the rate at which its side tests
    fall back to FP64 and cells are handed on), the plain FP64 engine, and
    the topology agreement of the three."""
    import voro_gb300 as vg
    from voro_gb300 import workloads as W
    w = W.fcc_jitter(cells=64, sigma=1e-7, seed=1004)
    n = len(w["ids"])
    con = vg.from_workload(w, mode="mixed")
    con.compute_all_cells()              # warm-up
    con.compute_all_cells()
    st = con.stats()
    m = con.cells()
    con.set_fp64_fallback(1.0)           # never hand the container over
    con.compute_all_cells()
    con.compute_all_cells()
    stf = con.stats()
    mf = con.cells()
    con.set_fp64_fallback(0.25)
    con.compute_all_cells(mode="fp64")
    con.compute_all_cells(mode="fp64")
    st64 = con.stats()
    f = con.cells()
    same = lambda a: (np.array_equal(f.nf, a.nf) and np.array_equal(f.nv, a.nv) and
                      np.array_equal(f.nb_off, a.nb_off) and np.array_equal(f.nb, a.nb))
    rel = max(float((np.abs(a.vol - f.vol) / f.vol).max()) for a in (m, mf))
    return {"workload": f"FCC 64^3 (a = 1, periodic cube L = 64), {n} particles, jitter sigma 1e-7 (seed 1004)",
            "cells_per_s": n / (st["step_ms"] / 1000.0),
            "cells_on_fp64_engine": int(st["fp64_engine_cells"]),
            "fp64_engine_cells_per_s": n / (st64["step_ms"] / 1000.0),
            "fp32_engine_forced": {
                "cells_per_s": n / (stf["step_ms"] / 1000.0),
                "side_tests": int(stf["side_tests"]), "fp64_repairs": int(stf["fp64_repairs"]),
                "fp64_repairs_per_test": stf["fp64_repairs"] / max(stf["side_tests"], 1),
                "cells_handed_on": int(stf["overflow_reruns"]),
                "cells_handed_on_fraction": stf["overflow_reruns"] / n},
            "marginal_cells": int(stf["marginal_cells"]), "failed_cells": int(st["failed_cells"] + stf["failed_cells"]),
            "topology_equal_to_fp64": bool(same(m) and same(mf)), "max_rel_volume_diff_vs_fp64": rel}


def batched_leg(count, nmax, steps, warmup, mode="mixed"):
    """Many containers (log-uniform sizes, mixed kinds): one vgpu_batch_compute
    (binning per container + one persistent launch for every cell) against a
    loop of per-container computes on the same containers.  Host wall clock."""
    import torch
    import voro_gb300 as vg
    from voro_gb300 import workloads as W
    ws = W.batched(count=count, nmin=64, nmax=nmax, seed=1005)
    total = sum(len(w["ids"]) for w in ws)
    cons = [vg.from_workload(w, mode=mode) for w in ws]
    b = vg.batch(cons)
    for _ in range(warmup):
        b.compute_all_cells(mode=mode)
    wall, kern, binms = [], [], []
    for _ in range(steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        b.compute_all_cells(mode=mode)
        wall.append(time.perf_counter() - t0)
        st = b.stats()
        kern.append(st["kernel_ms"])
        binms.append(st["bin_ms"])
    st = b.stats()
    loop = []
    for it in range(warmup + steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for c in cons:
            c.compute_all_cells(mode=mode)
        torch.cuda.synchronize()
        if it >= warmup:
            loop.append(time.perf_counter() - t0)

    def box_volume(w):
        g = w["geom"]
        return (g[1] - g[0]) * (g[3] - g[2]) * (g[5] - g[4]) if w["kind"] < 2 else g[0] * g[2] * g[5]

    vol_ok = all(abs(c.sum_cell_volumes() - box_volume(w)) <= 1e-9 * box_volume(w) for c, w in zip(cons, ws))
    wt = statistics.mean(wall)
    return {
        "workload": f"{count} containers, N log-uniform [64, {nmax}] (seed 1005), half container_periodic, "
                    f"a quarter radical; {total} particles",
        "value": total / wt, "unit": "cells/s", "ms_per_step": 1000.0 * wt,
        "timing": "host wall clock around vgpu_batch_compute (binning + one persistent launch per pass)",
        "kernel_only_cells_per_s": total / (statistics.mean(kern) / 1000.0),
        "batched_kernel_ms": statistics.mean(kern), "batched_bin_ms": statistics.mean(binms),
        "per_container_loop": {"value": total / statistics.mean(loop), "unit": "cells/s",
                               "ms_per_step": 1000.0 * statistics.mean(loop)},
        "speedup_vs_loop": statistics.mean(loop) / wt,
        "gpu_launches": int(st["kernel_launches"]),
        "engine": {"cells": st["cells"], "failed_cells": st["failed_cells"], "overflow_reruns": st["overflow_reruns"],
                   "marginal_cells": st["marginal_cells"], "sum_volume_ok": bool(vol_ok)},
    }


def reference_tests_per_cell(w, cells=20000):
    """T_cell of the flop model: the reference algorithm's vertex-plane side
    tests (m_calc calls, src/cell.cc:2050-2059) per cell, counted by the CPU
    port on the first cells of the same container."""
    try:
        from oracle import PortLib, build_port
        build_port()
        port = PortLib()
        _, m = port.time_cells(w, first=0, count=min(cells, len(w["ids"])), threads=os.cpu_count() or 1)
        return port.last_side_tests / max(m, 1), m
    except Exception:  # noqa: BLE001
        return None, 0


def run_reference(args):
    ws, rank, local = dist_env()
    if rank != 0:
        return 0
    w = workload(args.n)
    try:
        from oracle import PortLib, build_port
        build_port()
        port = PortLib()
    except Exception as e:  # noqa: BLE001
        print(json.dumps({"impl": "reference", "unavailable": f"CPU oracle port could not be built: {e}"}))
        return 0
    threads = os.cpu_count() or 1
    n_total = len(w["ids"])
    t, m = port.time_cells(w, first=0, count=min(20000, n_total), threads=threads)
    rate = m / max(t, 1e-9)
    per_step = int(min(n_total, max(m, rate * 8.0)))
    for _ in range(args.warmup):
        port.time_cells(w, first=0, count=min(per_step, 20000), threads=threads)
    times = []
    for s in range(args.steps):
        t, m = port.time_cells(w, first=0, count=per_step, threads=threads)
        times.append(t)
    ms = 1000.0 * statistics.mean(times)
    value = per_step / (ms / 1000.0)
    line = {
        "metric": "cells/s (Voronoi cells computed per second)", "value": value, "unit": "cells/s",
        "impl": "reference", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic",
        "config": {"workload": workload_name(w), "cells_per_step": per_step},
        "cpu_baseline": {"value": value, "unit": "cells/s", "cores": threads, "kind": "port",
                         "sample": f"first {per_step} cells of {n_total} per step, {threads} threads"},
        "e2e": {"value": value, "unit": "cells/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def run_ours(args):
    import torch
    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)
    import voro_gb300 as vg

    w = workload(args.n)
    n = len(w["ids"])
    dev = torch.device("cuda", torch.cuda.current_device())
    d_ids = torch.from_numpy(w["ids"]).to(dev)
    d_xyzr = torch.from_numpy(w["xyzr"]).to(dev)
    con = vg.container_periodic(*w["geom"], *w["grid"], 8, mode=args.mode)
    if args.density > 0:
        con.set_tuning(args.density, 0)
    if args.fp64_fallback > 0:
        con.set_fp64_fallback(args.fp64_fallback)
    con.put_device(n, d_ids.data_ptr(), d_xyzr.data_ptr(), keepalive=(d_ids, d_xyzr))
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    def barrier():
        if ws > 1:
            import torch.distributed as dist
            dist.barrier()
        torch.cuda.synchronize()

    tuned = None
    if args.density <= 0 and not args.no_tune:
        tuned = con.autotune()   # the engine's own autotuner: (tuning dict, ms)
    for _ in range(args.warmup):
        con.compute_all_cells()
    barrier()
    step_ms, kern_ms, bin_ms, clip_ms, fin_ms, launches = [], [], [], [], [], 0
    with Clocks(local) as clk:
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            con.compute_all_cells()
            st = con.stats()
            step_ms.append(st["step_ms"])
            kern_ms.append(st["kernel_ms"])
            bin_ms.append(st["bin_ms"])
            clip_ms.append(st["clip_ms"])
            fin_ms.append(st["finish_ms"])
            launches += int(st["kernel_launches"])
    barrier()
    st = con.stats()
    ms = max_over_ranks(statistics.mean(step_ms), ws, dev)
    value = job_throughput(n, ws, ms)
    clocks = clk.summary()

    # correctness guard on the measured configuration
    total = con.sum_cell_volumes()
    box = w["geom"][0] * w["geom"][2] * w["geom"][5]
    vol_ok = abs(total - box) <= 1e-9 * box

    # end to end through the public API with host buffers
    e2e = None
    if not args.no_e2e:
        ids_pin = torch.from_numpy(w["ids"]).pin_memory().numpy()
        xyzr_pin = torch.from_numpy(w["xyzr"]).pin_memory().numpy()
        con2 = vg.container_periodic(*w["geom"], *w["grid"], 8, mode=args.mode)
        if args.density > 0:
            con2.set_tuning(args.density, 0)
        elif tuned is not None:
            con2.set_tuning(tuned[0]["particles_per_block"], tuned[0]["warps_per_cta"], tuned[0]["cells_per_chunk"])
        h2d = ids_pin.nbytes + xyzr_pin.nbytes
        d2h = 0
        times = []
        pinned = lambda shape, dt: torch.empty(tuple(shape), dtype=getattr(torch, np.dtype(dt).name),
                                               pin_memory=True).numpy()
        res = None
        parts = {"put_ms": [], "compute_ms": [], "device_ms": [], "read_ms": []}
        for it in range(args.warmup + args.steps):
            barrier()
            t0 = time.perf_counter()
            con2.clear()
            con2.put_xyzr(ids_pin, xyzr_pin)
            tp = time.perf_counter()
            con2.compute_all_cells()
            tc = time.perf_counter()
            res = con2.cells(neighbors=True, out=res, alloc=pinned)
            torch.cuda.synchronize()
            t1 = time.perf_counter()
            if it >= args.warmup:
                times.append(t1 - t0)
                # where the wall clock went (the compute returns once its
                # results are on the device; device_ms: its CUDA-event time)
                parts["put_ms"].append(1000.0 * (tp - t0))
                parts["compute_ms"].append(1000.0 * (tc - tp))
                parts["device_ms"].append(con2.stats()["step_ms"])
                parts["read_ms"].append(1000.0 * (t1 - tc))
            d2h = (res.vol.nbytes + res.nf.nbytes + res.nb.nbytes + res.nb_off.nbytes + res.ids.nbytes +
                   res.pos.nbytes + res.cen.nbytes + res.nv.nbytes + res.maxr2.nbytes + res.flags.nbytes)
        e2e_s = max_over_ranks(statistics.mean(times), ws, dev)
        e2e = {"value": job_throughput(n, ws, 1000.0 * e2e_s), "unit": "cells/s", "h2d_bytes_per_step": int(h2d),
               "d2h_bytes_per_step": int(d2h), "ms_per_step": 1000.0 * e2e_s,
               "split_ms": {k: statistics.mean(v) for k, v in parts.items()}}

    if rank != 0:
        if ws > 1:
            import torch.distributed as dist
            dist.destroy_process_group()
        return 0

    kms = statistics.mean(kern_ms)
    cms = statistics.mean(clip_ms)
    fms = statistics.mean(fin_ms)
    hbm_peak, peak_kind = peaks()
    # the dominant kernel: the clipping kernel (device time of its launch, CUDA events on its stream)
    achieved_gbs = ALGO_BYTES_PER_CELL * n / (cms / 1000.0) / 1e9
    prof = load_profile_summary() or {}
    traffic = prof.get("dram_bytes_per_cell")
    if traffic is not None:
        traffic = traffic * n   # per launch: the capture's per-cell DRAM bytes times the cells of one launch
    side_tests_per_cell = st["side_tests"] / max(st["cells"], 1)
    t_ref, t_cells = reference_tests_per_cell(w)
    mixed_cells = con.cells()
    v_mean = float(np.mean(mixed_cells.nv))
    flops_cell = 6.0 * (t_ref if t_ref is not None else side_tests_per_cell) + 40.0 * v_mean
    props = torch.cuda.get_device_properties(dev)
    sm_mhz = clocks.get("sm_max_mhz") or 2070.0
    fp32_peak = props.multi_processor_count * 128 * 2 * sm_mhz * 1e6 / 1e12   # FMA lanes per SM: 128
    line = {
        "metric": "cells/s (Voronoi cells computed per second)",
        "value": value, "unit": "cells/s", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32+f64" if args.mode == "mixed" else "f64", "data": "synthetic",
        "config": {"workload": workload_name(w), "engine": args.mode,
                   "cells_per_step": n, "l2": "flushed between steps (512 MiB write)",
                   "engine_density": (tuned[0]["particles_per_block"] if tuned else
                                      (args.density if args.density > 0 else "default")),
                   "tuning": tuned[0] if tuned else con.tuning(),
                   "parallelism": f"{ws} independent replicas" if ws > 1 else "1 GPU"},
        "roofline": {"bound": "hbm", "achieved": achieved_gbs, "peak": hbm_peak, "unit": "GB/s",
                     "frac": achieved_gbs / hbm_peak, "traffic": traffic, "peak_kind": peak_kind,
                     "kernel": "cell_kernel<MIXED,2> (clipping)", "kernel_ms": cms,
                     "note": "instruction-issue/fetch-bound kernel; algorithmic bytes 136 B/cell "
                             "(36 in, 100 out); traffic from the ncu capture in profiles/, scaled by cells",
                     "finish_kernel_ms": fms, "cell_stage_ms": kms,
                     "pipe": {"unit": "TFLOP/s", "achieved": flops_cell * n / (kms / 1000.0) / 1e12,
                              "peak": fp32_peak, "peak_kind": f"nominal FP32 ({props.multi_processor_count} SMs "
                                                               f"x 128 lanes x 2 x {sm_mhz:.0f} MHz)",
                              "flops_per_cell": flops_cell,
                              "model": "F_cell = 6 T_cell + 40 V_cell; T_cell = reference side tests per cell "
                                       f"({t_ref if t_ref is not None else float('nan'):.1f}, CPU port on "
                                       f"{t_cells} cells), V_cell = mean vertices ({v_mean:.2f})"},
                     "issue": issue_roof(prof, n, cms, props.multi_processor_count, sm_mhz)},
        "e2e": e2e,
        "gpu_launches": launches,
        "clocks": clocks,
        "engine": {"kernel_ms": kms, "bin_ms": statistics.mean(bin_ms), "side_tests_per_cell": side_tests_per_cell,
                   "fp64_repairs": st["fp64_repairs"], "marginal_cells": st["marginal_cells"],
                   "overflow_reruns": st["overflow_reruns"], "failed_cells": st["failed_cells"],
                   "planes_tested_per_cell": st["planes_tested"] / max(st["cells"], 1),
                   "planes_cut_per_cell": st["planes_cut"] / max(st["cells"], 1),
                   "sum_volume_ok": bool(vol_ok)},
    }
    if ws == 1 and args.mode == "mixed" and not args.no_fp64:
        line["fp64"] = fp64_leg(con, n, flush, mixed_cells)
        line["mixed_over_fp64"] = value / line["fp64"]["value"]
    del mixed_cells, con
    if ws == 1 and not args.no_c4:
        line["c4"] = c4_leg()
    if ws == 1 and not args.no_batched:
        line["batched"] = batched_leg(args.batch_count, args.batch_nmax, steps=2, warmup=1, mode=args.mode)
    if ws == 1 and not args.no_cpu:
        cb, err = cpu_baseline(w, args.cpu_seconds)
        line["cpu_baseline"] = cb if cb else {"value": None, "unavailable": err}
        if cb:
            cb["one_core"] = cpu_one_core(w, args.cpu_one_core_seconds)
    print(json.dumps(line))
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


def run_batched(args):
    """The batched workload alone as the headline line (--workload batched)."""
    import torch
    torch.cuda.set_device(0)
    with Clocks(0) as clk:
        b = batched_leg(args.count, args.nmax, args.steps, args.warmup, mode=args.mode)
    line = {
        "metric": "cells/s (Voronoi cells computed per second), batched containers",
        "value": b.pop("value"), "unit": "cells/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": b.pop("ms_per_step"), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32+f64" if args.mode == "mixed" else "f64", "data": "synthetic",
        "config": {"workload": b.pop("workload"), "timing": b.pop("timing")},
        "clocks": clk.summary(),
    }
    line.update(b)
    print(json.dumps(line))
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "batched":
        return run_batched(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
