#!/usr/bin/env python3
"""Benchmark of the Voxel Cores hot path on GB300: end-to-end voxels/s.

A step is one pass of the whole path over one synthetic volume: boundary
sites, exact feature transform, lattice Voronoi complex with lambda measures,
FIFO-exact thinning at thresh = inside_size * t, and the remaining complex.
The default workload is the 512^3 thresholded Gaussian random field (white
noise blurred with sigma = 6 voxels, level 0).

  value : voxels/s with the volume already resident in HBM (device pointer in,
          device-resident results), timed with CUDA events on the library's
          stream.
  e2e   : the same metric through the public C-ABI call with HOST buffers:
          the volume is copied from pinned host memory every step and the
          remaining complex is read back to pinned host memory.

``--impl reference`` times the CPU implementation of the same path (the
restated reference algorithm in oracle/, single-threaded like the reference)
on a bounded sample of the workload, with the same metric and JSON line.
Under torchrun, ranks are independent replicas (each processes its own
volume); the timed region is bracketed by a barrier and the max over ranks
is taken.
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

METRIC = "end-to-end voxels/s at 512^3 (EDT+measure+thin), batched vs plain GPU; p99 ms"
UNIT = "voxels/s"
FALLBACK_HBM_GBS = 6800.0
CPU_SAMPLE_N = 128  # edge of the GRF sample timed on the host cores


def measured_hbm_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def make_workload(name: str, device=None):
    from voxel_ma_gb300 import volumes
    if name == "grf512":
        return volumes.grf(512, sigma=6.0, seed=0, device=device), "grf512_sigma6_level0"
    if name == "grf192":
        return volumes.grf(192, sigma=6.0, seed=0, device=device), "grf192_sigma6_level0"
    if name == "grf256":
        return volumes.grf(256, sigma=6.0, seed=0, device=device), "grf256_sigma6_level0"
    if name == "spheres256":
        return volumes.spheres(256, count=32, seed=0), "spheres256_32_seed0"
    if name == "torus64":
        return volumes.torus_mesh(64), "torus64_mesh"
    raise SystemExit(f"unknown workload {name}")


# ---------------------------------------------------------------------------
# CPU side (reference arm and cpu_baseline): the oracle's restatement of the
# reference algorithm, timed on a bounded sample of the workload.

def cpu_path_once(occ, t):
    import oracle
    t0 = time.perf_counter()
    oracle.run_plain(occ, t=t, threads=1)
    return time.perf_counter() - t0


def cpu_sample():
    from voxel_ma_gb300 import volumes
    occ = volumes.grf(CPU_SAMPLE_N, sigma=6.0, seed=0)
    return occ, f"GRF sigma=6 level 0 at {CPU_SAMPLE_N}^3 (same field statistics as the 512^3 workload)"


_REF_OCC = None


def _ref_worker_init():
    global _REF_OCC
    import oracle
    oracle.build(reference=False)
    _REF_OCC = cpu_sample()[0]


def _ref_worker_run(t):
    return cpu_path_once(_REF_OCC, t)


def host_threads() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def run_reference(args):
    """The reference's CPU path on every host thread: the reference is
    single-threaded per volume (its thinning is one FIFO queue), so the host's
    throughput is one volume per thread at a time.  Each step runs one sample
    volume on each of `threads` worker processes at once; voxels/s = threads x
    sample voxels / the step's wall time."""
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    import multiprocessing as mp
    import oracle
    oracle.build(reference=False)
    occ, sample = cpu_sample()
    nvox = occ.size
    threads = host_threads()
    ctx = mp.get_context("spawn")
    with ctx.Pool(threads, initializer=_ref_worker_init) as pool:
        def step():
            t0 = time.perf_counter()
            pool.map(_ref_worker_run, [args.t] * threads, chunksize=1)
            return time.perf_counter() - t0
        for _ in range(args.warmup):
            step()
        times = [step() for _ in range(args.steps)]
    mean = statistics.mean(times)
    value = threads * nvox / mean
    sample_desc = f"{threads} concurrent single-threaded runs, one per host thread, each on {sample}"
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": mean * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int32+f32",
        "data": "synthetic (seeded thresholded Gaussian random field)",
        "config": {"workload": "grf512_sigma6_level0", "sample": sample_desc, "t": args.t},
        "latency_ms": {"p50": float(np.percentile(times, 50) * 1e3), "p99": float(np.percentile(times, 99) * 1e3)},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample_desc},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------
# clocks during the timed region

class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None
        self.t_start = None
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                       "-lms", "200", "-i", str(device_index)], stdout=self.f,
                                      stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def wait_ready(self, timeout: float = 20.0):
        """Block until the sampler has written its first line, so that its
        start-up (which can stall driver calls) happens before timing."""
        t0 = time.time()
        while self.p is not None and time.time() - t0 < timeout:
            if os.path.getsize(self.f.name) > 0:
                break
            time.sleep(0.05)

    def mark(self):
        """Only samples taken after mark() are summarised."""
        self.f.flush()
        self.t_start = os.path.getsize(self.f.name)

    def stop(self):
        if self.p is not None:
            self.p.terminate()
            try:
                self.p.wait(timeout=5)
            except Exception:
                self.p.kill()
        self.f.flush()
        rows = []
        try:
            fh = open(self.f.name)
            if self.t_start:
                fh.seek(self.t_start)
                fh.readline()  # possibly partial line
            for line in fh:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9 and parts[1].replace(".", "").isdigit():
                    rows.append(parts)
        finally:
            os.unlink(self.f.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["clock sampling unavailable"]}
        sm = [float(r[1]) for r in rows]
        mx = max(float(r[2]) for r in rows)
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": reasons, "samples": len(rows),
                "power_w_max": max(float(r[3]) for r in rows if r[3].replace(".", "").isdigit())
                if any(r[3].replace(".", "").isdigit() for r in rows) else None}


# ---------------------------------------------------------------------------

KERNEL_REGIONS = ("thin_generations", "ft_rows", "ft_envelope_y", "ft_envelope_x", "vd_flags", "vd_emit",
                  "adjacency", "stage_sites", "stage_remaining")


def algorithmic_bytes(region: str, shape, vd: dict, nsites: int) -> float:
    """Compulsory bytes one launch of `region` moves: every input read once and
    every output written once (for the thinning: each record, the measures and
    the incidences of the complex once)."""
    X, Y, Z = shape
    N = (X + 1) * (Y + 1) * (Z + 1)
    nvox = X * Y * Z
    V, E, T, F = vd["nv"], vd["ne"], vd["nt"], vd["nface"]
    if region == "thin_generations":
        return 4 * (V + E + T) + 8 * E + 12 * T + 4 * (2 * E + 3 * T) + (V + E + T)
    if region == "ft_rows":
        return 12.0 * N
    if region in ("ft_envelope_y", "ft_envelope_x"):
        return 16.0 * N
    if region == "vd_flags":
        return 17.0 * N + nvox
    if region == "vd_emit":
        return 17.0 * N + 16 * V + 12 * E + 32 * T + 8 * F
    if region == "adjacency":
        return 8 * E + 12 * T + 4 * (V + 1) + 8 * E + 4 * (E + 1) + 12 * T
    if region == "stage_sites":
        return nvox + 4.0 * N + 12 * nsites
    if region == "stage_remaining":
        return 4 * (V + E + T) * 2
    return 0.0


def max_over_ranks(ms: float, dist=None, device=None) -> float:
    """The slowest rank's time (every rank calls it; one process: unchanged)."""
    if dist is None:
        return ms
    import torch
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(world: int, voxels_per_rank: int, steps: int, max_ms: float) -> float:
    """Whole-job voxels/s of `world` independent replicas (one volume per rank
    per step, weak scaling) timed by the slowest rank."""
    return world * voxels_per_rank * steps / (max_ms / 1e3)


def run_gpu(args):
    import torch

    from voxel_ma_gb300 import api

    rank, world, local = dist_env()
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    occ_np, workload = make_workload(args.workload, device=dev if args.workload.startswith("grf") else None)
    from voxel_ma_gb300 import volumes
    occ_sha = volumes.occupancy_sha256(occ_np)
    if workload in volumes.WORKLOAD_SHA256 and occ_sha != volumes.WORKLOAD_SHA256[workload]:
        raise SystemExit(f"{workload}: occupancy digest {occ_sha} is not the tested volume's")
    occ_dev = torch.from_numpy(occ_np).to(dev)
    occ_host = torch.from_numpy(occ_np).pin_memory()
    shape = tuple(occ_np.shape)
    nvox = int(np.prod(shape))

    ctx = api.Context(local)
    stream = ctx.torch_stream()

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize(dev)
        ctx.sync()

    # ---- autotuner (outside the timed region): launch shapes for this input
    tuned = None
    if not args.no_tune:
        ctx.set_volume(occ_dev)
        tuned = ctx.autotune(args.t)
    elif args.ft_method:
        ctx.set_ft_method(args.ft_method)

    # ---- device-resident value ------------------------------------------
    clocks = ClockSampler(local)
    clocks.wait_ready()
    for _ in range(args.warmup):
        r = ctx.run_plain(occ_dev, args.t)
    barrier()
    ctx.set_timing(True)
    ctx.reset_timings()
    launches0 = ctx.launch_count()
    clocks.mark()
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    evs[0].record(stream)
    for k in range(args.steps):
        r = ctx.run_plain(occ_dev, args.t)
        evs[k + 1].record(stream)
    torch.cuda.synchronize(dev)
    ctx.sync()
    launches = ctx.launch_count() - launches0
    timings = ctx.timings()
    ctx.set_timing(False)
    step_ms = [evs[k].elapsed_time(evs[k + 1]) for k in range(args.steps)]
    total_ms = max_over_ranks(evs[0].elapsed_time(evs[-1]), dist, dev)
    value = replica_throughput(world, nvox, args.steps, total_ms)

    # ---- end to end through the C ABI with host buffers -------------------
    rem = r["rem"]
    h_v = torch.empty((max(rem["nv"], 1), 3), dtype=torch.float32).pin_memory()
    h_e = torch.empty((max(rem["ne"], 1), 2), dtype=torch.int32).pin_memory()
    h_t = torch.empty((max(rem["nt"], 1), 3), dtype=torch.int32).pin_memory()

    def e2e_step():
        rr = ctx.run_plain(occ_host, args.t)
        s = rr["rem"]
        ctx.remaining_arrays_into(h_v[: s["nv"]], h_e[: s["ne"]], h_t[: s["nt"]])
        return rr

    for _ in range(max(1, args.warmup // 2)):
        e2e_step()
    barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    w0 = time.perf_counter()
    e0.record(stream)
    for _ in range(args.steps):
        rr = e2e_step()
    e1.record(stream)
    torch.cuda.synchronize(dev)
    wall_e2e = time.perf_counter() - w0
    e2e_ms = max_over_ranks(e0.elapsed_time(e1), dist, dev)
    clk = clocks.stop()
    # the CPU path's scaling points run in a child process beside the rest of
    # the legs, started only now: while it runs its 512^3 point (tens of GB of
    # host memory traffic) the host copies of an end-to-end step slow down
    # (59.9 -> 62.1-66.8 ms per step measured; device-resident steps unchanged)
    scaling = CpuScaling(args.t) if (rank == 0 and not args.no_cpu_baseline and not args.no_cpu_scaling) else None
    s = rr["rem"]
    d2h = s["nv"] * 12 + s["ne"] * 8 + s["nt"] * 12
    e2e_value = replica_throughput(world, nvox, args.steps, e2e_ms)

    # ---- topology (outside the timed regions): nClosedComponents of the
    # workload's complex -- an all-pass thinning plus face components
    closed = None
    if not args.no_probe:
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        n_closed = ctx.closed_components()
        closed = {"value": n_closed, "ms": (time.perf_counter() - t0) * 1e3,
                  "note": "nClosedComponents of the 512^3 lattice complex (all-pass thinning + face components), "
                          "host wall time of one call"}
        ctx.run_plain(occ_dev, args.t)  # the context holds the workload's own thinning again

    # ---- output formats (outside the timed regions): the remaining complex
    # written as the reference's pipeline writes it after thinning
    export = None
    if not args.no_probe:
        import tempfile
        from voxel_ma_gb300 import _lib
        try:
            with tempfile.TemporaryDirectory() as td:
                prefix = os.path.join(td, "grf512_thinned")
                t0 = time.perf_counter()
                ctx.write_remaining(prefix)
                ex_ms = (time.perf_counter() - t0) * 1e3
                sizes = {ext: os.path.getsize(prefix + ext) for ext in (".ply", ".r", ".ma")}
            export = {"ms": ex_ms, "bytes": sizes, "MB_per_s": sum(sizes.values()) / ex_ms / 1e3,
                      "note": "vc_write_remaining (.ply + .r + .ma) of the workload's remaining complex, "
                              "host wall time of one call (device read-back included)"}
        except (OSError, _lib.VoxelCoreError) as exc:
            # about 1.4 GB of text: a host without that much temporary space skips it
            export = {"unavailable": f"{type(exc).__name__}: {exc}"}

    # ---- octree input (outside the timed regions): the workload written as the
    # reference's .sof octree (host encoder), then decoded on the GPU
    octree = None
    if not args.no_probe:
        t0 = time.perf_counter()
        sof = api.encode_sof(occ_np)
        enc_s = time.perf_counter() - t0
        oct_ctx = api.Context(local)
        oct_ctx.set_timing(True)
        dec = []
        for _ in range(4):
            torch.cuda.synchronize(dev)
            oct_ctx.reset_timings()
            t0 = time.perf_counter()
            size = oct_ctx.set_volume_sof(sof)
            dec.append(time.perf_counter() - t0)
        # device time of the decode kernels (walks, large nodes, voxels) in the last call
        oct_gpu_ms = oct_ctx.timings().get("octree_decode", (float("nan"), 0))[0]
        n_oct_sites = oct_ctx.extract_sites()
        same = bool(np.array_equal(oct_ctx.volume()[: shape[0], : shape[1], : shape[2]], occ_np > 0))
        oct_ctx.close()
        dec_s = min(dec[1:])
        octree = {"file_bytes": len(sof), "voxels": size ** 3, "decode_ms": dec_s * 1e3,
                  "decode_voxels_per_s": size ** 3 / dec_s, "encode_ms_host": enc_s * 1e3,
                  "octree_sites": n_oct_sites, "round_trip": same, "decode_gpu_ms_last_call": oct_gpu_ms,
                  "note": "vc_set_volume_sof (host split pass over the type bytes + GPU subtree walks, stream copy included), best of 3 after one untimed call"}

    # ---- roofline of the dominant kernel -----------------------------------
    peak, peak_kind = measured_hbm_peak()
    regions = {k: v for k, v in timings.items() if k in KERNEL_REGIONS}
    dom = max(regions, key=lambda k: regions[k][0]) if regions else None
    roof = None
    if dom:
        ms, cnt = regions[dom]
        per_launch_s = ms / cnt / 1e3
        ab = algorithmic_bytes(dom, shape, r["vd"], r["n_sites"])
        ach = ab / per_launch_s / 1e9
        roof = {"kernel": dom, "bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s",
                "frac": ach / peak, "peak_kind": peak_kind, "algorithmic_bytes_per_launch": ab,
                "traffic": (TRAFFIC_PER_CELL[dom] * (r["vd"]["nv"] + r["vd"]["ne"] + r["vd"]["nt"])
                            if dom in TRAFFIC_PER_CELL else None),
                "traffic_source": ("ncu capture of the 192^3 case of this workload, scaled by cells"
                                   if dom in TRAFFIC_PER_CELL else None)}
        if dom in L2_REQUESTS_PER_CELL and not args.no_probe:
            # the thinning touches random records: its L2 request rate beside
            # the rates this GPU serves random 32-byte record touches at
            cells = r["vd"]["nv"] + r["vd"]["ne"] + r["vd"]["nt"]
            req_s = L2_REQUESTS_PER_CELL[dom] * cells / per_launch_s
            probe = {}
            try:
                for op, name in ((0, "load_8B"), (1, "two_loads_16B"), (2, "atomic_add"), (3, "atomic_max_and_add")):
                    probe[name] = ctx.debug_random_rate(op, PROBE_BYTES)
            except RuntimeError as exc:  # e.g. not enough free device memory for the probe's array
                probe = {"unavailable": str(exc)[:200]}
            roof["random_access"] = {
                "l2_requests_per_s": req_s,
                "l2_requests_source": "ncu capture of the 192^3 case (requests per cell) x cells / kernel time",
                "probe_record_touches_per_s": probe, "probe_array_bytes": PROBE_BYTES,
                "note": "probe: random 32-byte records in a 16 GB array (vc_debug_random_rate), best of 3"}
    stage_ms = {k: v[0] / max(v[1], 1) for k, v in sorted(timings.items())}

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int32+f32",
        "data": "synthetic (seeded thresholded smoothed random field, exact integer generator, blurred on device)",
        "config": {"workload": workload, "shape": list(shape), "t": args.t, "path": "plain single-volume",
                   "occupancy_sha256": occ_sha,
                   "l2": "inputs larger than L2 (per-step working set %.1f GB)" % (ctx.device_bytes() / 1e9),
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "latency_ms": {"p50": float(np.percentile(step_ms, 50)), "p99": float(np.percentile(step_ms, 99))},
        "complex": {"sites": r["n_sites"], "V": r["vd"]["nv"], "E": r["vd"]["ne"], "T": r["vd"]["nt"],
                    "thresh": r["thresh"], "generations": r["thin"]["generations"],
                    "processed": r["thin"]["processed"], "remaining": r["rem"]},
        "region_ms_per_step": stage_ms,
        "roofline": roof,
        "closed_components": closed,
        "octree": octree,
        "export": export,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": nvox, "d2h_bytes_per_step": d2h,
                "ms_per_step": e2e_ms / args.steps, "wall_s": wall_e2e},
        "gpu_launches": launches,
        "clocks": clk,
        "fp64_rescues": 0,
        "lambda_note": "lambda = sqrt of an exact integer squared distance (< 2^24) in IEEE f32: no FP64 rescue needed",
        "tuned": tuned,
    }
    # FP32 measures against FP64 on this workload's complex (outside the timed region)
    line["fp64_check"] = ctx.lambda_fp64_check()
    if not args.no_batch:
        line["batched"] = run_batched(ctx, dev, args, stream, dist)
        line["config"]["batched_workload"] = line["batched"]["workload"]
    if not args.no_serve and world == 1:
        ctx.close()
        line["serving"] = run_serving(dev, args)
        line["config"]["serving_workload"] = line["serving"]["workload"]
    if not args.no_1024 and world == 1:
        ctx.close()
        del occ_dev, occ_host
        torch.cuda.empty_cache()
        line["grf1024"] = run_grf1024(dev, args)
    if rank == 0 and not args.no_cpu_baseline:
        occ_s, sample = cpu_sample()
        times = [cpu_path_once(occ_s, args.t) for _ in range(2)]
        line["cpu_baseline"] = {"value": occ_s.size / min(times), "unit": UNIT, "cores": 1, "kind": "port",
                                "sample": sample + "; best of 2 runs of the oracle restatement"}
        if scaling is not None:
            line["cpu_baseline"]["scaling"] = scaling.collect()
    if rank == 0:
        print(json.dumps(line), flush=True)
    ctx.close()
    if dist is not None:
        dist.destroy_process_group()
    return 0


def _rem_digest(v, e, t) -> str:
    import hashlib
    h = hashlib.sha256()
    for a in (v, e, t):
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def _batch_remaining(ctx, res):
    """Each volume's remaining arrays (host numpy) of the batch in ctx."""
    return [(x["rem_vts"], x["rem_edges"], x["rem_tris"]) for x in ctx.batch_split(res)]


# ---------------------------------------------------------------------------
# Batched path: 256 random CSG volumes of per-axis sizes log-uniform in
# [32, 192] through one vc_batch_run per step, against the plain path looping
# over the same volumes one vc_run_plain at a time.

BATCH_N, BATCH_LO, BATCH_HI = 256, 32, 192


def run_batched(ctx, dev, args, stream, dist=None):
    """Under torchrun each rank takes its share of whole volumes
    (vc_partition_volumes by voxels) and runs it as one batch; value counts
    every rank's voxels over the slowest rank's time."""
    import torch

    from voxel_ma_gb300 import api, volumes
    rank, world, _ = dist_env()
    plans = [volumes._csg_plan(1000 + i, BATCH_LO, BATCH_HI)[0] for i in range(BATCH_N)]
    part = api.partition_volumes([int(np.prod(d)) for d in plans], world)
    mine = [i for i in range(BATCH_N) if part[i] == rank]
    all_voxels = int(sum(int(np.prod(d)) for d in plans))
    vols = [volumes.csg(1000 + i, BATCH_LO, BATCH_HI, device=dev) for i in mine]
    dims = np.array([tuple(v.shape) for v in vols], np.int32)
    sizes = [int(np.prod(d)) for d in dims]
    offs = np.concatenate([[0], np.cumsum(sizes)])
    occ_dev = torch.cat([v.reshape(-1) for v in vols])
    del vols
    occ_host = occ_dev.cpu().pin_memory()
    nvox = int(offs[-1])
    nmine = len(mine)
    views = [occ_dev[offs[i]:offs[i + 1]].view(*(int(x) for x in dims[i])) for i in range(nmine)]

    def batched():
        ctx.batch_set_volumes(occ=occ_dev, dims=dims)
        return ctx.batch_run(args.t, euler=False)

    tuned = None
    if not args.no_tune:  # the batch's own launch shapes (outside the timed region)
        ctx.batch_set_volumes(occ=occ_dev, dims=dims)
        tuned = ctx.autotune(args.t)

    def loop():
        return [ctx.run_plain(v, args.t)["rem"] for v in views]

    def timed(fn, steps):
        evs = [torch.cuda.Event(enable_timing=True) for _ in range(steps + 1)]
        evs[0].record(stream)
        out = None
        for k in range(steps):
            out = fn()
            evs[k + 1].record(stream)
        torch.cuda.synchronize(dev)
        ctx.sync()
        return out, [evs[k].elapsed_time(evs[k + 1]) for k in range(steps)]

    for _ in range(args.warmup):
        res = batched()
    if dist is not None:
        dist.barrier()
    launches0 = ctx.launch_count()
    res, b_ms = timed(batched, args.steps)
    b_launches = (ctx.launch_count() - launches0) / args.steps
    b_total = max_over_ranks(sum(b_ms), dist, dev)
    for _ in range(max(1, args.warmup // 2)):
        loop()
    launches0 = ctx.launch_count()
    rem_loop, l_ms = timed(loop, max(1, args.steps // 2))
    l_launches = (ctx.launch_count() - launches0) / max(1, args.steps // 2)
    # parity: each volume's remaining arrays, batched against its own plain run (digests)
    same = 0
    ctx.batch_set_volumes(occ=occ_dev, dims=dims)
    res = ctx.batch_run(args.t, euler=False)
    batch_digests = [_rem_digest(*a) for a in _batch_remaining(ctx, res)]
    for k, v in enumerate(views):
        ctx.run_plain(v, args.t)
        same += int(_rem_digest(*ctx.remaining_arrays()) == batch_digests[k])
    ctx.batch_set_volumes(occ=occ_dev, dims=dims)
    res = ctx.batch_run(args.t, euler=False)

    # end to end: host volumes in, remaining complexes out, every step
    tot = {k: sum(r["rem"][k] for r in res) for k in ("nv", "ne", "nt")}
    h_v = torch.empty((max(tot["nv"], 1), 3), dtype=torch.float32).pin_memory()
    h_e = torch.empty((max(tot["ne"], 1), 2), dtype=torch.int32).pin_memory()
    h_t = torch.empty((max(tot["nt"], 1), 3), dtype=torch.int32).pin_memory()

    def e2e():
        ctx.batch_set_volumes(occ=occ_host, dims=dims)
        out = ctx.batch_run(args.t, euler=False)
        s = ctx.rem_sizes
        ctx.remaining_arrays_into(h_v[: s["nv"]], h_e[: s["ne"]], h_t[: s["nt"]])
        return out

    e2e()
    _, e_ms = timed(e2e, args.steps)
    s = ctx.rem_sizes
    fp64 = ctx.lambda_fp64_check()  # the batch's complex, outside the timed regions
    b_mean, l_mean, e_mean = statistics.mean(b_ms), statistics.mean(l_ms), statistics.mean(e_ms)
    return {
        "workload": f"csg{BATCH_N}_loguniform_{BATCH_LO}_{BATCH_HI}",
        "volumes": BATCH_N, "voxels": all_voxels,
        "value": all_voxels / (b_total / args.steps / 1e3), "unit": UNIT,
        "volumes_per_s": BATCH_N / (b_total / args.steps / 1e3),
        "ranks": world, "rank0_volumes": nmine, "rank0_voxels": nvox,
        "ms_per_batch": b_mean,
        "latency_ms": {"p50": float(np.percentile(b_ms, 50)), "p99": float(np.percentile(b_ms, 99))},
        "plain_loop": {"value": nvox / (l_mean / 1e3), "volumes_per_s": BATCH_N / (l_mean / 1e3),
                       "ms_per_pass": l_mean, "gpu_launches_per_pass": l_launches},
        "speedup_vs_plain_loop": l_mean / b_mean,
        "gpu_launches_per_batch": b_launches,
        "e2e": {"value": nvox / (e_mean / 1e3), "unit": UNIT, "h2d_bytes_per_step": nvox,
                "d2h_bytes_per_step": s["nv"] * 12 + s["ne"] * 8 + s["nt"] * 12, "ms_per_step": e_mean},
        "parity": f"{same}/{nmine} volumes: batched remaining arrays (sha256) equal the plain path's",
        "tuned": tuned,
        "fp64_check": fp64,
        "thin_generations": ctx.batch_stats["generations"],
        "cells": {"V": ctx.vd_sizes["nv"], "E": ctx.vd_sizes["ne"], "T": ctx.vd_sizes["nt"]},
    }


# ---------------------------------------------------------------------------
# Request stream: Poisson arrivals at 200 req/s of volumes drawn from the
# torus, spheres and GRF generators with edges log-uniform in [32, 384],
# served by the continuous-batching request loop (vc_server_*) under a
# 120 GB memory cap, against one plain context serving the same arrivals
# first come first served (vc_run_plain per request).

SERVE_RATE, SERVE_SECONDS, SERVE_POOL, SERVE_CAP = 200.0, 6.0, 18, 120 << 30
SERVE_WORKERS, SERVE_MAX_BATCH = 3, 8
SERVE_SWEEP, SERVE_SWEEP_SECONDS = (200.0, 400.0, 800.0, 1600.0), 2.0


def serve_pool(dev):
    from voxel_ma_gb300 import volumes
    rng = np.random.default_rng(2024)
    pool = []
    for i in range(SERVE_POOL):
        n = int(np.clip(np.exp(rng.uniform(np.log(32), np.log(384))), 32, 384))
        kind = i % 3
        if kind == 0:
            occ = volumes.torus_mesh(n)
        elif kind == 1:
            occ = volumes.spheres(n, count=32, seed=i)
        else:
            occ = volumes.grf(n, sigma=6.0, seed=i, device=dev)
        pool.append(np.ascontiguousarray(occ))
    return pool


def _arrivals(rate: float, seconds: float, npool: int, seed: int):
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate, size=int(rate * seconds * 1.5) + 16)
    arrivals = np.cumsum(gaps)
    arrivals = arrivals[arrivals < seconds]
    return arrivals, rng.integers(0, npool, size=len(arrivals))


def _serve_server(srv, pool, t, arrivals, picks, keep_digests=False):
    ids = []
    t0 = time.perf_counter()
    for a, k in zip(arrivals, picks):
        d = t0 + a - time.perf_counter()
        if d > 0:
            time.sleep(d)
        ids.append(srv.submit(pool[k], t))
    res = [srv.wait(i) for i in ids]
    span = time.perf_counter() - t0
    digests = [_rem_digest(*srv.remaining(i, r)) for i, r in zip(ids, res)] if keep_digests else None
    for i in ids:
        srv.release(i)
    return np.array([r["latency_ms"] for r in res]), span, digests


def _serve_plain(ctx, pool, t, arrivals, picks, keep_digests=False):
    lat, digests = [], []
    t0 = time.perf_counter()
    for a, k in zip(arrivals, picks):
        d = t0 + a - time.perf_counter()
        if d > 0:
            time.sleep(d)
        ctx.run_plain(pool[k], t)
        arr = ctx.remaining_arrays()
        lat.append((time.perf_counter() - (t0 + a)) * 1e3)
        if keep_digests:
            digests.append(_rem_digest(*arr))
    return np.array(lat), time.perf_counter() - t0, (digests if keep_digests else None)


def _summary(lat, span, n):
    return {"throughput_req_s": n / span, "latency_ms": {"p50": float(np.percentile(lat, 50)),
                                                         "p99": float(np.percentile(lat, 99))}}


def run_serving(dev, args, workers=None, max_batch=None, with_plain=True, sweep=True):
    """Poisson arrivals at SERVE_RATE req/s for SERVE_SECONDS, served by the
    request loop and by one plain context first come first served (same
    arrivals, same volumes); then a sweep of offered rates (SERVE_SWEEP, a
    shorter window each) to the knee of both: the highest offered rate each
    keeps up with, and its p99 there."""
    from voxel_ma_gb300 import api
    pool = serve_pool(dev)
    arrivals, picks = _arrivals(SERVE_RATE, SERVE_SECONDS, len(pool), 7)
    voxels = np.array([pool[k].size for k in picks], np.int64)
    workers = workers or SERVE_WORKERS
    max_batch = max_batch or SERVE_MAX_BATCH
    srv = api.Server(dev.index or 0, workers=workers, mem_cap_bytes=SERVE_CAP, max_batch=max_batch)
    warm = [srv.submit(pool[k], args.t) for k in range(len(pool))]
    for i in warm:
        srv.wait(i)
        srv.release(i)
    b0 = srv.stats()["batches"]
    lat, span, dig_srv = _serve_server(srv, pool, args.t, arrivals, picks, keep_digests=with_plain)
    st = srv.stats()
    n = len(arrivals)
    # the digests of the server's results are taken after its timed run; the
    # plain results they are compared with come from one plain run per pool
    # volume (a volume's result does not depend on when it runs)
    if not with_plain:
        srv.close()
        out = {"workers": workers, "max_batch": max_batch, "batches": st["batches"] - b0}
        out.update(_summary(lat, span, n))
        return out
    ctx = api.Context(dev.index or 0)
    pool_digest = []
    for k in range(len(pool)):
        ctx.run_plain(pool[k], args.t)
        pool_digest.append(_rem_digest(*ctx.remaining_arrays()))
    plat, pspan, _ = _serve_plain(ctx, pool, args.t, arrivals, picks)
    same = sum(1 for a, k in zip(dig_srv, picks) if a == pool_digest[k])
    out = {
        "workload": f"poisson{int(SERVE_RATE)}_torus_spheres_grf_edge32_384",
        "arrival_rate_req_s": SERVE_RATE, "requests": n, "duration_s": SERVE_SECONDS,
        "pool": f"{SERVE_POOL} volumes (torus mesh, 32 spheres, GRF sigma 6), edge log-uniform in [32, 384]",
        "mem_cap_bytes": SERVE_CAP, "workers": workers, "max_batch": max_batch,
        "value": float(voxels.sum() / span), "unit": UNIT,
        "batches": st["batches"] - b0,
        "device_bytes_end": st["device_bytes"],
        "plain": {"value": float(voxels.sum() / pspan)},
        "parity": f"{same}/{n} requests: remaining arrays (sha256) equal the plain path's",
    }
    out.update(_summary(lat, span, n))
    out["plain"].update(_summary(plat, pspan, n))
    if sweep:
        rows = []
        for rate in SERVE_SWEEP:
            arr, pk = _arrivals(rate, SERVE_SWEEP_SECONDS, len(pool), 11)
            sl, ss, _ = _serve_server(srv, pool, args.t, arr, pk)
            pl, ps, _ = _serve_plain(ctx, pool, args.t, arr, pk)
            rows.append({"offered_req_s": rate, "requests": len(arr),
                         "server": _summary(sl, ss, len(arr)), "plain": _summary(pl, ps, len(arr))})

        def knee(side):
            # the highest offered rate served at >= 95 % of the offer
            ok = [r for r in rows if r[side]["throughput_req_s"] >= 0.95 * r["offered_req_s"]]
            best = max(ok, key=lambda r: r["offered_req_s"]) if ok else None
            return {"offered_req_s": best["offered_req_s"], "p99_ms": best[side]["latency_ms"]["p99"]} if best \
                else None
        out["sweep"] = {"window_s": SERVE_SWEEP_SECONDS, "rows": rows,
                        "knee": {"server": knee("server"), "plain": knee("plain")},
                        "max_throughput_req_s": {"server": max(r["server"]["throughput_req_s"] for r in rows),
                                                 "plain": max(r["plain"]["throughput_req_s"] for r in rows)}}
    ctx.close()
    srv.close()
    return out


# DRAM traffic per cell of the complex (V + E + T) of the thinning kernel,
# from one ncu capture of the 192^3 case of this workload (3.928 GB read +
# 1.838 GB written for 3,286,553 + 13,677,962 + 10,430,150 cells); the
# traffic grows with the complex, so the per-launch figure at 512^3 is this
# rate times its cells.
TRAFFIC_PER_CELL = {"thin_generations": (3.928310e9 + 1.838015e9) / (3286553 + 13677962 + 10430150)}
# L2 requests (atomics + reductions + reads + writes from the SMs) per cell of
# the same capture: 46.64 M + 15.86 M + 39.05 M + 22.97 M for the same cells.
L2_REQUESTS_PER_CELL = {"thin_generations": (46640018 + 15863455 + 39046856 + 22965656)
                        / (3286553 + 13677962 + 10430150)}
PROBE_BYTES = 16 << 30


# ---------------------------------------------------------------------------
# How the CPU path's voxels/s changes with the volume's size: single-threaded
# oracle runs at 128^3, 256^3 and 512^3 in a child process that runs beside
# the GPU measurements (one host core; its results are read at the end).

CPU_SCALING_SIZES = (128, 256, 512)
CPU_SCALING_WAIT_S = 480.0  # from the child's start; sizes not done by then are reported unfinished


def run_grf1024(dev, args):
    """Configuration 3 at 1024^3: the plain path on the 1024^3 field (same
    generator, sigma 6, seed 0; 1.07e9 voxels, a complex of about 4.2e9
    cells), in a context of its own once every other leg has closed its
    contexts.  Device-resident steps and end-to-end steps (host volume in,
    remaining complex out) as in the headline; the site list and feature
    transform of this volume are pinned to the oracle's digests and the rest
    of the path by its properties in the GPU tests."""
    import torch

    from voxel_ma_gb300 import api, volumes

    t0 = time.perf_counter()
    occ_np = volumes.grf(1024, sigma=6.0, seed=0, device=dev)
    gen_s = time.perf_counter() - t0
    torch.cuda.empty_cache()  # the blur's temporaries
    occ_dev = torch.from_numpy(occ_np).to(dev)
    occ_host = torch.from_numpy(occ_np).pin_memory()
    nvox = int(occ_np.size)
    steps = max(1, min(args.steps, 3))
    out = {"workload": "grf1024_sigma6_level0", "shape": list(occ_np.shape),
           "occupancy_sha256": volumes.occupancy_sha256(occ_np), "generate_s": gen_s}
    del occ_np
    with api.Context(dev.index if dev.index is not None else 0) as ctx:
        stream = ctx.torch_stream()
        r = ctx.run_plain(occ_dev, args.t)  # allocations
        r = ctx.run_plain(occ_dev, args.t)
        torch.cuda.synchronize(dev)
        ctx.sync()
        ctx.set_timing(True)
        ctx.reset_timings()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            r = ctx.run_plain(occ_dev, args.t)
        e1.record(stream)
        torch.cuda.synchronize(dev)
        ctx.sync()
        ms = e0.elapsed_time(e1) / steps
        timings = ctx.timings()
        ctx.set_timing(False)
        rem = r["rem"]
        h_v = torch.empty((max(rem["nv"], 1), 3), dtype=torch.float32).pin_memory()
        h_e = torch.empty((max(rem["ne"], 1), 2), dtype=torch.int32).pin_memory()
        h_t = torch.empty((max(rem["nt"], 1), 3), dtype=torch.int32).pin_memory()
        e0.record(stream)
        for _ in range(steps):
            rr = ctx.run_plain(occ_host, args.t)
            q = rr["rem"]
            ctx.remaining_arrays_into(h_v[: q["nv"]], h_e[: q["ne"]], h_t[: q["nt"]])
        e1.record(stream)
        torch.cuda.synchronize(dev)
        e2e_ms = e0.elapsed_time(e1) / steps
        eu = ctx.euler_remaining()
        vd = r["vd"]
        out.update({
            "value": nvox / (ms / 1e3), "unit": UNIT, "ms_per_step": ms, "steps": steps,
            "e2e": {"value": nvox / (e2e_ms / 1e3), "unit": UNIT, "ms_per_step": e2e_ms,
                    "h2d_bytes_per_step": nvox, "d2h_bytes_per_step": q["nv"] * 12 + q["ne"] * 8 + q["nt"] * 12},
            "complex": {"sites": r["n_sites"], "V": vd["nv"], "E": vd["ne"], "T": vd["nt"], "thresh": r["thresh"],
                        "generations": r["thin"]["generations"], "pushes": r["thin"]["pushes"],
                        "processed": r["thin"]["processed"], "remaining": rem},
            "euler_kept": eu["euler"] == vd["nv"] - vd["ne"] + vd["nt"],
            "same_as_previous_step": rr == r,
            "device_bytes": ctx.device_bytes(),
            "region_ms_per_step": {k: v[0] / max(v[1], 1) for k, v in sorted(timings.items())},
        })
    return out


def cpu_scaling_child(path: str, t: float) -> int:
    import oracle
    from voxel_ma_gb300 import volumes
    oracle.build(reference=False)
    for n in CPU_SCALING_SIZES:
        occ = volumes.grf(n, sigma=6.0, seed=0)
        t0 = time.perf_counter()
        r = oracle.run_plain(occ, t=t, threads=1)
        dt = time.perf_counter() - t0
        rec = {"edge": n, "voxels": int(occ.size), "seconds": dt, "voxels_per_s": occ.size / dt,
               "processed_pairs": int(r["thin"]["stats"]["processed"])}
        del r
        with open(path, "a") as f:
            f.write(json.dumps(rec) + "\n")
    return 0


class CpuScaling:
    """The child process running the scaling points (rank 0 only)."""

    def __init__(self, t: float):
        self.path = tempfile.NamedTemporaryFile("w", suffix=".jsonl", delete=False).name
        self.t0 = time.time()
        self.p = subprocess.Popen([sys.executable, os.path.abspath(__file__), "--cpu-scaling-child", self.path,
                                   "--t", str(t)], stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)

    def collect(self) -> dict:
        try:
            self.p.wait(timeout=max(1.0, CPU_SCALING_WAIT_S - (time.time() - self.t0)))
        except subprocess.TimeoutExpired:
            self.p.kill()
            self.p.wait()
        rows = [json.loads(x) for x in open(self.path) if x.strip()]
        os.unlink(self.path)
        done = {r["edge"] for r in rows}
        return {"kind": "port", "cores": 1, "workload": "GRF sigma=6 level 0, seed 0, same generator as the GPU "
                "workload", "points": rows,
                "unfinished": [n for n in CPU_SCALING_SIZES if n not in done],
                "note": "oracle restatement of the reference path, one thread, run beside the GPU measurements"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--workload", default="grf512")
    ap.add_argument("--t", type=float, default=0.04)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched-path measurement")
    ap.add_argument("--no-serve", action="store_true", help="skip the request-stream measurement")
    ap.add_argument("--no-tune", action="store_true", help="keep the library's default launch shapes")
    ap.add_argument("--no-probe", action="store_true",
                    help="skip the random-access probe and the topology and octree measurements")
    ap.add_argument("--ft-method", choices=["envelope", "window"], default=None,
                    help="with --no-tune: the feature transform's method for the plain path")
    ap.add_argument("--no-cpu-scaling", action="store_true", help="skip the CPU path's size-scaling points")
    ap.add_argument("--no-1024", action="store_true", help="skip the 1024^3 field")
    ap.add_argument("--cpu-scaling-child", default=None, help=argparse.SUPPRESS)
    args = ap.parse_args()
    if args.cpu_scaling_child:
        return cpu_scaling_child(args.cpu_scaling_child, args.t)
    if args.impl == "reference":
        return run_reference(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
