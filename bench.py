"""Benchmark of the Spiral answer path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gpu|reference]

Workload: the plain single-query answer against a 1 GiB database (n = 2,
p = 256, nu1 = 9, nu2 = 8: 2^17 records of 8 KiB, a 7 GiB CRT-NTT image
on the device), d = 2048, q = 268369921 * 249561089, t_exp = 8, t_gsw = 7,
t_conv = 4.  A step answers one query.  Synthetic seeded data: uniform u8
records, a seeded client (discrete Gaussian secret, sigma 6.4) and a query
for a seeded random record.  The database image (7 GiB: two 28-bit residues
per coefficient) is larger than L2,
so every step streams it from HBM.

Printed as one JSON line (rank 0):
  value   queries/s with the query already on the device (staged), timed with
          CUDA events over K back-to-back answers on the library's stream
  e2e     queries/s through sp_answer with host buffers (query H2D, response
          D2H inside the timed region), host wall clock
  roofline  first-dimension multiply: algorithmic bytes / CUDA-event launch
          time against the measured HBM copy bandwidth
  cpu_baseline  the CPU oracle (the reference's answer path restated in C,
          OpenMP on this host's cores) answering one full 1 GiB query, timed;
          its response is compared byte for byte with the GPU's
  parity  config2_bytes_equal (GPU response == CPU oracle response) and
          batched_bytes_equal (every response of the B = 32 and B = 64
          batches == the same query answered alone)
With --gpus N > 1 (torchrun), every rank answers its own queries against its
own replica of the database ("replicas only": the path does not shard here).
"""
from __future__ import annotations

import argparse
import faulthandler
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "gpu-pir_gb300"))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "1GiB DB single-query answers/s (Spiral PIR, GPU)"
UNIT = "queries/s"
WORKLOAD = {"workload": "spiral-answer-1gib", "db_plain_bytes": 1 << 30, "db_device_bytes": 7 << 30,
            "records": 1 << 17, "record_bytes": 8192, "n": 2, "p": 256, "nu1": 9, "nu2": 8,
            "d": 2048, "t_exp": 8, "t_gsw": 7, "t_conv": 4, "batch": 1,
            "l2": "database image (7 GiB) larger than L2 (129 MB); no flush needed"}
THROTTLE = {0x8: "hw_slowdown", 0x40: "hw_thermal_slowdown", 0x20: "sw_thermal_slowdown",
            0x4: "sw_power_cap", 0x80: "hw_power_brake_slowdown", 0x1: "gpu_idle",
            0x2: "applications_clocks_setting", 0x100: "display_clock_setting"}


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class _Nvml:
    """SM clock, maximum SM clock, power and clock-event reasons of one GPU,
    read through NVML (libnvidia-ml, the library nvidia-smi reads); read-only."""

    def __init__(self, index: int):
        import ctypes
        self.ct = ctypes
        lib = ctypes.CDLL("libnvidia-ml.so.1")
        if lib.nvmlInit_v2() != 0:
            raise OSError("nvmlInit failed")
        h = ctypes.c_void_p()
        if lib.nvmlDeviceGetHandleByIndex_v2(ctypes.c_uint(index), ctypes.byref(h)) != 0:
            raise OSError("no NVML device %d" % index)
        try:
            self.reasons_fn = lib.nvmlDeviceGetCurrentClocksEventReasons
        except AttributeError:
            self.reasons_fn = lib.nvmlDeviceGetCurrentClocksThrottleReasons
        self.lib, self.h = lib, h

    def sample(self):
        ct, lib, h = self.ct, self.lib, self.h
        sm, mx, mw, rs = ct.c_uint(), ct.c_uint(), ct.c_uint(), ct.c_ulonglong()
        if (lib.nvmlDeviceGetClockInfo(h, 1, ct.byref(sm)) or lib.nvmlDeviceGetMaxClockInfo(h, 1, ct.byref(mx))
                or self.reasons_fn(h, ct.byref(rs))):
            return None
        power = mw.value / 1e3 if lib.nvmlDeviceGetPowerUsage(h, ct.byref(mw)) == 0 else 0.0
        return float(sm.value), float(mx.value), power, int(rs.value)


def _nvml_index(local: int) -> int:
    """NVML numbers GPUs by PCI order and ignores CUDA_VISIBLE_DEVICES."""
    vis = os.environ.get("CUDA_VISIBLE_DEVICES", "").split(",")
    if local < len(vis) and vis[local].strip().isdigit():
        return int(vis[local])
    return local


class ClockSampler:
    """SM clocks, power and clock-event reasons sampled during the timed
    regions: NVML every 5 ms in a thread (nvidia-smi every 50 ms where NVML
    cannot be loaded).  Only samples inside a window() count."""

    def __init__(self, index: int):
        self.index = index
        self.samples = []      # (perf_counter, sm MHz, max sm MHz, W, reasons)
        self.windows = []
        self.proc = None
        self.thread = None
        self.source = None
        self.halt = threading.Event()

    def start(self):
        try:
            nv = _Nvml(_nvml_index(self.index))
            if nv.sample() is None:
                raise OSError("NVML query failed")
            self.source = "nvml, 5 ms"
            self.thread = threading.Thread(target=self._poll, args=(nv,), daemon=True)
        except (OSError, AttributeError):
            cmd = ["nvidia-smi", "-i", str(self.index),
                   "--query-gpu=clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active",
                   "--format=csv,noheader,nounits", "-lms", "50"]
            try:
                self.proc = subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            except OSError:
                return self
            self.source = "nvidia-smi, 50 ms"
            self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()
        t_end = time.perf_counter() + 3.0    # the first sample precedes the timed regions
        while not self.samples and time.perf_counter() < t_end and self.thread.is_alive():
            time.sleep(0.01)
        return self

    def _poll(self, nv):
        while not self.halt.is_set():
            s = nv.sample()
            if s:
                self.samples.append((time.perf_counter(),) + s)
            self.halt.wait(0.005)

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 4:
                try:
                    self.samples.append((time.perf_counter(), float(parts[0]), float(parts[1]), float(parts[2]),
                                         int(parts[3], 16)))
                except ValueError:
                    pass

    class _Window:
        def __init__(self, owner):
            self.owner = owner

        def __enter__(self):
            self.t0 = time.perf_counter()

        def __exit__(self, *a):
            self.owner.windows.append((self.t0, time.perf_counter()))

    def window(self):
        return ClockSampler._Window(self)

    def stop(self) -> None:
        self.halt.set()
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)

    def summary(self, windows) -> dict | None:
        """Median / minimum SM clock, power and reasons over the samples taken
        inside `windows` (a list of (begin, end) perf_counter pairs)."""
        inside = [s for s in list(self.samples) if any(a <= s[0] <= b for a, b in windows)]
        if not inside:
            return None
        sm = sorted(s[1] for s in inside)
        reasons = set()
        for s in inside:
            for bit, name in THROTTLE.items():
                if s[4] & bit and name != "gpu_idle":
                    reasons.add(name)
        return {"sm_mhz": sm[len(sm) // 2], "sm_min_mhz": sm[0], "sm_max_mhz": max(s[2] for s in inside),
                "power_w_max": max(s[3] for s in inside), "samples": len(inside),
                "timed_s": sum(b - a for a, b in windows), "source": self.source,
                "reasons": sorted(reasons)}


def measured_peaks(key: str = "hbm_gbs"):
    """Measured peak (HBM GB/s, or bf16 TFLOP/s burst) from MEASURED_PEAKS.json,
    else the fallback figures (6.8 TB/s, 1.9 PFLOP/s)."""
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        if key in d:
            return float(d[key]), "measured"
    return (6800.0 if key == "hbm_gbs" else 1900.0), "fallback"


def measured_traffic(algo_bytes: float):
    """DRAM bytes of one k_db_mul launch at the benchmark's size, scaled from
    the ncu capture of a smaller case (profiles/db_mul_traffic.json: its
    DRAM bytes over its algorithmic bytes; the multiply's traffic grows in
    proportion to the image it streams), or None without a capture."""
    path = os.path.join(ROOT, "profiles", "db_mul_traffic.json")
    if not os.path.exists(path):
        return None
    with open(path) as f:
        d = json.load(f)
    return float(d["traffic_over_algorithmic"]) * algo_bytes


def expansion_round_outputs(p, nu1: int, nu2: int) -> list:
    """Live outputs of every expansion round of one query, after the
    reference's pruning (gpu-pir/expansion.cuh:92-97)."""
    g, stop, max_bits = p.g(nu1, nu2), p.stop_round(nu2), p.t_gsw * nu2
    out = []
    for r in range(g):
        n = 0
        for i in range(2 << r):
            if r > stop and i & 1:
                continue
            if r == stop and i & 1 and i // 2 >= max_bits:
                continue
            n += 1
        out.append(n)
    return out


def expansion_outputs(p, nu1: int, nu2: int) -> int:
    """Expansion outputs computed per query."""
    return sum(expansion_round_outputs(p, nu1, nu2))


def expansion_kernel_outputs(p, nu1: int, nu2: int, B: int, sms: int = 152) -> dict:
    """Outputs of a B-query batch by the expansion kernel that computes them
    (the library's rule: a round with at least 2 x SMs outputs runs one CTA
    per output, or one per parent with at least 4 x SMs parents; fewer
    outputs run the split kernel, counted here with the one-per-output
    figure)."""
    out = {"k_expand_round<1>": 0, "k_expand_pair": 0}
    for r, n in enumerate(expansion_round_outputs(p, nu1, nu2)):
        paired = (2 << r) * B >= 2 * sms and (1 << r) * B >= 4 * sms
        out["k_expand_pair" if paired else "k_expand_round<1>"] += n * B
    return out


def int_roofline(p, sh, B: int, stages_ms: dict, sm_mhz: float | None) -> dict | None:
    """Issue-slot roofline of the NTT-bound stages of a B-query batch: warp
    instructions per fold, per expansion output and per converted polynomial
    from the ncu capture of a small batch (profiles/int_pipe.json) times the
    items of this batch, over the stage's CUDA-event time, against the SMs'
    issue ceiling (4 schedulers x 1 warp instruction per cycle per SM) at the
    SM clock sampled during the run; the ALU pipe (the busier integer pipe)
    against its own ceiling."""
    path = os.path.join(ROOT, "profiles", "int_pipe.json")
    if not os.path.exists(path) or not sm_mhz:
        return None
    with open(path) as f:
        k = json.load(f)["kernels"]
    sms = 152
    issue_peak = sms * 4 * sm_mhz * 1e6
    folds = B * p.T * ((1 << sh.nu2) - 1)
    polys = B * p.T * 2 * (1 << sh.nu2)
    outs = expansion_kernel_outputs(p, sh.nu1, sh.nu2, B, sms)
    if "k_expand_pair" not in k:     # counts captured before the paired kernel
        outs = {"k_expand_round<1>": sum(outs.values())}
    out = {"sm_mhz": sm_mhz, "issue_peak_warp_inst_per_s": issue_peak, "source": "profiles/int_pipe.json"}
    for stage, parts, ms in (("fold", (("k_fold_level<1>", folds), ("k_acc_to_raw", polys)), stages_ms["fold"]),
                             ("expand", tuple((name, n) for name, n in outs.items() if n), stages_ms["expand"])):
        inst = sum(k[name]["warp_inst_per_item"] * n for name, n in parts)
        alu = sum(k[name]["alu_inst_per_item"] * n for name, n in parts)
        alu_rate = k[parts[0][0]].get("alu_warp_inst_per_scheduler_cycle_peak") or 0.5
        achieved = inst / (ms / 1e3)
        out[stage] = {"items": {name: n for name, n in parts}, "warp_inst": inst, "ms": ms,
                      "achieved_warp_inst_per_s": achieved, "issue_frac": achieved / issue_peak,
                      "alu_pipe_frac": alu / (ms / 1e3) / (issue_peak * alu_rate)}
    return out


def make_workload(seed: int = 0, n_queries: int = 64):
    """The 1 GiB database, a seeded client with its public keys, and
    `n_queries` queries for distinct seeded records."""
    from spiralpir import client as C
    from spiralpir import params as P

    p, sh = P.PARAMS, P.SHAPE_1GIB
    cl = C.Client(p, seed=seed + 1)
    keys = cl.public_keys(sh.nu1, sh.nu2)
    recs = C.random_records(sh, p, seed=seed + 2)
    rng = np.random.default_rng(seed + 3)
    idx = [int(x) for x in rng.choice(sh.num_records, size=n_queries, replace=False)]
    queries = [cl.query(sh, i) for i in idx]
    return p, sh, cl, keys, recs, idx, queries


class CpuOracle:
    """The CPU oracle (the C restatement of the reference's answer path, with
    OpenMP over the host's cores) holding the 1 GiB database encoded into
    CRT-NTT form on the host (8 GiB of u32 planes; encoding is set-up, not
    timed)."""

    def __init__(self, p, sh, recs, keys, threads: int | None = None):
        import oracle as O

        self.O, self.p, self.sh, self.keys = O, p, sh, keys
        if threads:
            O.set_threads(threads)
        self.cores = O.num_threads()
        t0 = time.perf_counter()
        self.db = O.db_encode(recs, p.n, sh.nu1, sh.nu2, p.pt_bits)
        self.encode_s = time.perf_counter() - t0

    def answer(self, q) -> tuple[np.ndarray, float]:
        """Full answer of one query (expansion, conversion, the multiply over
        all 2^nu2 columns, all 2^nu2 - 1 folds per instance, packing);
        returns the response bytes and the seconds it took."""
        p, sh, k = self.p, self.sh, self.keys
        t0 = time.perf_counter()
        resp = self.O.answer(self.db, q, k.exp_left, k.exp_right, k.conv, k.pack, n=p.n, nu1=sh.nu1, nu2=sh.nu2,
                             pt_bits=p.pt_bits, q2_bits=p.q2_bits, t_left=p.t_exp_left, t_right=p.t_exp_right,
                             t_gsw=p.t_gsw, t_conv=p.t_conv)
        return resp, time.perf_counter() - t0

    def db_mul_s(self, nu1: int, nu2: int, reps: int = 1) -> float:
        """Seconds per query of the first-dimension multiply alone (the
        reference's CPU loop, gpu-pir/db_mul_test.cu:240-282: 128-bit
        accumulation then one reduction, restated in C) at shape (nu1, nu2)
        on seeded residues."""
        O, T = self.O, self.p.T
        rng = np.random.default_rng(nu1 * 100 + nu2)

        def residues(shape):
            out = np.empty(tuple(shape) + (2, 2048), dtype=np.uint32)
            out[..., 0, :] = rng.integers(0, O.Q1, size=tuple(shape) + (2048,), dtype=np.uint32)
            out[..., 1, :] = rng.integers(0, O.Q2, size=tuple(shape) + (2048,), dtype=np.uint32)
            return out

        db = self.db if (nu1, nu2) == (self.sh.nu1, self.sh.nu2) else residues((T, 1 << nu2, 1 << nu1))
        sel = residues((1 << nu1, 2))
        O.db_mul(db, sel, T, nu1, nu2)
        t0 = time.perf_counter()
        for _ in range(reps):
            O.db_mul(db, sel, T, nu1, nu2)
        return (time.perf_counter() - t0) / reps


def cpu_baseline(orc: CpuOracle, q, gpu_resp: np.ndarray) -> dict:
    """One full 1 GiB query answered by the CPU oracle on this host's cores,
    timed; its response bytes are compared with the GPU's response to the
    same query.  Also times the first-dimension multiply alone (the
    reference's CPU loop restated) at the 8 MiB, 64 MiB and 1 GiB shapes."""
    resp, secs = orc.answer(q)
    mul = {name: orc.db_mul_s(nu1, nu2, reps) * 1e3
           for name, nu1, nu2, reps in (("8MiB", 7, 3, 20), ("64MiB", 8, 5, 4), ("1GiB", 9, 8, 1))}
    return {"value": 1.0 / secs, "unit": UNIT, "cores": orc.cores, "kind": "port",
            "seconds_per_query": secs, "db_encode_s": orc.encode_s,
            "bytes_equal_to_gpu": bool(np.array_equal(resp, gpu_resp)),
            "db_mul_ms_per_query": mul,
            "sample": "one full 1 GiB query (all 256 columns of the multiply, all 255 folds per "
                      "instance) by the C oracle with OpenMP; the database encoded on the host "
                      "beforehand (not timed)"}


def init_ranks(timeout_s: float | None = None) -> None:
    """The gloo process group of a multi-replica run (one rank per GPU),
    with a bounded timeout: a rank that fails or exits before a collective
    makes the others' next collective raise after `timeout_s` (default
    $SPIRALPIR_PG_TIMEOUT_S or 600 s) instead of waiting forever."""
    import datetime

    import torch.distributed as dist
    if timeout_s is None:
        timeout_s = float(os.environ.get("SPIRALPIR_PG_TIMEOUT_S", "600"))
    dist.init_process_group("gloo", timeout=datetime.timedelta(seconds=timeout_s))


def max_over_ranks(values, world: int) -> list:
    """Element-wise maximum of per-rank figures over all ranks (one gloo
    all-reduce); the figures themselves when world == 1."""
    if world == 1:
        return [float(v) for v in values]
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(v) for v in values], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(x) for x in t.tolist()]


def run_reference(args, rank, world):
    """The reference arm: the CPU oracle (the reference's answer path restated
    in C, OpenMP over all host cores) answering full 1 GiB queries, one query
    per step, on rank 0 only."""
    if rank != 0:
        return
    p, sh, cl, keys, recs, idx, queries = make_workload(seed=0, n_queries=8)
    orc = CpuOracle(p, sh, recs, keys)
    resp, _ = orc.answer(queries[0])
    decoded = bool(np.array_equal(cl.decode(resp), recs[idx[0]]))
    for i in range(1, args.warmup):
        orc.answer(queries[i % len(queries)])
    ts = []
    t_all = time.perf_counter()
    for i in range(args.steps):
        ts.append(orc.answer(queries[i % len(queries)])[1])
    wall = time.perf_counter() - t_all
    per = sum(ts) / len(ts)
    line = {"metric": METRIC, "value": 1.0 / per, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": per * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u32 (exact modular)", "data": "synthetic", "config": WORKLOAD,
            "impl": "reference",
            "cpu_baseline": {"value": 1.0 / per, "unit": UNIT, "cores": orc.cores, "kind": "port",
                             "sample": "one full 1 GiB query per step (all 256 columns, all 255 folds per "
                                       "instance); the database encoded on the host before the first step"},
            "e2e": {"value": 1.0 / per, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "timed_wall_s": wall, "db_encode_s": orc.encode_s, "decoded_ok": decoded,
            "note": "The reference ships no runnable CPU answer path (its CUDA does not compile as shipped and "
                    "its Python model is thread-faithful and about 1.4 s per fold), so this arm runs the C "
                    "oracle that restates the reference's algorithms (kind: port)."}
    print(json.dumps(line), flush=True)


def stage_split(g, count: int, runs: int = 1) -> dict:
    """The library's stats over `runs` staged runs of `count` queries with
    its stage timing on (events between the stages), the ms_* fields per
    run; two runs before them capture the timed plan's graph, and the timing
    is off again afterwards (the timed headline runs without it)."""
    g.set_stage_timing(True)
    try:
        for _ in range(2):
            g.run_staged(count)
        g.stats_reset()
        for _ in range(runs):
            g.run_staged(count)
        st = g.stats()
    finally:
        g.set_stage_timing(False)
    return {k: (v / runs if k.startswith("ms_") else v) for k, v in st.items()}


def run_gpu(args, rank, world, local):
    from spiralpir.lib import SpiralGPU

    p, sh, cl, keys, recs, idx, queries = make_workload(seed=rank)
    batch = args.batch
    gpu = SpiralGPU(p, max_batch=max(batch, 1))
    gpu.set_client_keys(1, keys)
    t0 = time.perf_counter()
    gpu.load_db(1, recs, sh.nu1, sh.nu2)
    load_s = time.perf_counter() - t0
    progress("headline")
    # correctness of the measured configuration
    resp0 = gpu.answer(1, 1, queries[0])
    ok = bool(np.array_equal(cl.decode(resp0), recs[idx[0]]))
    if not ok:
        raise SystemExit("decoded record differs from the database record")
    barrier = None
    if world > 1:
        import torch.distributed as dist
        init_ranks()
        barrier = dist.barrier
    # clocks are sampled from before the warm-up; samples inside the timed
    # regions (the staged run, the multiply alone, the end-to-end loop) count
    clocks = ClockSampler(local).start()
    # warm-up (answers through the public API, then staged runs); answering
    # reuses the slots, so the queries are staged after it
    for i in range(args.warmup):
        gpu.answer(1, 1, queries[i % len(queries)])
    for s in range(batch):
        gpu.stage_query(s, 1, 1, queries[s % len(queries)])
    gpu.time_staged(batch, args.warmup)
    # device-resident timed region
    if barrier:
        barrier()
    gpu.stats_reset()
    with clocks.window():
        ms = gpu.time_staged(batch, args.steps)
    st = gpu.stats()
    launches_per_answer = st["launches"] / max(1, args.steps)
    # per-stage split: CUDA events between the stages of three more staged runs
    split = stage_split(gpu, batch, runs=3)
    # first-dimension multiply alone (roofline): CUDA events around its launches
    with clocks.window():
        mul_ms = gpu.time_db_mul(1, batch, max(args.steps, 5))
    # end to end through the public API (host buffers)
    lat = []
    resp_bytes = int(gpu.response_bytes)
    out = np.empty(resp_bytes, dtype=np.uint8)
    # host buffers in the C ABI's layout (uint64 CRT residues), as a caller
    # of sp_answer holds them
    q64 = [np.ascontiguousarray(q, dtype=np.uint64) for q in queries]
    with clocks.window():
        t_e2e = time.perf_counter()
        for i in range(args.steps):
            t1 = time.perf_counter()
            gpu.answer(1, 1, q64[i % len(q64)], out=out)
            lat.append(time.perf_counter() - t1)
        e2e_s = time.perf_counter() - t_e2e
    clk = clocks.summary(clocks.windows)
    if barrier:
        barrier()
    progress("batched")
    # batched answering (B queries per pipeline run), same database; every
    # batched response is compared byte for byte with the same query
    # answered alone and decoded
    batched = None
    batch_equal, batch_decoded = True, True
    if args.batched > 1:
        sizes = [args.batched, 2 * args.batched]
        alone = [gpu.answer(1, 1, queries[s % len(queries)]) for s in range(max(sizes))]
        gpu2 = SpiralGPU(p, max_batch=max(sizes))
        gpu2.set_client_keys(1, keys)
        gpu2.load_db(1, recs, sh.nu1, sh.nu2)
        batched = []
        for B in sizes:
            for s in range(B):
                gpu2.stage_query(s, 1, 1, queries[s % len(queries)])
            gpu2.time_staged(B, 2)
            with clocks.window():
                bms = gpu2.time_staged(B, max(2, args.steps // 4))
            bsplit = stage_split(gpu2, B)
            eq = dec = 0
            for s in range(B):
                rb = gpu2.fetch_response(s)
                eq += bool(np.array_equal(rb, alone[s]))
                dec += bool(np.array_equal(cl.decode(rb), recs[idx[s % len(idx)]]))
            batch_equal = batch_equal and eq == B
            batch_decoded = batch_decoded and dec == B
            entry = {"B": B, "queries_per_s": B / (bms / 1e3), "ms_per_batch": bms,
                     "distinct_queries": min(B, len(queries)), "bytes_equal_single": eq, "decoded_ok": dec,
                     "speedup_vs_single": (B / bms) / (batch / ms),
                     "db_mul_variant": 1 + int(np.argmax(bsplit["db_mul_by_variant"])),
                     "stages_ms": {k[3:]: bsplit[k] for k in
                                   ("ms_expand", "ms_convert", "ms_db_mul", "ms_fold", "ms_pack", "ms_total")}}
            # tensor-core multiply alone: exact fp16 digit products, 16 per
            # residue product (4 x 4 digits), 2 ciphertext rows, B queries
            gpu2.set_db_mul_variant(3)
            with clocks.window():
                tc_ms = gpu2.time_db_mul(1, B, 3)
            gpu2.set_db_mul_variant(0)
            flops = 2.0 * 16 * 2 * B * (sh.num_records * p.T * 2048 * 2)
            tpeak, tkind = measured_peaks("bf16_tflops")
            entry["roofline_tc"] = {"bound": "tensor", "kernel": "k_db_mul_tc (+ digit split, transpose)",
                                    "achieved": flops / (tc_ms / 1e3) / 1e12, "peak": tpeak, "unit": "TFLOP/s",
                                    "frac": flops / (tc_ms / 1e3) / 1e12 / tpeak, "peak_source": tkind,
                                    "flops_per_launch": flops, "launch_ms": tc_ms}
            entry["clocks"] = clocks.summary(clocks.windows[-2:])
            entry["roofline_int"] = int_roofline(p, sh, B, entry["stages_ms"],
                                                 (entry["clocks"] or clk or {}).get("sm_mhz"))
            # what 8x the single-query rate would need of the per-query stages
            sm = entry["stages_ms"]
            per_q = (ms / batch) / 8
            entry["gap_to_8x"] = {
                "target_ms_per_query": per_q, "measured_ms_per_query": bms / B,
                "expand_fold_ms_per_query": (sm["expand"] + sm["fold"]) / B,
                "expand_fold_budget_ms_per_query": per_q - (sm["db_mul"] + sm["pack"] + sm["convert"]) / B,
                "bound": "expansion and fold: length-2048 transforms at the issue fractions of roofline_int"}
            batched.append(entry)
        gpu2.close()
    other = None
    if world == 1 and not args.no_other:
        gpu.close()
        gpu = None
        n_win = len(clocks.windows)
        other = bench_other(p, cl, keys, recs, clocks, with_8gib=not args.skip_8gib)
        other["clocks"] = clocks.summary(clocks.windows[n_win:])
    clocks.stop()

    value = batch * 1e3 / ms * world
    # image: two 28-bit residues (7 bytes) per plaintext coefficient; selectors
    # (2 rows x 2 primes x u32 per row and slot) and outputs (2 rows x 2
    # primes x u32 per combo and slot) of each query
    algo_bytes = sh.num_records * p.T * 2048 * 7 + (sh.rows * 2048 * 16 + p.T * sh.cols * 4 * 2048 * 4) * batch
    peak, peak_kind = measured_peaks()
    achieved = algo_bytes / (mul_ms / 1e3) / 1e9
    traffic = measured_traffic(algo_bytes)
    lat_ms = sorted(x * 1e3 for x in lat)
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / batch, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u32 (exact modular)",
            "data": "synthetic (seeded records, client and query)", "config": WORKLOAD,
            "e2e": {"value": args.steps / e2e_s * world, "unit": UNIT, "h2d_bytes_per_step": 4 * 2048 * 8,
                    "d2h_bytes_per_step": resp_bytes,
                    "p50_ms": lat_ms[len(lat_ms) // 2], "p99_ms": lat_ms[min(len(lat_ms) - 1, int(0.99 * len(lat_ms)))]},
            "roofline": {"bound": "hbm", "kernel": "k_db_mul", "achieved": achieved, "peak": peak,
                         "unit": "GB/s", "frac": achieved / peak, "peak_source": peak_kind,
                         "algorithmic_bytes_per_launch": algo_bytes, "launch_ms": mul_ms,
                         "traffic": traffic},
            "stages_ms": {k[3:]: split[k] for k in
                          ("ms_expand", "ms_convert", "ms_db_mul", "ms_fold", "ms_pack", "ms_total")},
            "gpu_launches": int(st["launches"]), "launches_per_answer": launches_per_answer,
            "batched": batched, "clocks": clk, "db_load_s": load_s, "decoded_ok": ok}
    if other is not None:
        line["other_configs"] = other
    if gpu is not None:
        gpu.close()
    if rank == 0:
        progress("CPU oracle")
        orc = CpuOracle(p, sh, recs, keys)
        line["cpu_baseline"] = cpu_baseline(orc, queries[0], resp0)
        del orc
        line["parity"] = {"config2_bytes_equal": line["cpu_baseline"]["bytes_equal_to_gpu"],
                          "batched_bytes_equal": batch_equal if batched else None,
                          "batched_decoded_ok": batch_decoded if batched else None}
    if world > 1:
        # the slowest rank sets the whole job's time
        ms_max, e2e_max = max_over_ranks([ms, e2e_s], world)
        line["ms_per_step"] = ms_max / batch
        line["value"] = batch * 1e3 / ms_max * world
        line["e2e"]["value"] = args.steps / e2e_max * world
        import torch.distributed as dist
        dist.destroy_process_group()
    if rank == 0:
        print(json.dumps(line), flush=True)


def main():
    faulthandler.enable()     # a native crash prints the Python stack on stderr
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["gpu", "reference"], default="gpu")
    ap.add_argument("--batch", type=int, default=1, help="queries per step (1 = plain single-query path)")
    ap.add_argument("--batched", type=int, default=32, help="also measure a B-query batch (0 to skip)")
    ap.add_argument("--no-other", action="store_true", help="skip the uneven-batch, 8 GiB and serving workloads")
    ap.add_argument("--skip-8gib", action="store_true", help="the other workloads without the 8 GiB database")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    rank, world, local = dist_info()
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if world > 1:
        os.environ["CUDA_VISIBLE_DEVICES"] = str(local)
    run_gpu(args, rank, world, local)



# ------------------------------------------------- the other workloads
# Each returns a dict for the JSON line; bench_other() runs them after the
# headline measurement and records a failing one as {"error": ...} instead
# of losing the whole line.

def bench_uneven(p, cl, keys, recs1g, clocks) -> dict:
    """Uneven batches: B in {8, 32, 64} queries alternating between the
    1 GiB database (nu1 = 9, nu2 = 8) and a 64 MiB database (nu1 = 8,
    nu2 = 5), answered in one pipeline run (one multiply launch per
    database).  Every batched response is compared byte for byte with the
    same query answered alone, and decoded."""
    from spiralpir import client as C
    from spiralpir import params as P
    from spiralpir.lib import SpiralGPU

    shapes = {1: P.SHAPE_1GIB, 2: P.SHAPE_64MIB}
    recs = {1: recs1g, 2: C.random_records(P.SHAPE_64MIB, p, seed=201)}
    rng = np.random.default_rng(7)
    out = []
    with SpiralGPU(p, max_batch=64) as g:
        g.set_client_keys(1, keys)
        for db, sh in shapes.items():
            g.load_db(db, recs[db], sh.nu1, sh.nu2)
        for B in (8, 32, 64):
            reqs, idx = [], []
            for s in range(B):
                db = 1 + s % 2
                i = int(rng.integers(0, shapes[db].num_records))
                reqs.append((1, db, cl.query(shapes[db], i)))
                idx.append(i)
            # staged (device-resident) timing: slots grouped by database
            order = sorted(range(B), key=lambda s: reqs[s][1])
            for slot, s in enumerate(order):
                g.stage_query(slot, *reqs[s])
            g.time_staged(B, 2)
            with clocks.window():
                ms = g.time_staged(B, 5)
            st = stage_split(g, B)
            batch = g.answer_batch(reqs)
            alone = [g.answer(*r) for r in reqs]
            eq = sum(bool(np.array_equal(a, b)) for a, b in zip(batch, alone))
            dec = sum(bool(np.array_equal(cl.decode(r), recs[reqs[s][1]][idx[s]])) for s, r in enumerate(batch))
            out.append({"B": B, "mix": "1GiB:64MiB = 1:1", "ms_per_batch": ms, "queries_per_s": B / ms * 1e3,
                        "stages_ms": {k[3:]: st[k] for k in ("ms_expand", "ms_convert", "ms_db_mul", "ms_fold",
                                                            "ms_pack", "ms_total")},
                        "bytes_equal_single": eq, "decoded_ok": dec})
    return {"batches": out}


def bench_8gib(p, recs8, clocks) -> dict:
    """The 8 GiB database (nu1 = 9, nu2 = 11: 2^20 records, a 56 GiB packed
    image): one query per pipeline run and B = 16 in one run, the multiply's
    HBM fraction, and the multiply variants' time per query as B grows (the
    arithmetic-intensity crossover).  The B = 16 responses are compared with
    the same queries answered alone; all are decoded (decode failures at this
    depth come from the parameters' noise budget, not from the arithmetic,
    which is bit-exact)."""
    from spiralpir import client as C
    from spiralpir import params as P
    from spiralpir.lib import SpiralGPU

    sh = P.SHAPE_8GIB
    cl = C.Client(p, seed=301)
    keys = cl.public_keys(sh.nu1, sh.nu2)
    rng = np.random.default_rng(302)
    idx = [int(x) for x in rng.choice(sh.num_records, size=16, replace=False)]
    qs = [cl.query(sh, i) for i in idx]
    peak, _ = measured_peaks()
    with SpiralGPU(p, max_batch=16) as g:
        g.set_client_keys(1, keys)
        t1 = time.perf_counter()
        g.load_db(1, recs8, sh.nu1, sh.nu2)
        load_s = time.perf_counter() - t1
        alone = [g.answer(1, 1, q) for q in qs]
        g.stage_query(0, 1, 1, qs[0])
        g.time_staged(1, 1)
        with clocks.window():
            ms1 = g.time_staged(1, 3)
            mul = g.time_db_mul(1, 1, 3)
        img = sh.num_records * p.T * 2048 * 7
        abytes = img + sh.rows * 2048 * 16 + p.T * sh.cols * 4 * 2048 * 4
        for s in range(16):
            g.stage_query(s, 1, 1, qs[s])
        g.time_staged(16, 1)
        with clocks.window():
            ms16 = g.time_staged(16, 2)
        eq = sum(bool(np.array_equal(g.fetch_response(s), alone[s])) for s in range(16))
        dec = sum(bool(np.array_equal(cl.decode(alone[s]), recs8[idx[s]])) for s in range(16))
        macs_q = sh.num_records * p.T * 2048 * 2 * 2
        per_q_bytes = sh.rows * 2048 * 16 + p.T * sh.cols * 4 * 2048 * 4
        crossover = []
        for variant, bs in ((1, (1,)), (2, (2, 8, 16)), (3, (2, 4, 8, 16))):
            g.set_db_mul_variant(variant)
            for B in bs:
                ms = g.time_db_mul(1, B, 2)
                crossover.append({"variant": variant, "B": B, "ms": ms, "ms_per_query": ms / B,
                                  "gbs": (img + B * per_q_bytes) / ms / 1e6, "tmacs": B * macs_q / ms / 1e9})
        g.set_db_mul_variant(0)
    return {"t_exp": [p.t_exp_left, p.t_exp_right], "load_s": load_s, "single_ms": ms1, "single_qps": 1e3 / ms1,
            "db_mul_ms": mul, "db_mul_gbs": abytes / mul / 1e6, "db_mul_frac": abytes / mul / 1e6 / peak,
            "B16_ms": ms16, "B16_qps": 16e3 / ms16, "B16_bytes_equal_single": eq, "decoded_ok": dec,
            "queries": 16, "db_mul_crossover": crossover}


def bench_serving(p, recs_by_name, clocks, rates=(250.0, 500.0, 1000.0, 2000.0), n_req=400,
                  n_warm=300) -> dict:
    """Serving: the 64 MiB, 1 GiB and 8 GiB databases resident, 256 clients
    (32 distinct key sets) under an HBM budget that holds about 120 clients'
    keys, so registering each rate's 96 active clients evicts the least
    recently used.  Seeded Poisson arrivals with a uniform mix over the
    databases go (1) to the continuous-batching server (one server for all
    rates, after warm-up runs at the lowest and highest rate that let the
    autotuner see the batch classes) and (2) to the plain single-query loop (one sp_answer at a
    time); both report achieved queries/s and p50/p99 latency.  The server's
    responses are compared byte for byte with the single-query loop's (the
    same queries answered alone) and decoded."""
    from spiralpir import client as C
    from spiralpir import params as P
    from spiralpir.lib import SpiralGPU
    from spiralpir.serving import Server, poisson_load, single_query_loop

    names = list(recs_by_name)
    shapes = {"64MiB": P.SHAPE_64MIB, "1GiB": P.SHAPE_1GIB, "8GiB": P.SHAPE_8GIB}
    ids = {n: i + 1 for i, n in enumerate(names)}
    key_sets = [C.Client(p, seed=400 + k) for k in range(32)]
    keys = [cl.public_keys(9, 11) for cl in key_sets]
    key_bytes = sum(a.nbytes for a in (keys[0].exp_left, keys[0].exp_right, keys[0].conv, keys[0].pack))
    rng = np.random.default_rng(401)

    def workload(n):
        active = [int(x) for x in rng.choice(256, size=96, replace=False)]
        reqs, checks = [], []
        for _ in range(n):
            cid = active[int(rng.integers(0, len(active)))]
            name = names[int(rng.integers(0, len(names)))]
            i = int(rng.integers(0, shapes[name].num_records))
            reqs.append((cid, ids[name], key_sets[cid % 32].query(shapes[name], i)))
            checks.append((cid, name, i))
        return active, reqs, checks

    warm = [workload(n_warm // 2), workload(n_warm // 2)]
    runs = [workload(n_req) for _ in rates]

    def ctx(budget):
        g = SpiralGPU(p, max_batch=32, hbm_budget_bytes=budget)
        for n in names:
            g.load_db(ids[n], recs_by_name[n], shapes[n].nu1, shapes[n].nu2)
        for k in range(8):
            g.set_client_keys(k, keys[k])
        return g

    g = ctx(0)
    srv = Server(g, lanes=2)          # reserves both lanes' workspace
    used = g.hbm_used()
    srv.stop()
    g.close()
    budget = used + 120 * key_bytes
    g = ctx(budget)
    registered = 0

    def register(active):
        nonlocal registered
        for cid in active:            # registering evicts the least recently used clients
            g.set_client_keys(cid, keys[cid % 32])
            registered += 1

    served = []
    with Server(g, lanes=2) as srv:
        # warm-up at the lowest and the highest rate: the batch classes of
        # both are tuned before the measured runs
        for (active, reqs, _), rate in zip(warm, (min(rates), max(rates))):
            register(active)
            poisson_load(srv, reqs, rate_qps=rate, seed=1)
        for rate, (active, reqs, _) in zip(rates, runs):
            register(active)
            with clocks.window():
                served.append(poisson_load(srv, reqs, rate_qps=rate, seed=int(rate)))
        st = srv.stats()
    rows = []
    for rate, (active, reqs, checks), res in zip(rates, runs, served):
        register(active)
        with clocks.window():
            plain = single_query_loop(g, reqs, rate_qps=rate, seed=int(rate))
        out, alone = res.pop("responses"), plain.pop("responses")
        res["bytes_equal_single"] = sum(bool(np.array_equal(a, b)) for a, b in zip(out, alone))
        wrong = {}
        for r, (cid, name, i) in zip(out, checks):
            if not np.array_equal(key_sets[cid % 32].decode(r), recs_by_name[name][i]):
                wrong[name] = wrong.get(name, 0) + 1
        res["decode_failures_by_db"] = wrong
        rows.append({"batching": res, "single_query_loop": plain})
    g.close()
    return {"dbs": names, "clients": 256, "distinct_key_sets": 32, "hbm_budget_bytes": budget,
            "key_bytes_per_client": key_bytes, "client_registrations": registered, "lanes": 2, "max_batch": 32,
            "requests_per_rate": n_req, "warmup_requests": n_warm, "batches": st["batches"], "rates": rows}


def progress(msg: str) -> None:
    """A progress note on stderr (the JSON line goes to stdout)."""
    print(f"[bench {time.strftime('%H:%M:%S')}] {msg}", file=sys.stderr, flush=True)


def bench_other(p, cl, keys, recs1g, clocks, with_8gib: bool = True) -> dict:
    """Configs beyond the headline: uneven batches, the 8 GiB database and
    the serving loop (each guarded: an error is recorded, not raised)."""
    from spiralpir import client as C
    from spiralpir import params as P

    out = {}
    t0 = time.perf_counter()
    progress("uneven batches")
    try:
        out["uneven_batches"] = bench_uneven(p, cl, keys, recs1g, clocks)
    except Exception as e:  # noqa: BLE001 - recorded in the line
        out["uneven_batches"] = {"error": repr(e)}
    recs = {"64MiB": C.random_records(P.SHAPE_64MIB, p, seed=203), "1GiB": recs1g}
    if with_8gib:
        progress("8 GiB database")
        try:
            recs["8GiB"] = C.random_records(P.SHAPE_8GIB, p, seed=204)
            out["db_8gib"] = bench_8gib(p, recs["8GiB"], clocks)
        except Exception as e:  # noqa: BLE001
            out["db_8gib"] = {"error": repr(e)}
    progress("serving")
    try:
        out["serving"] = bench_serving(p, recs, clocks)
    except Exception as e:  # noqa: BLE001
        out["serving"] = {"error": repr(e)}
    out["seconds"] = time.perf_counter() - t0
    return out


if __name__ == "__main__":
    main()
