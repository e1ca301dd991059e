"""Benchmark of the quantized vector-sparse SDDMM / SpMM path on GB300.

Headline workload: SDDMM L8-R8, A and B 4096 x 64 int8, output mask 4096 x
4096 with V = 8 column vectors at sparsity 0.9 (uniform vector placement),
int32 output, signed lanes.  One step = one batched launch over `--batch`
independent instances (own A, B and output, shared mask), sized so the
step's data (about 470 MB) exceeds twice the 129 MB L2: no L2 flush is
needed between steps.  Extra lines of the same JSON object report the L4-R4
and L16-R8 SDDMM variants and the SpMM L8-R8 configuration (A 1024 x 1024,
V = 8, sparsity 0.9, B 1024 x 256).

`--impl reference` times the reference's CPU implementation of the path (the
host SDDMM routine) on the host cores instead.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

MMA_NAMES = {1: "int8mma", 2: "f16mma", 3: "tcgen05", 4: "dp4a"}
METRIC = "quantized SpMM/SDDMM TOP/s vs roofline; sparse-attn req/s + p50/p99 latency"
UNIT = "TOP/s"
SEQ, HEAD_DIM, VEC, SPARSITY = 4096, 64, 8, 0.9


def _peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": float(d["hbm_gbs"]), "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


class ClockSampler:
    """Samples SM clocks and throttle reasons with nvidia-smi during a region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.lines = []
        if self.proc is not None:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [ln for ln in out.splitlines() if ln.strip()]

    def summary(self) -> dict:
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in getattr(self, "lines", []):
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, val in zip(names, f[5:9]):
                if val.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# ----------------------------------------------------------------------------
# workload construction
# ----------------------------------------------------------------------------

def sddmm_operands(pa: int, pb: int, batch: int, seed: int = 42, V: int = VEC, sparsity: float = SPARSITY):
    """The headline SDDMM's mask (plain vector CSR) and `batch` instances of
    packed A and B, numpy only (no library is loaded)."""
    from magicube_gb300 import synth
    mask = synth.uniform_mask(SEQ // V, SEQ, V, sparsity, seed=seed)
    rng = np.random.default_rng(seed + 1)
    lhs = rng.integers(0, 256, size=(batch, SEQ * HEAD_DIM * pa // 8), dtype=np.uint8)
    rhs = rng.integers(0, 256, size=(batch, SEQ * HEAD_DIM * pb // 8), dtype=np.uint8)
    return mask, lhs, rhs


def sddmm_workload(pa: int, pb: int, batch: int, seed: int = 42, V: int = VEC, sparsity: float = SPARSITY):
    from magicube_gb300 import formats
    mask, lhs, rhs = sddmm_operands(pa, pb, batch, seed, V, sparsity)
    hm = formats.prepare_sddmm(mask, alignment=8)
    return mask, hm, lhs, rhs


SPMM_M = SPMM_K = 1024
SPMM_N = 256


def spmm_operands():
    """SpMM L8-R8 configuration: A 1024 x 1024 at V = 8, sparsity 0.9 (102
    uniformly placed vectors per vector-row), values uniform int8; one value
    set shared by the instances, numpy only."""
    from magicube_gb300 import synth
    mask = synth.uniform_mask(SPMM_M // VEC, SPMM_K, VEC, SPARSITY, seed=7)
    rng = np.random.default_rng(8)
    vals = rng.integers(0, 256, size=mask.nnz_vec * VEC, dtype=np.uint8)
    return mask, vals, rng


def measured_traffic_per_instance() -> float | None:
    """DRAM bytes per SDDMM instance from the committed ncu summary of the
    headline kernel (profiles/sddmm_k64_L8R8_4096x4096x64_V8.md)."""
    p = ROOT / "profiles" / "sddmm_k64_L8R8_4096x4096x64_V8.md"
    try:
        for line in p.read_text().splitlines():
            if line.startswith("traffic_bytes_per_instance:"):
                return float(line.split(":")[1])
    except OSError:
        pass
    return None


def sddmm_bytes(hm, pa: int, pb: int, batch: int, V: int = VEC) -> tuple[float, float]:
    """(algorithmic bytes per launch, ops per launch) of a batched SDDMM, on
    the true nonzero vectors (the padding slots of the aligned layout are
    not counted): A and B once per instance, one int32 per stored score, the
    mask's column indices, offset pairs and row order once."""
    nnz = hm.mask.nnz_vec
    per_inst = SEQ * HEAD_DIM * pa / 8 + SEQ * HEAD_DIM * pb / 8 + nnz * V * 4
    mask_bytes = nnz * 4 + hm.mask.m_vec * 2 * 4 + hm.mask.m_vec * 4
    ops = 2.0 * nnz * V * HEAD_DIM * batch
    return per_inst * batch + mask_bytes, ops


def time_cuda(fn, steps: int, warmup: int, stream) -> list[float]:
    import torch
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    for a, b in evs:
        a.record(stream)
        fn()
        b.record(stream)
    torch.cuda.synchronize()
    return [a.elapsed_time(b) for a, b in evs]


# ----------------------------------------------------------------------------
# CPU baseline (the oracle's restatement of the reference's host routine)
# ----------------------------------------------------------------------------

class HostSddmmMask:
    """The headline mask's aligned pairs and padded columns, built by the
    oracle's numpy aligner: the CPU legs load no library of this package."""

    def __init__(self, mask, alignment: int = 8):
        import oracle
        self.mask = mask
        self.pairs, self.aligned_nnz = oracle.align_pairs(mask.row_offsets, alignment)
        self.cols = oracle.pad_columns(mask.row_offsets, mask.col_indices, self.pairs, self.aligned_nnz)


def cpu_sddmm(hmask: HostSddmmMask, lhs: np.ndarray, rhs: np.ndarray, instances: list[int], rows: int,
              threads: int) -> tuple[float, float]:
    """Time the host SDDMM routine (the oracle's restatement of
    Host_sddmm_integers, SDDMM/SDDMM/sddmm_benchmark.cpp:24-60, signed lanes)
    over the first `rows` vector-rows of each listed instance.  Instances are
    dealt to `threads` workers; a single instance is split by vector-rows.
    Each worker writes its own output buffer.  Returns (seconds, ops)."""
    import oracle
    L = oracle.lib()
    m = hmask.mask
    pairs, cols = hmask.pairs, hmask.cols
    if len(instances) >= threads:
        items = [[(i, 0, rows) for i in instances[w::threads]] for w in range(threads)]
    else:
        bounds = [int(x) for x in np.linspace(0, rows, threads + 1)]
        items = [[(instances[0], bounds[w], bounds[w + 1])] for w in range(threads)]
    outs = [np.zeros(hmask.aligned_nnz * VEC, dtype=np.int32) for _ in range(threads)]

    def work(w: int) -> None:
        for inst, lo, hi in items[w]:
            if hi <= lo:
                continue
            L.mco_sddmm_host(int(lhs[inst].ctypes.data) + lo * VEC * HEAD_DIM, int(rhs[inst].ctypes.data),
                             int(outs[w].ctypes.data), hi - lo, VEC, HEAD_DIM, SEQ, 8, 8,
                             int(pairs.ctypes.data) + lo * 2 * 4, int(cols.ctypes.data), 8, 0, oracle.SIGNED)

    t0 = time.perf_counter()
    with ThreadPoolExecutor(max_workers=threads) as ex:
        for f in [ex.submit(work, w) for w in range(threads)]:
            f.result()  # re-raises a worker's exception
    dt = time.perf_counter() - t0
    nnz = 0
    for w in range(threads):
        for _, lo, hi in items[w]:
            nnz += int(m.row_offsets[hi] - m.row_offsets[lo])
    return dt, 2.0 * nnz * VEC * HEAD_DIM


def cpu_spmm(mask, vals: np.ndarray, rhs: np.ndarray, threads: int) -> tuple[float, float]:
    """Time the host SpMM routine (the oracle's restatement of
    compute_ref_integers, SpMM/SpMM/spmm_benchmark.cpp:69-120, signed lanes)
    on `threads` full instances of the SpMM L8-R8 configuration at once, one
    per worker (rhs[w] is instance w's B).  Returns (seconds, ops)."""
    import oracle
    L = oracle.lib()
    ro = np.ascontiguousarray(mask.row_offsets, dtype=np.int32)
    ci = np.ascontiguousarray(mask.col_indices, dtype=np.int32)
    outs = [np.empty((SPMM_M, SPMM_N), dtype=np.int32) for _ in range(threads)]

    def work(w: int) -> None:
        L.mco_spmm_host(int(vals.ctypes.data), int(rhs[w].ctypes.data), int(outs[w].ctypes.data), mask.m_vec, VEC,
                        SPMM_K, SPMM_N, 8, 8, 8, int(ro.ctypes.data), int(ci.ctypes.data), oracle.SIGNED)

    t0 = time.perf_counter()
    with ThreadPoolExecutor(max_workers=threads) as ex:
        for f in [ex.submit(work, w) for w in range(threads)]:
            f.result()
    dt = time.perf_counter() - t0
    return dt, 2.0 * mask.nnz_vec * VEC * SPMM_N * threads


def _repeat_for(fn, budget_s: float, cap: int = 50) -> tuple[float, float, int]:
    """Run fn() -> (seconds, ops) about `budget_s` seconds; totals and count."""
    dt, ops = fn()
    tot_t, tot_ops, n = dt, ops, 1
    while tot_t < budget_s and n < cap:
        dt, ops = fn()
        tot_t, tot_ops, n = tot_t + dt, tot_ops + ops, n + 1
    return tot_t, tot_ops, n


def cpu_baseline(budget_s: float = 12.0) -> dict:
    """The reference's CPU implementation of the path on one host core: the
    host SDDMM routine on the headline workload (a bounded sample of its
    vector-rows) and, beside it, the host SpMM routine on the SpMM L8-R8
    configuration (whole instances)."""
    mask, lhs, rhs = sddmm_operands(8, 8, 1)
    hmask = HostSddmmMask(mask)
    rows = 64
    t, ops, n = _repeat_for(lambda: cpu_sddmm(hmask, lhs, rhs, [0], rows, 1), budget_s)
    smask, vals, rng = spmm_operands()
    srhs = rng.integers(0, 256, size=(1, SPMM_K * SPMM_N), dtype=np.uint8)
    st, sops, sn = _repeat_for(lambda: cpu_spmm(smask, vals, srhs, 1), budget_s / 3)
    return {"value": ops / t / 1e12, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": f"host SDDMM L8-R8 routine (oracle restatement of Host_sddmm_integers), {rows} of "
                      f"{SEQ // VEC} vector-rows of one 4096x4096x64 V=8 s=0.9 instance, single thread, "
                      f"{n} repetitions",
            "spmm": {"value": sops / st / 1e12, "unit": UNIT, "cores": 1, "kind": "port",
                     "sample": "host SpMM L8-R8 routine (oracle restatement of compute_ref_integers), one full "
                               f"1024x1024x256 V=8 s=0.9 instance per repetition, {sn} repetitions, single thread",
                     "ms_per_instance": st / sn * 1e3}}


def run_reference(args) -> None:
    """The reference arm: the reference's CPU implementation of the path (the
    host SDDMM routine, restated by the oracle) on the headline workload, all
    host cores.  Each step is the GPU arm's whole step (`--batch` instances,
    each with its own A and B), the instances dealt to the threads.  The host
    SpMM routine on the SpMM L8-R8 configuration is reported beside it.  No
    library of this package is loaded."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import oracle
    oracle.build()
    threads = os.cpu_count() or 1
    B = args.batch
    mask, lhs, rhs = sddmm_operands(8, 8, B)
    hmask = HostSddmmMask(mask)
    rows = SEQ // VEC
    inst = list(range(B))
    for _ in range(args.warmup):
        cpu_sddmm(hmask, lhs, rhs, inst[:threads], rows, threads)
    t, ops = 0.0, 0.0
    for _ in range(args.steps):
        dt, o = cpu_sddmm(hmask, lhs, rhs, inst, rows, threads)
        t += dt
        ops += o
    v = ops / t / 1e12
    smask, vals, rng = spmm_operands()
    srhs = rng.integers(0, 256, size=(threads, SPMM_K * SPMM_N), dtype=np.uint8)
    st, sops, sn = _repeat_for(lambda: cpu_spmm(smask, vals, srhs, threads), 5.0, cap=10)
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "int8", "data": "synthetic",
        "config": headline_config(B, args.gpus),
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"every step the whole headline step: {B} full 4096x4096x64 V=8 s=0.9 SDDMM "
                                   "instances (own A and B each), host routine (oracle restatement of "
                                   f"Host_sddmm_integers), instances dealt to {threads} threads"},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "spmm": {"value": sops / st / 1e12, "unit": UNIT, "cores": threads, "kind": "port",
                 "sample": f"host SpMM L8-R8 routine (oracle restatement of compute_ref_integers), {threads} full "
                           f"1024x1024x256 V=8 s=0.9 instances at once (one per thread), {sn} repetitions"},
    }))


def headline_config(batch: int, world: int) -> dict:
    return {"workload": "SDDMM L8-R8: A,B 4096x64 int8, mask 4096x4096 V=8 sparsity 0.9 uniform, "
                        "int32 out, signed lanes",
            "instances_per_step": batch,
            "l2": "inputs+outputs per step exceed 2x L2 (no flush)", "parallelism": f"replicas x{world}"}


# ----------------------------------------------------------------------------
# GPU arm
# ----------------------------------------------------------------------------

def run_gpu(args) -> None:
    import torch

    from magicube_gb300 import ops
    from magicube_gb300.replicas import Replicas

    reps = Replicas("nccl")
    world, rank, local = reps.world, reps.rank, reps.local
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    stream = torch.cuda.current_stream()
    peaks = _peaks()

    def sync_all():
        torch.cuda.synchronize()
        reps.barrier()

    def max_over_ranks(x: float) -> float:
        return reps.max(x, dev)

    B = args.batch
    results = {}
    launches_per_step = 1

    def sddmm_case(pa, pb, timed_region_clock=False, mma=args.mma, variant=0, V=VEC, sparsity=SPARSITY):
        mask, hm, lhs_h, rhs_h = sddmm_workload(pa, pb, B, V=V, sparsity=sparsity)
        dm = ops.DeviceSddmmMask.from_host(hm, dev)
        lhs = torch.from_numpy(lhs_h).to(dev)
        rhs = torch.from_numpy(rhs_h).to(dev)
        out = torch.empty((B, hm.aligned_nnz * V), dtype=torch.int32, device=dev)
        fn = lambda: ops.sddmm(dm, lhs, rhs, HEAD_DIM, pa, pb, signed=True, out=out, batch=B, mma_kind=mma,
                                    variant=variant)
        sync_all()
        if timed_region_clock:
            with ClockSampler(local) as cs:
                ms = time_cuda(fn, args.steps, args.warmup, stream)
            clocks = cs.summary()
        else:
            ms, clocks = time_cuda(fn, args.steps, args.warmup, stream), None
        sync_all()
        byts, opc = sddmm_bytes(hm, pa, pb, B, V)
        t = max_over_ranks(sum(ms) / 1e3)
        avg = t / args.steps
        return {"tops": opc * world * args.steps / t / 1e12, "ms": avg * 1e3, "gbs": byts / avg / 1e9,
                "bytes": byts, "ops": opc, "clocks": clocks, "mask": hm, "dm": dm, "lhs_h": lhs_h, "rhs_h": rhs_h,
                "out": out, "lhs": lhs, "rhs": rhs}

    def verify_sddmm(r, pa, pb, V, instances) -> bool:
        """Untimed check of finished outputs against the oracle (bit for bit),
        with the aligned layout rebuilt by the oracle's own aligner."""
        import oracle
        hm = r["mask"]
        pairs, n_al = oracle.align_pairs(hm.mask.row_offsets, 8)
        if n_al != hm.aligned_nnz or not np.array_equal(pairs, hm.row_offsets):
            return False
        for i in instances:
            ref = oracle.sddmm_host(r["lhs_h"][i], r["rhs_h"][i], pairs, hm.col_indices, hm.mask.m_vec, V, HEAD_DIM,
                                    SEQ, pa, pb, oracle.SIGNED)
            if not np.array_equal(r["out"][i].cpu().numpy(), ref):
                return False
        return True

    head = sddmm_case(8, 8, timed_region_clock=True)
    verified = verify_sddmm(head, 8, 8, VEC, [0, B - 1])

    # e2e through the C ABI with host buffers: H2D of the step's operands, the
    # launch, D2H of the step's outputs, all inside the timed region.
    lhs_pin = torch.from_numpy(head["lhs_h"]).pin_memory()
    rhs_pin = torch.from_numpy(head["rhs_h"]).pin_memory()
    out_pin = torch.empty(head["out"].shape, dtype=torch.int32).pin_memory()
    dm = head["dm"]

    def e2e_step():
        head["lhs"].copy_(lhs_pin, non_blocking=True)
        head["rhs"].copy_(rhs_pin, non_blocking=True)
        ops.sddmm(dm, head["lhs"], head["rhs"], HEAD_DIM, 8, 8, signed=True, out=head["out"], batch=B,
                  mma_kind=args.mma)
        out_pin.copy_(head["out"], non_blocking=True)

    e2e_steps = max(3, args.steps // 4)
    sync_all()
    ms_e2e = time_cuda(e2e_step, e2e_steps, max(args.warmup, 3), stream)
    sync_all()
    t_e2e = max_over_ranks(sum(ms_e2e) / 1e3)
    e2e = {"value": head["ops"] * world * e2e_steps / t_e2e / 1e12, "unit": UNIT,
           "h2d_bytes_per_step": int(lhs_pin.numel() + rhs_pin.numel()),
           "d2h_bytes_per_step": int(out_pin.numel() * 4)}
    del lhs_pin, rhs_pin, out_pin

    variants = {}
    if not args.headline_only:
        # the other tensor paths of the headline SDDMM; the other precision
        # pairs and the SpMM run on mma.sync (int8 unless --mma f16)
        others = [m for m in (1, 2, 3, 4) if m != args.mma]
        sync_mma = 2 if args.mma == 2 else 1
        cases = [(4, 4, "sddmm_L4R4", sync_mma, 0, VEC), (16, 8, "sddmm_L16R8", 0, 0, VEC),
                 (16, 8, "sddmm_L16R8_int8mma", 1, 0, VEC)]
        cases += [(8, 8, f"sddmm_L8R8_{MMA_NAMES[m]}", m, 0, VEC) for m in others]
        cases += [(8, 8, "sddmm_L8R8_per_row_kernel", sync_mma, 1, VEC)]
        # V = 2 and 4: the int8 MMA computes 8 lanes of which V are used; dp4a
        # computes only the V lanes
        cases += [(8, 8, f"sddmm_L8R8_V{v}_{MMA_NAMES[m]}", m, 0, v) for v in (2, 4) for m in (1, 4)]
        cases += [(4, 4, f"sddmm_L4R4_V{v}_{MMA_NAMES[m]}", m, 0, v) for v in (2, 4) for m in (1, 4)]
        cases += [(4, 4, "sddmm_L4R4_dp4a", 4, 0, VEC)]
        cases = [c + (SPARSITY,) for c in cases]
        # every score of 128 x 256 tiles on the tcgen05 f16 tensor cores with a
        # masked epilogue, against the per-nonzero int8 kernel across sparsity
        for sp in (0.5, 0.7, 0.9):
            cases += [(8, 8, f"sddmm_L8R8_s{sp}_{tag}", 1, var, VEC, sp) for var, tag in ((0, "k64"), (4, "dense_tile"))]
        for pa, pb, name, mma, var, v, sp in cases:
            r = sddmm_case(pa, pb, mma=mma, variant=var, V=v, sparsity=sp)
            variants[name] = {"tops": r["tops"], "ms": r["ms"], "gbs": r["gbs"],
                              "hbm_frac": r["gbs"] / peaks["hbm_gbs"],
                              "verified": verify_sddmm(r, pa, pb, v, [B - 1])}
            del r
            torch.cuda.empty_cache()
        # the dense-tile kernel reads packed values, or the slot-major layout the
        # packer also writes (its builders then load whole slots)
        for mma, var, tag, lay in ((1, 0, MMA_NAMES[1], 0), (1, 3, "tma_gather_kernel", 0), (2, 0, MMA_NAMES[2], 0),
                                   (sync_mma, 1, "per_row_kernel", 0), (0, 4, "dense_tile", 0),
                                   (0, 4, "dense_tile_slot_major", 2)):
            variants[f"spmm_L8R8_1024x1024x256_{tag}"] = spmm_variant(
                args, dev, stream, peaks, world, sync_all, max_over_ranks, mma, var, lay)
        # small vectors: an int8 MMA computes 8 vector lanes of which V are
        # used; the dp4a consumers compute only the V lanes
        for v in (2, 4):
            for pa, pb in ((8, 8), (8, 4), (4, 4)):
                for mma in (1, 4):
                    variants[f"spmm_L{pa}R{pb}_4096x4096x256_V{v}_s0.9_{MMA_NAMES[mma]}"] = spmm_point(
                        args, dev, stream, peaks, 4096, 4096, 256, v, pa, pb, mma)
                    torch.cuda.empty_cache()
            # the dense-tile kernel (tcgen05 f16, every product of 256-row tiles):
            # its speed does not depend on V
            variants[f"spmm_L8R8_4096x4096x256_V{v}_s0.9_dense_tile_slot_major"] = spmm_point(
                args, dev, stream, peaks, 4096, 4096, 256, v, 8, 8, 0, variant=4, layout=2)
            torch.cuda.empty_cache()
        for sp in (0.5, 0.7):
            for var, tag, lay in ((0, "default", 0), (4, "dense_tile_slot_major", 2)):
                variants[f"spmm_L8R8_2048x2048x256_V8_s{sp}_{tag}"] = spmm_point(
                    args, dev, stream, peaks, 2048, 2048, 256, 8, 8, 8, 0, sparsity=sp, variant=var, layout=lay)
                torch.cuda.empty_cache()
    attention = serving_res = packer = projection = competitors = native_server = None
    if not args.headline_only and rank == 0:
        torch.cuda.empty_cache()
        packer = packer_suite(args, dev, peaks)
        torch.cuda.empty_cache()
        projection = projection_suite(args, dev, peaks)
        torch.cuda.empty_cache()
        competitors = competitor_suite(args, dev)
        torch.cuda.empty_cache()
        attention = attention_suite(args, dev)
        torch.cuda.empty_cache()
        native_server = native_server_suite(args, dev)
        torch.cuda.empty_cache()
        if args.serving_requests > 0:
            serving_res = serving_suite(args, dev)

    tpk = tensor_peaks(dev)
    if args.mma == 3:
        mp = ROOT / "MEASURED_PEAKS.json"
        tensor_peak = float(json.loads(mp.read_text())["bf16_tflops"]) if mp.exists() else 1900.0
        tensor_peak_source = "measured dense bf16 GEMM burst (MEASURED_PEAKS.json)" if mp.exists() else "fallback"
    else:
        tensor_peak = tpk["int8_mma_sync" if args.mma == 1 else "f16_mma_sync"]
        tensor_peak_source = "measured mma.sync probe (mcProbeTensorPeak)"
    if rank == 0:
        gbs = head["gbs"]
        line = {
            "metric": METRIC, "value": head["tops"], "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": head["ms"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "int8", "data": "synthetic",
            "config": headline_config(B, world),
            "roofline": {"bound": "hbm", "achieved": gbs, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                         "frac": gbs / peaks["hbm_gbs"],
                         "traffic": (measured_traffic_per_instance() * B
                                     if measured_traffic_per_instance() and args.mma == 1 else None),
                         "traffic_source": "ncu capture of 32 instances scaled to the launch (see profiles/)",
                         "algorithmic_bytes": head["bytes"], "peak_source": peaks["source"]},
            # The contraction's tensor path and its measured peak: mma.sync int8
            # / f16 (probe), or tcgen05 kind::f16 (the measured dense bf16/f16
            # GEMM rate); sm_103a has no integer tcgen05.mma.
            "tensor_roofline": {"tensor_path": MMA_NAMES[args.mma], "achieved": head["tops"], "peak": tensor_peak,
                                "unit": "TOP/s",
                                "frac": head["tops"] / tensor_peak, "peak_source": tensor_peak_source,
                                "probe_tops": tpk},
            "e2e": e2e,
            "verified": verified,
            "verified_how": "instances 0 and last of the final timed step equal the oracle (host SDDMM routine "
                            "restated, signed lanes) bit for bit",
            "gpu_launches": args.steps * launches_per_step,
            "clocks": head["clocks"],
            "variants": variants,
            "batched_attention": attention,
            "attention_server": native_server,
            "serving": serving_res,
            "device_packer": packer,
            "qkv_projection": projection,
            "competitors": competitors,
        }
        if not args.no_cpu_baseline:
            line["cpu_baseline"] = cpu_baseline()
        print(json.dumps(line))
    reps.close()


def spmm_variant(args, dev, stream, peaks, world, sync_all, max_over_ranks, mma: int, variant: int = 0,
                 layout: int = 0) -> dict:
    """SpMM L8-R8: A 1024x1024 V=8 sparsity 0.9, B 1024x256, 256 instances per
    launch (own B and C each, one value set) so a step exceeds 2x L2.
    Algorithmic bytes on the true nonzeros: values nnz V, B K N and C M N 4 per
    instance, column indices, offset pairs and row order once.  The first and
    last instances are checked against the oracle after the timed loop."""
    import torch

    import oracle
    from magicube_gb300 import formats, ops
    M, K, N, B = SPMM_M, SPMM_K, SPMM_N, 256
    mask, vals, rng = spmm_operands()
    h = formats.prepare_spmm(mask, vals, 8, 8, layout=layout)
    d = ops.DeviceSpmmLhs.from_host(h, dev)
    d.values = d.values.repeat(B)  # one value set per instance
    rhs_h = rng.integers(0, 256, size=(B, K * N), dtype=np.uint8)
    rhs = torch.from_numpy(rhs_h).to(dev)
    out = torch.empty((B, M, N), dtype=torch.int32, device=dev)
    fn = lambda: ops.spmm(d, rhs, N, signed=True, out=out, batch=B, values_stride=h.values.size, mma_kind=mma,
                          variant=variant, value_layout=layout)
    sync_all()
    ms = time_cuda(fn, args.steps, args.warmup, stream)
    sync_all()
    t = max_over_ranks(sum(ms) / 1e3) / args.steps
    opc = 2.0 * mask.nnz_vec * VEC * N * B
    byts = B * (mask.nnz_vec * VEC + K * N + M * N * 4) + mask.nnz_vec * 4 + mask.m_vec * 12
    verified = all(np.array_equal(out[i].cpu().numpy(),
                                  oracle.spmm_host(vals, rhs_h[i], mask.row_offsets, mask.col_indices, mask.m_vec, VEC,
                                                   K, N, 8, 8, oracle.SIGNED)) for i in (0, B - 1))
    return {"tops": opc * world / t / 1e12, "ms": t * 1e3, "gbs": byts / t / 1e9,
            "hbm_frac": byts / t / 1e9 / peaks["hbm_gbs"], "instances_per_step": B, "verified": verified}


def spmm_point(args, dev, stream, peaks, M: int, K: int, N: int, V: int, pa: int, pb: int, mma: int,
               sparsity: float = SPARSITY, seed: int = 17, variant: int = 0, layout: int = 0) -> dict:
    """One SpMM point of the precision/shape sweep (row lengths normal, cv
    0.3): enough instances per launch that a step moves more than 2.5x L2,
    median of `--steps` CUDA-event timings; the last instance is checked
    against the oracle.  Algorithmic bytes as in the sweep."""
    import torch

    import oracle
    from magicube_gb300 import formats, ops, synth
    mask = synth.normal_mask(M // V, K, V, sparsity, cv=0.3, seed=seed)
    vals = synth.random_bytes(mask.nnz_vec * V * pa // 8, seed + 1)
    h = formats.prepare_spmm(mask, vals, pa, pb, layout=layout)
    l2 = int(getattr(torch.cuda.get_device_properties(dev), "L2_cache_size", 0)) or 129 * 2 ** 20
    per_inst = h.values.size + K * N * pb // 8 + M * N * 4
    B = max(1, min(1024, -(-int(2.5 * l2) // per_inst)))
    d = ops.DeviceSpmmLhs.from_host(h, dev)
    d.values = d.values.repeat(B)
    rhs_h = synth.random_bytes(B * K * N * pb // 8, seed + 2).reshape(B, -1)
    rhs = torch.from_numpy(rhs_h).to(dev)
    out = torch.empty((B, M, N), dtype=torch.int32, device=dev)
    fn = lambda: ops.spmm(d, rhs, N, signed=True, out=out, batch=B, values_stride=h.values.size,  # noqa: E731
                          mma_kind=mma, variant=variant, value_layout=layout)
    t = statistics.median(time_cuda(fn, args.steps, args.warmup, stream)) / 1e3
    opc = 2.0 * mask.nnz_vec * V * N * B
    byts = B * (mask.nnz_vec * V * pa / 8 + K * N * pb / 8 + M * N * 4) + 4 * mask.nnz_vec + 4 * (mask.m_vec + 1)
    ref = oracle.spmm_host(vals, rhs_h[B - 1], mask.row_offsets, mask.col_indices, mask.m_vec, V, K, N, pa, pb,
                           oracle.SIGNED)
    return {"tops": opc / t / 1e12, "ms": t * 1e3, "gbs": byts / t / 1e9, "hbm_frac": byts / t / 1e9 / peaks["hbm_gbs"],
            "instances_per_step": B, "verified": bool(np.array_equal(out[B - 1].cpu().numpy(), ref))}


def attention_suite(args, dev) -> dict:
    """Batched uneven sparse attention: 64 instances x 4 heads, head dim 64,
    sequence lengths uniform in [512, 4096] (multiples of 64), each instance's
    mask a 256-wide band plus random V=8 column vectors at total sparsity 0.9;
    int8 Q/K/V, int8 probabilities.  All instances and heads in one
    graph-captured launch sequence against the plain per-instance launches,
    the latter both from a host loop and replayed from one CUDA graph that
    holds all 4 x 64 launches (no host launch cost).  Each requantization
    mode is timed against per-instance launches of the same mode: fixed
    scale (the reference's), and row-max (per-row divisors), whose fused
    outputs are checked equal to the per-instance ones bit for bit.  The
    output error against the float64 oracle of the unquantized attention is
    stated over all 64 instances (median and maximum relative Frobenius
    error)."""
    import torch

    import oracle.attention as oatt
    from magicube_gb300 import batched, synth
    rng = np.random.default_rng(11)
    n_inst, H, d, V = 64, 4, 64, 8
    lens = (rng.integers(512, 4097, size=n_inst) // 64 * 64).clip(512, 4096).tolist()
    masks = [synth.band_random_mask(L, V, 256, 0.9, seed=100 + i) for i, L in enumerate(lens)]
    total = int(sum(lens))
    gen = torch.Generator().manual_seed(12)
    qkv_host = (torch.randn(3, H, total, d, generator=gen) * 0.5).half()
    amax = float(qkv_host.abs().max())
    # a float32 scale: the Python launches square it in float64 and the C++
    # engine in float32, the same value when the scale itself is a float32
    sq, ss = float(np.float32(127.0 / amax)), 127.0
    b = batched.BatchedSparseAttention(masks, H, d, 8, 8, scale_qkv=sq, scale_sfmx=ss, device=dev, tune=True)
    b.qkv.copy_(qkv_host.to(dev))
    b.capture()
    stream = torch.cuda.current_stream()
    med = lambda xs: statistics.median(xs)  # noqa: E731
    t_b = med(time_cuda(lambda: b.replay(), args.steps, args.warmup, stream))
    qkvs = [b.qkv[:, :, int(b.token_offsets[i]):int(b.token_offsets[i + 1])].contiguous() for i in range(n_inst)]
    base = {}
    for mode in ("fixed", "rowmax"):
        p = batched.PerInstanceSparseAttention(masks, H, d, 8, 8, scale_qkv=sq, scale_sfmx=ss, device=dev,
                                               requant=mode)
        t_host = med(time_cuda(lambda: p(qkvs), args.steps, args.warmup, stream))
        p.capture(qkvs)
        t_graph = med(time_cuda(lambda: p.replay(), args.steps, args.warmup, stream))
        base[mode] = {"host_loop_ms": t_host, "graph_ms": t_graph, "outs": [c.out.clone() for c in p.cores]}
        del p
        torch.cuda.empty_cache()
    same = all(torch.equal(b.instance_output(i), o) for i, o in enumerate(base["fixed"]["outs"]))
    ref_out = b.core.out.clone()
    fused = {}
    for mode in ("fixed", "rowmax"):
        f = batched.BatchedSparseAttention(masks, H, d, 8, 8, scale_qkv=sq, scale_sfmx=ss, device=dev, fused=True,
                                           requant=mode, tune=True)
        f.qkv.copy_(b.qkv)
        f.capture()
        t_f = med(time_cuda(lambda: f.replay(), args.steps, args.warmup, stream))
        bm = base[mode]
        fused[mode] = {"ms": t_f, "req_per_s": n_inst / (t_f / 1e3),
                       "per_instance_host_loop_ms": bm["host_loop_ms"], "per_instance_graph_ms": bm["graph_ms"],
                       "speedup_vs_per_instance_host_loop": bm["host_loop_ms"] / t_f,
                       "speedup_vs_per_instance_graph": bm["graph_ms"] / t_f,
                       "launches": 2, "status": int(f.core.status.item()), "tuned": f.core.fused_cfg,
                       "identical_to_per_instance": all(torch.equal(f.instance_output(i), o)
                                                        for i, o in enumerate(bm["outs"]))}
        if mode == "fixed":
            fused[mode]["identical_to_separate_steps"] = bool(torch.equal(f.core.out, ref_out))
        fused[mode]["_out"] = f.core.out.clone()
        del f
        torch.cuda.empty_cache()
    # the same row-max attention through the library's C++ engine
    # (mcAttnBatch*: mask builder, quantize + fused launch, its own tuner and
    # CUDA graph; no PyTorch on the path)
    eng = batched.NativeBatchedSparseAttention(masks, H, d, 8, 8, scale_qkv=sq, scale_sfmx=ss, device=dev,
                                               requant="rowmax")
    eng.qkv.copy_(b.qkv)
    eng.tune()
    eng.capture()
    t_e = med(time_cuda(lambda: eng.replay(), args.steps, args.warmup, stream))
    native = {"ms": t_e, "req_per_s": n_inst / (t_e / 1e3), "tuned": eng.config,
              "speedup_vs_per_instance_graph": base["rowmax"]["graph_ms"] / t_e,
              "identical_to_python_fused": bool(torch.equal(eng.out, fused["rowmax"]["_out"])),
              "launches": 2, "status": eng.status()}
    del eng
    torch.cuda.empty_cache()
    # the other precision pairs of the fused kernel (tuned), each against the
    # separate batched launches of the same pair: L16-R8 (16-bit
    # probabilities at the full range, fixed requantization) and L8-R4 (4-bit
    # Q / K / V, row-max requantization)
    pairs = {}
    for (lb, rb, mode, s_q, s_p) in ((16, 8, "fixed", sq, 32767.0), (8, 4, "rowmax", 7.0 / amax, 127.0)):
        key = f"L{lb}R{rb}_{mode}"
        kw = dict(scale_qkv=s_q, scale_sfmx=s_p, device=dev, requant=mode)
        f = batched.BatchedSparseAttention(masks, H, d, lb, rb, fused=True, tune=True, **kw)
        f.qkv.copy_(b.qkv)
        f.capture()
        t_f = med(time_cuda(lambda: f.replay(), args.steps, args.warmup, stream))
        sep = batched.BatchedSparseAttention(masks, H, d, lb, rb, tune=False, **kw)
        same_bits = bool(torch.equal(sep(b.qkv), f.core.out))
        pairs[key] = {"ms": t_f, "req_per_s": n_inst / (t_f / 1e3), "tuned": f.core.fused_cfg,
                      "identical_to_separate_launches": same_bits, "scales": {"qkv": s_q, "softmax": s_p},
                      "_out": f.core.out.clone()}
        del f, sep
        torch.cuda.empty_cache()
    nnz = sum(m.nnz_vec for m in masks)
    ops = 4.0 * nnz * V * d * H
    # accuracy: every instance against the float64 oracle (row-wise form)
    outs = {"batched_fixed": b.core.out, "fused_fixed": fused["fixed"]["_out"], "fused_rowmax": fused["rowmax"]["_out"]}
    outs.update({f"fused_{k}": v["_out"] for k, v in pairs.items()})
    errs = {k: [] for k in outs}
    for i in range(n_inst):
        a, z = int(b.token_offsets[i]), int(b.token_offsets[i + 1])
        q, k, v = (qkv_host[j, :, a:z].double().numpy() for j in range(3))
        ref = oatt.sparse_attention_fp64_rows(q, k, v, masks[i].row_offsets, masks[i].col_indices, V, d ** -0.5)
        nref = np.linalg.norm(ref)
        for key, o in outs.items():
            got = o[:, a:z].double().cpu().numpy()
            errs[key].append(float(np.linalg.norm(got - ref) / nref))
    for m in list(fused.values()) + list(pairs.values()):
        del m["_out"]
    err_summary = {k: {"median": statistics.median(v), "max": max(v), "instances": len(v)} for k, v in errs.items()}
    return {"config": "64 instances x 4 heads, d=64, L ~ U[512,4096], band 256 + random V=8, sparsity 0.9, "
                      "int8 Q/K/V, int8 probabilities",
            "tokens": total, "nonzero_vectors": int(nnz), "batched_ms": t_b,
            "per_instance_host_loop_ms": base["fixed"]["host_loop_ms"],
            "per_instance_graph_ms": base["fixed"]["graph_ms"],
            "batched_req_per_s": n_inst / (t_b / 1e3),
            "speedup_vs_per_instance_host_loop": base["fixed"]["host_loop_ms"] / t_b,
            "speedup_vs_per_instance_graph": base["fixed"]["graph_ms"] / t_b,
            "batched_tops": ops / (t_b / 1e3) / 1e12,
            "launches": {"batched": 4, "per_instance": 4 * n_inst, "batched_is_cuda_graph": True},
            "results_identical": bool(same), "scales": {"qkv": sq, "softmax": ss},
            "fused": fused,
            "fused_other_pairs": pairs,
            "native_engine_rowmax": native,
            "rel_error_vs_fp64_all_instances": err_summary,
            "autotuned": {"sddmm": b.core.sddmm_cfg, "spmm": b.core.spmm_cfg}}


def packer_suite(args, dev, peaks) -> dict:
    """The vector-sparse packer on the GPU (mcDevice*: aligned pairs, padded
    columns, packed values, longest-first row order) against the library's
    host packer, on one SpMM L8-R8 operand: 16,384 vector-rows (M = 131,072),
    K = 4096, V = 8, row lengths ~ Normal(0.1 K, 0.3 mu), random int8 values.
    Device packing runs without a host round trip (upper-bound buffers)."""
    import torch

    from magicube_gb300 import device_format as dfm
    from magicube_gb300 import formats, synth
    m = synth.normal_mask(16384, 4096, VEC, 0.9, seed=21)
    vals = synth.random_bytes(m.nnz_vec * VEC, 22)
    t0 = time.perf_counter()
    h = formats.prepare_spmm(m, vals, 8, 8)
    host_s = time.perf_counter() - t0
    ro, ci = torch.from_numpy(m.row_offsets).to(dev), torch.from_numpy(m.col_indices).to(dev)
    dv = torch.from_numpy(vals).to(dev)
    stream = torch.cuda.current_stream()

    def step():
        dfm.prepare_spmm(ro, ci, dv, VEC, m.ncols, 8, 8, sync=False)

    ms = time_cuda(step, 10, 3, stream)
    t = sum(ms) / len(ms)
    d = dfm.prepare_spmm(ro, ci, dv, VEC, m.ncols, 8, 8)
    same = (np.array_equal(d.values.cpu().numpy(), h.values) and np.array_equal(d.col_indices.cpu().numpy(),
                                                                                 h.col_indices))
    mv, nnz, al = m.m_vec, m.nnz_vec, h.aligned_nnz
    nbytes = (4 * (mv + 1) + 4 * nnz + nnz * VEC) + (8 * mv + 4 * al + al * VEC + 4 * mv)
    gbs = nbytes / (t / 1e3) / 1e9
    return {"workload": "SpMM L8-R8 operand: 16384 vector-rows x 4096, V=8, sparsity 0.9 (normal row lengths), "
                        "packed value layout, sorted rows",
            "nnz_vec": int(nnz), "aligned_nnz": int(al), "algorithmic_bytes": int(nbytes),
            "device_ms": t, "device_gbs": gbs, "hbm_frac": gbs / peaks["hbm_gbs"],
            "host_ms": host_s * 1e3, "speedup_vs_host_packer": host_s * 1e3 / t,
            "identical_to_host_packer": bool(same)}


def projection_suite(args, dev, peaks) -> dict:
    """The attention's input projection (hidden 256 -> Q, K, V of 4 heads x 64)
    over the batched-attention token count (160,640 tokens): the fused tcgen05
    projection + quantization (mcQkvProjectQuantize) against the unfused path
    (cuBLAS fp16 F.linear, permute to [3, H, T, d], mcQuantize)."""
    import torch
    import torch.nn.functional as F

    from magicube_gb300 import _lib
    from magicube_gb300.projection import qkv_project_quantize
    T, E, H, bits, scale = 160640, 256, 4, 8, 40.0
    g = torch.Generator().manual_seed(31)
    x = (torch.randn(T, E, generator=g) * 0.5).half().to(dev)
    w = (torch.randn(3 * E, E, generator=g) / 16).half().to(dev)
    b = (torch.randn(3 * E, generator=g) * 0.1).half().to(dev)
    out = torch.empty((3, H, T * (E // H) * bits // 32), dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream()
    sh = ctypes.c_void_p(stream.cuda_stream)

    def fused():
        qkv_project_quantize(x, w, b, H, bits, scale, out=out)

    def unfused():
        qkv = F.linear(x, w, b).view(T, 3, H, E // H).permute(1, 2, 0, 3).contiguous()
        _lib.check(_lib.lib().mcQuantize(qkv.data_ptr(), out.data_ptr(), qkv.numel(), bits, scale, sh), "mcQuantize")

    ms_f = statistics.median(time_cuda(fused, 20, 5, stream))
    ms_u = statistics.median(time_cuda(unfused, 20, 5, stream))
    nbytes = 2 * T * E + 2 * 3 * E * E + 2 * 3 * E + 3 * T * E * bits // 8
    flops = 2.0 * T * E * 3 * E
    gbs = nbytes / (ms_f / 1e3) / 1e9
    return {"workload": "x [160640, 256] half @ W [768, 256]^T + b -> int8 Q, K, V [3][4][160640][64]",
            "fused_ms": ms_f, "unfused_ms": ms_u, "speedup": ms_u / ms_f,
            "algorithmic_bytes": int(nbytes), "fused_gbs": gbs, "hbm_frac": gbs / peaks["hbm_gbs"],
            "fused_tflops": flops / (ms_f / 1e3) / 1e12,
            "launches": {"fused": 1, "unfused": "F.linear + permute copy + mcQuantize"}}


def competitor_suite(args, dev) -> dict:
    """The reference's competitor baselines (baselines/spmm_benchmark.cpp:
    cuBLAS int8 / fp16 dense GEMM, cuSPARSE fp16 CSR SpMM; cuSPARSE SDDMM) on
    this GPU through torch (cuBLASLt, cuSPARSE), against this library's kernels
    called once per matrix, on the two headline shapes: SpMM A 1024 x 1024 (V=8
    vectors at sparsity 0.9) x B 1024 x 256, and SDDMM A, B 4096 x 64 with a
    4096 x 4096 V=8 mask at sparsity 0.9.  Times are device microseconds per
    matrix: 20 calls captured in a CUDA graph, replayed, CUDA events around
    the replay (the host launch overhead of single calls would otherwise hide
    kernels of a few microseconds); "eager" marks a call whose capture failed
    and that was timed call by call instead."""
    import torch

    from magicube_gb300 import formats, ops, synth
    rng = np.random.default_rng(5)
    modes = {}

    def us(fn, name):
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):
            for _ in range(3):
                fn()
            torch.cuda.synchronize()
            try:
                g = torch.cuda.CUDAGraph()
                with torch.cuda.graph(g, stream=side):
                    for _ in range(20):
                        fn()
                ms = time_cuda(g.replay, 10, 2, side)
                modes[name] = "graph"
                return statistics.median(ms) * 1e3 / 20
            except Exception:  # noqa: BLE001 -- fall back to per-call timing
                torch.cuda.synchronize()
                modes[name] = "eager"
                return statistics.median(time_cuda(fn, 50, 5, side)) * 1e3

    def csr_of(mask, ncols, dtype, values=None):
        # element-level CSR of the vector-sparse matrix (each vector = V rows)
        V = mask.vec_length
        rows, cols = [], []
        for i in range(mask.m_vec):
            c = mask.col_indices[mask.row_offsets[i]:mask.row_offsets[i + 1]]
            for v in range(V):
                rows.append(np.full(c.size, i * V + v))
                cols.append(c)
        r = np.concatenate(rows)
        c = np.concatenate(cols)
        vals = torch.from_numpy(values if values is not None else rng.standard_normal(r.size).astype(np.float32))
        coo = torch.sparse_coo_tensor(torch.from_numpy(np.stack([r, c])), vals, (mask.m_vec * V, ncols))
        return coo.to(dtype).to(dev).to_sparse_csr()

    res = {}
    # ---- SpMM ----
    M = K = 1024
    N = 256
    mask = synth.uniform_mask(M // VEC, K, VEC, SPARSITY, seed=7)
    vals = rng.integers(0, 256, size=mask.nnz_vec * VEC, dtype=np.uint8)
    h = formats.prepare_spmm(mask, vals, 8, 8)
    d = ops.DeviceSpmmLhs.from_host(h, dev)
    rhs8 = torch.from_numpy(rng.integers(0, 256, size=K * N, dtype=np.uint8)).to(dev)
    out = torch.empty((M, N), dtype=torch.int32, device=dev)
    a8 = torch.randint(-128, 128, (M, K), dtype=torch.int8, device=dev)
    b8 = torch.randint(-128, 128, (K, N), dtype=torch.int8, device=dev)
    a16, b16 = a8.half(), b8.half()
    acsr = csr_of(mask, K, torch.float16)
    res["spmm_1024x1024x256_V8_s0.9"] = {
        "magicube_L8R8_us": us(lambda: ops.spmm(d, rhs8, N, signed=True, out=out), "spmm_magicube"),
        "cublas_int8_dense_us": us(lambda: torch._int_mm(a8, b8), "spmm_cublas_int8"),
        "cublas_fp16_dense_us": us(lambda: torch.mm(a16, b16), "spmm_cublas_fp16"),
        "cusparse_fp16_csr_us": us(lambda: torch.mm(acsr, b16), "spmm_cusparse"),
    }
    # ---- SDDMM ----
    smask, hm, lhs_h, rhs_h = sddmm_workload(8, 8, 1)
    dm = ops.DeviceSddmmMask.from_host(hm, dev)
    lhs = torch.from_numpy(lhs_h).to(dev)
    rhs = torch.from_numpy(rhs_h).to(dev)
    sout = torch.empty(hm.aligned_nnz * VEC, dtype=torch.int32, device=dev)
    qa = torch.randint(-128, 128, (SEQ, HEAD_DIM), dtype=torch.int8, device=dev)
    qb = torch.randint(-128, 128, (HEAD_DIM, SEQ), dtype=torch.int8, device=dev)
    fa, fb = qa.half(), qb.half()
    smask_csr = csr_of(smask, SEQ, torch.float32, np.ones(smask.nnz_vec * VEC, np.float32))
    fa32, fb32 = qa.float(), qb.float()
    res["sddmm_4096x4096x64_V8_s0.9"] = {
        "magicube_L8R8_us": us(lambda: ops.sddmm(dm, lhs, rhs, HEAD_DIM, 8, 8, signed=True, out=sout),
                               "sddmm_magicube"),
        "cublas_int8_dense_us": us(lambda: torch._int_mm(qa, qb), "sddmm_cublas_int8"),
        "cublas_fp16_dense_us": us(lambda: torch.mm(fa, fb), "sddmm_cublas_fp16"),
        "cusparse_fp32_sddmm_us": us(lambda: torch.sparse.sampled_addmm(smask_csr, fa32, fb32), "sddmm_cusparse"),
    }
    for v in res.values():
        base = v["magicube_L8R8_us"]
        v["speedup_vs"] = {k[:-3]: round(x / base, 2) for k, x in v.items() if k.endswith("_us") and k != "magicube_L8R8_us"}
    res["timing"] = modes
    return res


def formats_align(mask, alignment):
    from magicube_gb300 import formats
    pairs, n = formats.align_row_offsets(mask, alignment)
    cols = formats.pad_column_indices(mask, pairs, n, False)
    return (pairs, cols), n


def native_server_suite(args, dev) -> dict:
    """The C++ request loop (mcAttnServer*) on the batched-attention workload
    as a stream of requests: 64 sequences, lengths uniform in [512, 4096],
    band 256 + random V=8 vectors at sparsity 0.9, 4 heads of 64, row-max
    requantization; Q/K/V and masks resident on the device.  Arrivals all at
    once, and Poisson at 100,000 and 20,000 requests/s.  Continuous batching
    (batches of up to 32,768 tokens, two on the device) against one request
    at a time (one request per batch, one batch on the device); each server
    is run once untimed on the same requests first.  The outputs of the two
    modes are compared bit for bit."""
    import torch

    from magicube_gb300 import batched, synth
    rng = np.random.default_rng(11)
    n, H = 64, 4
    lens = (rng.integers(512, 4097, size=n) // 64 * 64).clip(512, 4096).tolist()
    masks = [synth.band_random_mask(L, VEC, 256, 0.9, seed=100 + i) for i, L in enumerate(lens)]
    g = torch.Generator().manual_seed(12)
    qkvs = [(torch.randn(3, H, L, 64, generator=g) * 0.5).half().to(dev) for L in lens]
    amax = max(float(q.abs().max()) for q in qkvs)
    sq = float(np.float32(127.0 / amax))
    modes = {"continuous": dict(max_batch_tokens=32768, max_inflight=2),
             "one_at_a_time": dict(max_batch_tokens=1, max_inflight=1)}
    arr_rng = np.random.default_rng(5)
    runs, outs_by_mode = [], {}
    for rate in (None, 100000.0, 20000.0):
        arrivals = np.zeros(n) if rate is None else np.cumsum(arr_rng.exponential(1.0 / rate, size=n))
        run = {"arrival_rate": "all at once" if rate is None else rate}
        for mode, kw in modes.items():
            srv = batched.NativeAttentionServer(heads=H, scale_qkv=sq, scale_sfmx=127.0, requant="rowmax", **kw)
            outs = [torch.empty((H, L, 64), dtype=torch.float16, device=dev) for L in lens]
            made = [srv.request(m, q, o, float(a), dev) for m, q, o, a in zip(masks, qkvs, outs, arrivals)]
            reqs = [r for r, _ in made]
            srv.run(reqs)
            lat, st = srv.run(reqs)
            run[mode] = {"req_per_s": st["req_per_s"], "p50_ms": st["p50_ms"], "p99_ms": st["p99_ms"],
                         "batches": st["batches"], "max_inflight_seen": st["max_inflight_seen"],
                         "served": st["served"], "rejected": st["rejected"]}
            outs_by_mode[mode] = outs
            del srv, made
        run["ratio_req_per_s"] = run["continuous"]["req_per_s"] / max(run["one_at_a_time"]["req_per_s"], 1e-9)
        runs.append(run)
    same = all(torch.equal(a, b) for a, b in zip(outs_by_mode["continuous"], outs_by_mode["one_at_a_time"]))
    return {"config": f"{n} sequences x {H} heads, d=64, L ~ U[512,4096], band 256 + random V=8, sparsity 0.9, "
                      "int8 Q/K/V, row-max requantization; C++ request loop (mcAttnServer)",
            "runs": runs, "outputs_identical_across_modes": bool(same)}


def serving_suite(args, dev) -> dict:
    """Continuous batching of a 2-layer sparse encoder (hidden 256, 4 x 64
    heads, FFN 1024, random-init weights), int8 vector-sparse attention at
    sparsity 0.95; Poisson arrivals at each rate of `--serving-rates`, lengths
    lognormal (median 2048, clipped to [256, 8192]).  The server runs the
    fused attention kernel; the baseline serves the same requests one at a
    time on the plain separate SDDMM / softmax / SpMM launches (same bits,
    row-max requantization).  The attention output's error against the
    float64 oracle is stated for a few requests of this workload."""
    import torch

    from magicube_gb300 import model, serving
    torch.manual_seed(0)
    enc = model.SparseEncoder(2, 256, 4, 1024).to(dev).half().eval()
    # row-max requantization (probabilities relative to each row's maximum):
    # the accurate 8-bit mode; the fused and the separate launches give the
    # same bits in it
    fused = lambda: enc.set_attention("fused", "rowmax")  # noqa: E731
    plain = lambda: enc.set_attention("separate", "rowmax")  # noqa: E731
    warm = serving.make_requests(4, 0.0, seed=99)
    serving.ContinuousBatchingServer(fused(), device=dev).serve(warm)
    serving.serve_sequential(plain(), serving.make_requests(2, 0.0, seed=98), device=dev)
    out = []
    for rate in args.serving_rates:
        # Each server first serves the same request set unmeasured, so both
        # measured runs see warmed allocator pools for the same shapes.
        serving.ContinuousBatchingServer(fused(), max_inflight=3, overlap_tokens=args.serving_overlap_tokens,
                                         device=dev).serve(serving.make_requests(args.serving_requests, rate, seed=5))
        reqs = serving.make_requests(args.serving_requests, rate, seed=5)
        srv = serving.ContinuousBatchingServer(fused(), max_inflight=3, overlap_tokens=args.serving_overlap_tokens,
                                               device=dev)
        cb = srv.serve(reqs)
        serving.serve_sequential(plain(), serving.make_requests(args.serving_requests, rate, seed=5), device=dev)
        # the one-at-a-time baseline is host-bound and varies between runs:
        # three measured runs, the median by throughput is reported
        seqs = sorted((serving.serve_sequential(plain(), serving.make_requests(args.serving_requests, rate, seed=5),
                                                device=dev) for _ in range(3)), key=lambda r: r["req_per_s"])
        seq = seqs[1]
        out.append({"arrival_rate": rate, "overlap_tokens": args.serving_overlap_tokens, "continuous": cb,
                    "sequential": seq, "sequential_req_per_s_runs": [r["req_per_s"] for r in seqs],
                    "mean_batch": float(np.mean([len(b) for b in srv.batches])),
                    "peak_batches_in_flight": srv.peak_inflight, "admissions_held_back": srv.held_back,
                    "req_per_s_ratio": cb["req_per_s"] / seq["req_per_s"]})
    return {"config": "2-layer sparse encoder, hidden 256, 4x64 heads, FFN 1024, sparsity 0.95, "
                      "lengths lognormal(median 2048) in [256, 8192]",
            "kernels": {"continuous": "fused attention kernel", "sequential": "separate SDDMM/softmax/SpMM"},
            "runs": out,
            "requant": "rowmax",
            "attention_rel_error_vs_fp64": encoder_attention_error(fused(), dev)}


def encoder_attention_error(enc, dev, n_requests: int = 4) -> dict:
    """The served encoder's attention output against the float64 oracle of
    the unquantized attention, per layer, for a few requests of the serving
    workload (lengths lognormal, median 2048): the layer's own input (the
    model's fp16 hidden state), its LayerNorm and projection weights; the
    oracle projects in float64 without quantization and applies the softmax
    over the request's mask of that layer.  Relative Frobenius error of the
    [heads, tokens, 64] output (median and maximum)."""
    import torch

    import oracle.attention as oatt
    from magicube_gb300 import serving
    from magicube_gb300.model import attention_fused_quantized
    from magicube_gb300.projection import qkv_project_quantize
    reqs = serving.make_requests(n_requests, 0.0, seed=5)
    errs = []
    with torch.no_grad():
        for r in reqs:
            serving._upload_csr(r, dev)
            masks = serving.pack_batch_masks([r], len(enc.layers), 8, 16, dev)
            x = r.dev["x"]
            for li, (layer, m) in enumerate(zip(enc.layers, masks)):
                h = layer.ln1(x)
                qkv_q = qkv_project_quantize(h, layer.in_proj.weight, layer.in_proj.bias, layer.heads,
                                             layer.rhs_bits, layer.scale_qkv)
                att = attention_fused_quantized(qkv_q, r.seq_len, m, layer.scale_qkv, layer.scale_sfmx,
                                                layer.requant, layer.lhs_bits, layer.rhs_bits, layer.fused_cfg)
                w = layer.in_proj.weight.double().cpu().numpy()
                bias = layer.in_proj.bias.double().cpu().numpy()
                qkv = h.double().cpu().numpy() @ w.T + bias  # [T, 3E]
                T, E, H = r.seq_len, layer.hidden, layer.heads
                qkv = qkv.reshape(T, 3, H, E // H).transpose(1, 2, 0, 3)  # [3, H, T, d]
                mk = r.masks[li]
                ref = oatt.sparse_attention_fp64_rows(qkv[0], qkv[1], qkv[2], mk.row_offsets, mk.col_indices, 8,
                                                      (E // H) ** -0.5)
                got = att.double().cpu().numpy()
                errs.append({"request_tokens": T, "layer": li,
                             "rel_error": float(np.linalg.norm(got - ref) / np.linalg.norm(ref))})
                x = layer(x, m)
            r.dev.clear()
    e = [x["rel_error"] for x in errs]
    return {"requant": enc.layers[0].requant, "pair": f"L{enc.layers[0].lhs_bits}-R{enc.layers[0].rhs_bits}",
            "median": statistics.median(e), "max": max(e), "per_request_layer": errs}


def tensor_peaks(dev) -> dict:
    """Measured tensor peaks (TOP/s): mma.sync int8 (k = 32 and k = 16), int4
    and f16; tcgen05.mma kind::f16 at M = 128, N = 16 / 64 / 256."""
    import torch

    from magicube_gb300 import _lib
    sink = torch.empty(4 * 256 * 8 * torch.cuda.get_device_properties(dev).multi_processor_count,
                       dtype=torch.uint8, device=dev)
    out = {}
    for kind, name in ((0, "int8_mma_sync"), (1, "int4_mma_sync"), (2, "f16_mma_sync"), (3, "int8_k16_mma_sync"),
                       (4, "int8_dp4a"), (5, "int8_mma_plus_dp4a")):
        ms, ops = ctypes.c_float(), ctypes.c_double()
        _lib.check(_lib.probe_lib().mcProbeTensorPeak(kind, sink.data_ptr(), sink.numel(), 2048, ctypes.byref(ms),
                                                ctypes.byref(ops), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)),
                   "mcProbeTensorPeak")
        out[name] = ops.value / (ms.value * 1e-3) / 1e12
    timeouts = torch.zeros(1, dtype=torch.int32, device=dev)
    for n in (16, 64, 256):  # tcgen05.mma kind::f16, M = 128, K = 16 (padding included)
        ms, ops = ctypes.c_float(), ctypes.c_double()
        _lib.check(_lib.probe_lib().mcProbeTensorCorePeak(n, 8000, ctypes.byref(ms), ctypes.byref(ops),
                                                    timeouts.data_ptr(),
                                                    ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)),
                   "mcProbeTensorCorePeak")
        out[f"tcgen05_f16_m128n{n}"] = ops.value / (ms.value * 1e-3) / 1e12
    return out


SWEEP_SIZES = (512, 1024, 2048, 4096)
SWEEP_SPARSITY = (0.5, 0.7, 0.8, 0.9, 0.95, 0.98)
SWEEP_PAIRS = ((16, 8), (8, 8), (8, 4), (4, 4), (16, 4))
SWEEP_COLUMNS = ("M", "K", "N", "sparsity", "V", "pair", "batch", "nnz_vec", "us_per_instance", "tops", "gbs",
                 "hbm_frac", "tensor_util", "roofline_frac", "bound")


def run_sweep(args) -> None:
    """SpMM precision/shape sweep on synthetic pruned-weight matrices.

    M, K in {512, 1024, 2048, 4096} (every pair with `--sweep full`, M = K
    with `--sweep square`), N in {128, 256}, sparsity in {0.5, 0.7, 0.8, 0.9,
    0.95, 0.98}, V in {2, 4, 8}, per-vector-row lengths ~ Normal(mu, 0.3 mu)
    clipped to [0, K] with mu = (1 - sparsity) K, pairs L16-R8, L8-R8, L8-R4,
    L4-R4, L16-R4, signed lanes, int32 output.  Each point is one batched
    launch over enough instances (own packed values, B and C; one mask) that
    a step moves more than 2.5x L2, timed with CUDA events (median of
    `--steps`).  The values and B are uniformly random bytes generated on the
    device in the packed layouts (every bit pattern is a valid operand).
    Algorithmic bytes per launch: unpadded values nnz V bits_A/8, B K N
    bits_B/8 and C M N 4 per instance, column indices and offsets once;
    ops 2 nnz V N per instance.  The roofline time is max(bytes / HBM peak,
    MMA ops / measured int8 mma.sync peak), MMA ops counting both byte planes
    of a 16-bit A (4-bit operands run unpacked on the int8 MMA)."""
    import torch

    from magicube_gb300 import formats, ops, synth
    dev = torch.device("cuda:0")
    stream = torch.cuda.current_stream()
    peaks = _peaks()
    int8_peak = tensor_peaks(dev)["int8_mma_sync"]
    l2 = int(getattr(torch.cuda.get_device_properties(dev), "L2_cache_size", 0)) or 129 * 2 ** 20
    target = int(2.5 * l2)
    shapes = ([(m, k) for m in SWEEP_SIZES for k in SWEEP_SIZES] if args.sweep == "full"
              else [(s, s) for s in SWEEP_SIZES])
    steps, warmup = max(args.steps, 1), max(args.warmup, 3)
    rows = []
    t_start = time.time()
    with ClockSampler(0) as clk:
        for M, K in shapes:
            for V in (2, 4, 8):
                for sp in SWEEP_SPARSITY:
                    mask = synth.normal_mask(M // V, K, V, sp, cv=0.3, seed=M * 7 + K * 13 + V * 101 + int(sp * 1000))
                    if mask.nnz_vec == 0:
                        continue
                    ri = torch.from_numpy(formats.sorted_row_swizzle(mask)).to(dev)
                    layouts = {}
                    for chunk in (16, 32):
                        pairs, n_al = formats.align_row_offsets(mask, chunk)
                        cols = formats.pad_column_indices(mask, pairs, n_al, shuffle8=(chunk == 32))
                        layouts[chunk] = (torch.from_numpy(pairs).to(dev), torch.from_numpy(cols).to(dev), n_al)
                    idx_bytes = 4 * mask.nnz_vec + 4 * (mask.m_vec + 1)
                    for pa, pb in SWEEP_PAIRS:
                        ro_d, ci_d, n_al = layouts[formats.spmm_chunk(pa, pb)]
                        vstride = n_al * V * formats.lane_bits(pa) // 8
                        for N in (128, 256):
                            per_inst = vstride + K * N * pb // 8 + M * N * 4
                            B = max(1, min(4096, -(-target // per_inst)))
                            vals = torch.randint(0, 256, (B * vstride,), dtype=torch.uint8, device=dev)
                            rhs = torch.randint(0, 256, (B, K * N * pb // 8), dtype=torch.uint8, device=dev)
                            out = torch.empty((B, M, N), dtype=torch.int32, device=dev)
                            d = ops.DeviceSpmmLhs(M // V, V, K, pa, pb, ri, ro_d, ci_d, vals)
                            fn = lambda: ops.spmm(d, rhs, N, signed=True, out=out, batch=B, values_stride=vstride)
                            t = statistics.median(time_cuda(fn, steps, warmup, stream)) / 1e3
                            opc = 2.0 * mask.nnz_vec * V * N * B
                            mma_ops = opc * (2 if pa == 16 else 1)
                            byts = B * (mask.nnz_vec * V * pa / 8 + K * N * pb / 8 + M * N * 4) + idx_bytes
                            t_hbm, t_tc = byts / (peaks["hbm_gbs"] * 1e9), mma_ops / (int8_peak * 1e12)
                            rows.append([M, K, N, sp, V, f"L{pa}-R{pb}", B, mask.nnz_vec, round(t / B * 1e6, 4),
                                         round(opc / t / 1e12, 3), round(byts / t / 1e9, 1),
                                         round(byts / t / 1e9 / peaks["hbm_gbs"], 4),
                                         round(mma_ops / t / 1e12 / int8_peak, 4),
                                         round(max(t_hbm, t_tc) / t, 4), "hbm" if t_hbm >= t_tc else "tensor"])
                            del vals, rhs, out, d
            print(f"sweep: M={M} K={K} done, {len(rows)} points, {time.time() - t_start:.0f} s",
                  file=sys.stderr, flush=True)
    col = {c: i for i, c in enumerate(SWEEP_COLUMNS)}
    summary = {}
    for pa, pb in SWEEP_PAIRS:
        name = f"L{pa}-R{pb}"
        sel = [r for r in rows if r[col["pair"]] == name]
        hi = [r for r in sel if r[col["sparsity"]] >= 0.9]
        if not sel:
            continue
        summary[name] = {
            "points": len(sel),
            "geomean_gbs": float(np.exp(np.mean(np.log([r[col["gbs"]] for r in sel])))),
            "max_gbs": max(r[col["gbs"]] for r in sel),
            "max_tops": max(r[col["tops"]] for r in sel),
            "median_roofline_frac": statistics.median(r[col["roofline_frac"]] for r in sel),
            "sparsity_ge_0.9": {
                "points": len(hi),
                "median_hbm_frac": statistics.median(r[col["hbm_frac"]] for r in hi) if hi else None,
                "median_roofline_frac": statistics.median(r[col["roofline_frac"]] for r in hi) if hi else None,
                "points_at_ge_60pct_roofline": sum(r[col["roofline_frac"]] >= 0.6 for r in hi)},
        }
    line = {"sweep": "spmm precision/shape", "shapes": args.sweep, "steps": steps, "warmup": warmup,
            "data": "synthetic (normal row lengths, cv 0.3; random packed operands)",
            "l2": f"each step moves > 2.5x L2 ({target / 1e6:.0f} MB)",
            "peaks": {"hbm_gbs": peaks["hbm_gbs"], "hbm_source": peaks["source"], "int8_mma_sync_tops": int8_peak},
            "seconds": round(time.time() - t_start, 1), "clocks": clk.summary(), "summary": summary,
            "columns": list(SWEEP_COLUMNS), "points": rows}
    text = json.dumps(line)
    if args.sweep_out:
        Path(args.sweep_out).parent.mkdir(parents=True, exist_ok=True)
        Path(args.sweep_out).write_text(text + "\n")
    print(text)


def run_profile_case(args) -> None:
    """A small case of one kernel for ncu captures: `--batch` instances of the
    headline SDDMM (about 7.3 MB each) or of the SpMM L8-R8 configuration
    (about 1.4 MB each), launched `--reps` times."""
    import torch

    from magicube_gb300 import formats, ops, synth
    dev = torch.device("cuda:0")
    if args.profile in ("attention", "attention-steps"):
        from magicube_gb300 import batched, synth
        rng = np.random.default_rng(11)
        lens = (rng.integers(512, 4097, size=args.batch) // 64 * 64).clip(512, 4096).tolist()
        masks = [synth.band_random_mask(L, VEC, 256, 0.9, seed=100 + i) for i, L in enumerate(lens)]
        f = batched.BatchedSparseAttention(masks, 4, 64, 8, 8, scale_qkv=40.0, scale_sfmx=127.0, device=dev,
                                           fused=args.profile == "attention", requant=args.requant, tune=True)
        f.qkv.copy_((torch.randn(f.qkv.shape, generator=torch.Generator().manual_seed(12)) * 0.5).half())
        for _ in range(args.reps):
            f()
        torch.cuda.synchronize()
        print(json.dumps({"profile_case": args.profile, "instances": args.batch, "reps": args.reps}))
        return
    if args.profile == "projection":
        from magicube_gb300.projection import qkv_project_quantize
        T, E, H = 131072, 256, 4  # x 64 MB + out 96 MB: more than the 129 MB L2
        g = torch.Generator().manual_seed(31)
        x = (torch.randn(T, E, generator=g) * 0.5).half().to(dev)
        w = (torch.randn(3 * E, E, generator=g) / 16).half().to(dev)
        b = (torch.randn(3 * E, generator=g) * 0.1).half().to(dev)
        for _ in range(args.reps):
            qkv_project_quantize(x, w, b, H, 8, 40.0)
        torch.cuda.synchronize()
        print(json.dumps({"profile_case": "projection", "tokens": T, "reps": args.reps}))
        return
    if args.profile == "packer":
        from magicube_gb300 import device_format as dfm
        from magicube_gb300 import synth
        m = synth.normal_mask(16384, 4096, VEC, 0.9, seed=21)
        vals = synth.random_bytes(m.nnz_vec * VEC, 22)
        ro, ci = torch.from_numpy(m.row_offsets).to(dev), torch.from_numpy(m.col_indices).to(dev)
        dv = torch.from_numpy(vals).to(dev)
        for _ in range(args.reps):
            dfm.prepare_spmm(ro, ci, dv, VEC, m.ncols, 8, 8, sync=False)
        torch.cuda.synchronize()
        print(json.dumps({"profile_case": "packer", "reps": args.reps}))
        return
    if args.profile == "spmm-v2":
        # SpMM L8-R8, M = K = 4096, N = 256, V = 2, sparsity 0.9 (normal row
        # lengths): about 6 MB per instance
        M = K = 4096
        N, V = 256, 2
        mask = synth.normal_mask(M // V, K, V, SPARSITY, cv=0.3, seed=17)
        vals = synth.random_bytes(mask.nnz_vec * V, 18)
        h = formats.prepare_spmm(mask, vals, 8, 8)
        d = ops.DeviceSpmmLhs.from_host(h, dev)
        d.values = d.values.repeat(args.batch)
        rhs = torch.randint(0, 256, (args.batch, K * N), dtype=torch.uint8, device=dev)
        out = torch.empty((args.batch, M, N), dtype=torch.int32, device=dev)
        for _ in range(args.reps):
            ops.spmm(d, rhs, N, signed=True, out=out, batch=args.batch, values_stride=h.values.size,
                     mma_kind=args.mma, variant=args.spmm_kernel)
        torch.cuda.synchronize()
        print(json.dumps({"profile_case": args.profile, "batch": args.batch, "reps": args.reps}))
        return
    if args.profile == "sddmm":
        mask, hm, lhs_h, rhs_h = sddmm_workload(8, 8, args.batch)
        dm = ops.DeviceSddmmMask.from_host(hm, dev)
        lhs, rhs = torch.from_numpy(lhs_h).to(dev), torch.from_numpy(rhs_h).to(dev)
        out = torch.empty((args.batch, hm.aligned_nnz * VEC), dtype=torch.int32, device=dev)
        for _ in range(args.reps):
            ops.sddmm(dm, lhs, rhs, HEAD_DIM, 8, 8, signed=True, out=out, batch=args.batch, mma_kind=args.mma,
                      variant=args.sddmm_kernel)
    else:
        M = K = 1024
        N = 256
        mask = synth.uniform_mask(M // VEC, K, VEC, SPARSITY, seed=7)
        vals = np.random.default_rng(8).integers(0, 256, size=mask.nnz_vec * VEC, dtype=np.uint8)
        layout = formats.VALUES_SLOT_MAJOR if args.spmm_values == "slot_major" else formats.VALUES_PACKED
        h = formats.prepare_spmm(mask, vals, 8, 8, layout=layout)
        d = ops.DeviceSpmmLhs.from_host(h, dev)
        d.values = d.values.repeat(args.batch)
        rhs = torch.randint(0, 256, (args.batch, K * N), dtype=torch.uint8, device=dev)
        out = torch.empty((args.batch, M, N), dtype=torch.int32, device=dev)
        for _ in range(args.reps):
            ops.spmm(d, rhs, N, signed=True, out=out, batch=args.batch, values_stride=h.values.size,
                     mma_kind=0 if args.spmm_kernel == 4 else args.mma, variant=args.spmm_kernel, value_layout=layout)
    torch.cuda.synchronize()
    print(json.dumps({"profile_case": args.profile, "batch": args.batch, "reps": args.reps}))


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--batch", type=int, default=64, help="instances per step")
    ap.add_argument("--impl", choices=["magicube_gb300", "reference"], default="magicube_gb300")
    ap.add_argument("--headline-only", action="store_true")
    ap.add_argument("--requant", choices=["fixed", "rowmax"], default="rowmax",
                    help="requantization of the --profile attention case")
    ap.add_argument("--profile", choices=["sddmm", "spmm", "spmm-v2", "attention", "attention-steps", "packer",
                                          "projection"],
                    default=None,
                    help="run only a small case of one kernel (for ncu captures)")
    ap.add_argument("--reps", type=int, default=3, help="launches of the --profile case")
    ap.add_argument("--serving-rates", type=lambda x: [float(v) for v in x.split(",")],
                    default=[200.0, 2000.0, 20000.0],
                    help="Poisson arrival rates (requests/s) of the serving runs")
    ap.add_argument("--serving-requests", type=int, default=96, help="requests per serving run (0 skips it)")
    ap.add_argument("--serving-overlap-tokens", type=int, default=8192,
                    help="queued tokens at which the server overlaps a new batch with running ones")
    ap.add_argument("--mma", choices=["int8", "f16", "tc", "dp4a"], default="int8",
                    help="arithmetic path of the headline SDDMM: int8 / f16 mma.sync, tcgen05 or CUDA-core dp4a "
                         "(all bit-exact; see include/magicube_gb300.h)")
    ap.add_argument("--sddmm-kernel", choices=["auto", "per_row", "stream", "dense"], default="auto",
                    help="SDDMM kernel variant of the --profile sddmm case")
    ap.add_argument("--spmm-kernel", choices=["auto", "per_row", "stream", "tma", "resident", "dense"], default="auto",
                    help="SpMM kernel variant of the --profile spmm and spmm-v2 cases")
    ap.add_argument("--spmm-values", choices=["packed", "slot_major"], default="packed",
                    help="value layout of the --profile spmm case (slot-major: the dense-tile kernel's own)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--sweep", choices=["square", "full"], default=None,
                    help="run only the SpMM precision/shape sweep (M = K, or every M, K pair)")
    ap.add_argument("--sweep-out", default=None, help="also write the sweep's JSON line to this file")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    args.mma = {"int8": 1, "f16": 2, "tc": 3, "dp4a": 4}[args.mma]
    args.sddmm_kernel = {"auto": 0, "per_row": 1, "stream": 2, "dense": 4}[args.sddmm_kernel]
    args.spmm_kernel = {"auto": 0, "per_row": 1, "stream": 2, "tma": 3, "resident": 5, "dense": 4}[args.spmm_kernel]
    if args.sweep:
        run_sweep(args)
    elif args.profile:
        if args.batch == 64 and args.profile == "spmm":
            args.batch = 128
        run_profile_case(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
