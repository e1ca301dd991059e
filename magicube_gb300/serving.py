"""Continuous-batching server for the sparse encoder.

Requests carry a sequence of their own length and (per encoder layer) their
own vector-sparse attention mask.  On admission a request's tokens and the
plain CSR of its masks are copied to the device once (the masks are packed
there by the GPU packer) and stay resident until it completes.  The scheduler
admits queued requests into a new batch when no batch is in flight, or, for
overlap, when the queued tokens reach a threshold and an in-flight slot is
free, always within the free HBM (the batch's estimated working set); a batch
is one block-diagonal forward pass over the admitted requests (the token
tensors concatenated, the masks stacked into one mask per layer) launched on
its own CUDA stream.  Completion is observed through CUDA events, and each
request's latency is (completion - arrival).

serve_sequential is the baseline: one request at a time, in arrival order,
each its own forward pass.
"""
from __future__ import annotations

import time
from collections import deque
from dataclasses import dataclass, field

import numpy as np
import torch

from . import device_format, formats, synth
from .batched import AttentionMaskDev
from .formats import VectorSparse


@dataclass
class Request:
    rid: int
    seq_len: int
    arrival: float                   # seconds after the start of the run
    x: torch.Tensor                  # [seq_len, hidden] half (host until admitted)
    masks: list[VectorSparse]        # one per encoder layer
    out: torch.Tensor | None = None  # [seq_len, hidden] half
    t_admit: float = float("nan")
    t_done: float = float("nan")
    dev: dict = field(default_factory=dict)
    error: str | None = None         # set when the request was rejected at admission

    @property
    def latency(self) -> float:
        return self.t_done - self.arrival


def make_requests(n: int, rate: float, hidden: int = 256, layers: int = 2, V: int = 8, sparsity: float = 0.95,
                  median: int = 2048, clip: tuple[int, int] = (256, 8192), sigma: float = 0.5,
                  seed: int = 0) -> list[Request]:
    """Poisson arrivals at `rate` requests/s; lengths lognormal(median) clipped,
    rounded to a multiple of 64; uniform random column vectors at `sparsity`."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate, size=n) if rate > 0 else np.zeros(n)
    arrivals = np.cumsum(gaps) - gaps[0]
    lens = np.clip(np.exp(rng.normal(np.log(median), sigma, size=n)), clip[0], clip[1])
    lens = (np.round(lens / 64) * 64).astype(int).clip(clip[0], clip[1])
    reqs = []
    for i in range(n):
        L = int(lens[i])
        x = (torch.randn(L, hidden, generator=torch.Generator().manual_seed(seed * 100003 + i)) * 0.5).half()
        masks = [synth.uniform_mask(L // V, L, V, sparsity, seed=seed * 1000 + i * 10 + l) for l in range(layers)]
        reqs.append(Request(i, L, float(arrivals[i]), x, masks))
    return reqs


def _upload(req: Request, alignment: int, device) -> None:
    """Copy a request's tokens and the plain CSR of its masks to the device
    (once) and pack the masks there (mcDevicePack, no host round trip: slot
    arrays sized by the upper bound nnz + m_vec * (alignment - 1))."""
    if req.dev:
        return
    dev = torch.device(device)
    req.dev["x"] = req.x.to(dev, non_blocking=True)
    per_layer = []
    for m in req.masks:
        if dev.type == "cuda":
            ro = torch.from_numpy(m.row_offsets).to(dev, non_blocking=True)
            ci = torch.from_numpy(m.col_indices).to(dev, non_blocking=True)
            dm = device_format.prepare_sddmm(ro, ci, m.vec_length, m.ncols, alignment=alignment, sync=False)
            per_layer.append((dm.row_offsets, dm.col_indices, dm.row_indices, m.m_vec, dm.aligned_nnz,
                              _max_row(m)))
        else:  # host tensors: the library's host packer (exact slot counts)
            pairs, n = formats.align_row_offsets(m, alignment)
            cols = formats.pad_column_indices(m, pairs, n, shuffle8=False)
            per_layer.append((torch.from_numpy(pairs), torch.from_numpy(cols),
                              torch.from_numpy(formats.sorted_row_swizzle(m)), m.m_vec, n, _max_row(m)))
    req.dev["masks"] = per_layer


def _max_row(m) -> int:
    """Longest vector-row (nonzero vectors) of a host mask."""
    return int(np.diff(m.row_offsets).max()) if m.m_vec else 0


def _upload_csr(req: Request, device) -> None:
    """Copy a request's tokens and the plain CSR of its masks to the device
    (once); the server packs whole batches from these."""
    if req.dev:
        return
    dev = torch.device(device)
    req.dev["x"] = req.x.to(dev, non_blocking=True)
    req.dev["csr"] = [(torch.from_numpy(m.row_offsets).to(dev, non_blocking=True),
                       torch.from_numpy(m.col_indices).to(dev, non_blocking=True), m.m_vec, m.nnz_vec, _max_row(m))
                      for m in req.masks]


def pack_batch_masks(reqs: list[Request], layers: int, V: int, alignment: int, device) -> list[AttentionMaskDev]:
    """One block-diagonal attention mask per layer over the batch: the
    requests' CSRs are concatenated on the device (row offsets shifted by the
    nonzeros before them, column indices by the tokens before them) and
    packed by one device packer call per layer, rows longest first across
    the whole batch.  Each row's result is the same as in its own mask."""
    dev = torch.device(device)
    lens = [r.seq_len for r in reqs]
    tok_base = np.concatenate([[0], np.cumsum(lens)[:-1]]).astype(np.int32)
    total_tokens = int(sum(lens))
    out = []
    for l in range(layers):
        csr = [r.dev["csr"][l] for r in reqs]
        m_vecs = [c[2] for c in csr]
        nnzs = [c[3] for c in csr]
        nnz_base = np.concatenate([[0], np.cumsum(nnzs)[:-1]]).astype(np.int32)
        total_m, total_nnz = int(sum(m_vecs)), int(sum(nnzs))
        shifts = torch.from_numpy(np.stack([nnz_base, tok_base])).to(dev, non_blocking=True)
        counts = torch.from_numpy(np.array([m_vecs, nnzs], dtype=np.int64)).to(dev, non_blocking=True)
        ro = torch.cat([torch.zeros(1, dtype=torch.int32, device=dev)] + [c[0][1:] for c in csr])
        ro[1:] += torch.repeat_interleave(shifts[0], counts[0], output_size=total_m)
        ci = torch.cat([c[1] for c in csr]) if total_nnz else torch.zeros(0, dtype=torch.int32, device=dev)
        if total_nnz:
            ci += torch.repeat_interleave(shifts[1], counts[1], output_size=total_nnz)
        dm = device_format.prepare_sddmm(ro, ci, V, total_tokens, alignment=alignment, sync=False)
        out.append(AttentionMaskDev(total_m, V, total_tokens, dm.aligned_nnz, dm.row_indices, dm.row_offsets,
                                    dm.col_indices, max(c[4] for c in csr)))
    return out


def batch_masks(reqs: list[Request], layers: int, V: int) -> list[AttentionMaskDev]:
    """One block-diagonal attention mask per layer over the batch (device ops)."""
    out = []
    for l in range(layers):
        pairs, cols, ri = [], [], []
        abase = tbase = mbase = longest = 0
        for r in reqs:
            p, c, i, m_vec, n, mx = r.dev["masks"][l]
            longest = max(longest, mx)
            pairs.append(p + abase)
            cols.append(torch.where(c >= 0, c + tbase, c))
            ri.append(i + mbase)
            abase += n
            tbase += r.seq_len
            mbase += m_vec
        if abase == 0:
            cols = [torch.full((1,), -1, dtype=torch.int32, device=pairs[0].device)]
        out.append(AttentionMaskDev(mbase, V, tbase, abase, torch.cat(ri), torch.cat(pairs), torch.cat(cols),
                                    longest))
    return out


def footprint_bytes(reqs: list[Request], hidden: int, heads: int, layers: int, V: int,
                    scores_in_memory: bool = True) -> int:
    """Upper bound on the device working set of one batched forward pass,
    used for admission.  Calibrated against torch.cuda.max_memory_allocated
    on GB300 for the 2-layer encoder (hidden 256, 4 heads, requests of 256 to
    8192 tokens, alone and in batches): at most 25 bytes per token and hidden
    unit for the activations, projections and FFN intermediates; with the
    separate attention launches (`scores_in_memory`) 1.5 bytes per stored
    score of the largest layer's mask (the half scores and int8
    probabilities live while the FFN's larger intermediates do not); the
    packed masks (padded columns and pairs); then a 25 % margin.  The
    estimate stays within 1.6x of the measured peak."""
    T = sum(r.seq_len for r in reqs)
    per_layer = [sum(r.masks[l].nnz_vec for r in reqs) for l in range(layers)]
    m_vec = sum(r.seq_len // V for r in reqs)
    act = T * hidden * 26
    att = max(per_layer) * V * heads * 3 // 2 if scores_in_memory else 0
    masks = sum(per_layer) * 8 + layers * m_vec * 16
    return int(1.25 * (act + att + masks))


class ContinuousBatchingServer:
    """Admission: a new batch starts when no batch is in flight, or when the
    queued tokens reach `overlap_tokens` (then batches overlap on their own
    streams, up to `max_inflight`); otherwise queued requests wait for the
    running batch and are admitted together.  Light load therefore runs one
    request at a time (no device time-sharing between lone requests), heavy
    load batches and overlaps."""

    def __init__(self, model, hidden: int = 256, heads: int = 4, V: int = 8, rhs_bits: int = 8,
                 max_inflight: int = 3, max_batch_tokens: int = 65536, hbm_reserve: int = 2 << 30,
                 overlap_tokens: int = 8192, device="cuda"):
        self.model, self.hidden, self.heads, self.V = model, hidden, heads, V
        self.layers = len(model.layers)
        self.alignment = 16 if rhs_bits == 8 else 32
        self.max_inflight, self.max_batch_tokens, self.hbm_reserve = max_inflight, max_batch_tokens, hbm_reserve
        self.overlap_tokens = overlap_tokens
        self.device = torch.device(device)
        self.streams = [torch.cuda.Stream(device=self.device) for _ in range(max_inflight)]
        self.batches: list[list[int]] = []
        self.peak_inflight = 0        # most batches on the device at once
        self.held_back = 0            # admissions deferred because the batch did not fit the free HBM
        self.rejected: list[int] = []  # requests that cannot fit even alone on an idle device

    def footprint(self, reqs: list[Request]) -> int:
        """Working-set estimate of a batch on this server's model."""
        scores = any(getattr(layer, "attention", "separate") != "fused" for layer in self.model.layers)
        return footprint_bytes(reqs, self.hidden, self.heads, self.layers, self.V, scores_in_memory=scores)

    def _fits(self, reqs: list[Request]) -> bool:
        free, _ = torch.cuda.mem_get_info(self.device)
        return self.footprint(reqs) + self.hbm_reserve <= free

    def serve(self, requests: list[Request]) -> dict:
        pending = deque(sorted(requests, key=lambda r: r.arrival))
        queue: deque[Request] = deque()
        inflight: list[tuple[torch.cuda.Event, list[Request], int]] = []
        self.inflight = inflight
        free_streams = list(range(self.max_inflight))
        done = 0
        t0 = time.perf_counter()
        with torch.no_grad():
            while done < len(requests):
                now = time.perf_counter() - t0
                while pending and pending[0].arrival <= now:
                    r = pending.popleft()
                    queue.append(r)
                # completions
                still = []
                for ev, batch, si in inflight:
                    if ev.query():
                        tdone = time.perf_counter() - t0
                        for r in batch:
                            r.t_done = tdone
                            r.dev.clear()
                        done += len(batch)
                        free_streams.append(si)
                    else:
                        still.append((ev, batch, si))
                inflight[:] = still
                # admission of a new batch: as many queued requests as the
                # token budget and the free HBM allow.  A request that does
                # not fit even alone on an idle device is rejected instead of
                # launched; one that does not fit next to the batches in
                # flight waits for them.
                queued_tokens = sum(r.seq_len for r in queue)
                if queue and free_streams and (not inflight or queued_tokens >= self.overlap_tokens):
                    batch, tokens = [], 0
                    while queue:
                        r = queue[0]
                        if batch and tokens + r.seq_len > self.max_batch_tokens:
                            break
                        if not self._fits(batch + [r]):
                            if not batch and not inflight:
                                queue.popleft()
                                r.error = "does not fit the free device memory"
                                r.t_done = time.perf_counter() - t0
                                self.rejected.append(r.rid)
                                done += 1
                                continue
                            self.held_back += 1
                            break
                        batch.append(queue.popleft())
                        tokens += r.seq_len
                    if batch:
                        si = free_streams.pop()
                        s = self.streams[si]
                        with torch.cuda.stream(s):
                            for r in batch:
                                _upload_csr(r, self.device)
                                r.t_admit = time.perf_counter() - t0
                            masks = pack_batch_masks(batch, self.layers, self.V, self.alignment, self.device)
                            x = torch.cat([r.dev["x"] for r in batch], dim=0)
                            y = self.model(x, masks)
                            off = 0
                            for r in batch:
                                r.out = y[off:off + r.seq_len]
                                off += r.seq_len
                            ev = torch.cuda.Event()
                            ev.record(s)
                        inflight.append((ev, batch, si))
                        self.peak_inflight = max(self.peak_inflight, len(inflight))
                        self.batches.append([r.rid for r in batch])
                        continue
                if not inflight and not queue and pending:
                    time.sleep(max(0.0, min(0.001, pending[0].arrival - (time.perf_counter() - t0))))
        torch.cuda.synchronize()
        return summarize(requests, time.perf_counter() - t0)


def serve_sequential(model, requests: list[Request], V: int = 8, rhs_bits: int = 8, device="cuda") -> dict:
    """Baseline: one request at a time in arrival order, each its own forward pass."""
    alignment = 16 if rhs_bits == 8 else 32
    layers = len(model.layers)
    t0 = time.perf_counter()
    with torch.no_grad():
        for r in sorted(requests, key=lambda q: q.arrival):
            now = time.perf_counter() - t0
            if r.arrival > now:
                time.sleep(r.arrival - now)
            r.t_admit = time.perf_counter() - t0
            _upload(r, alignment, device)
            masks = batch_masks([r], layers, V)
            r.out = model(r.dev["x"], masks)
            torch.cuda.synchronize()
            r.t_done = time.perf_counter() - t0
            r.dev.clear()
    return summarize(requests, time.perf_counter() - t0)


def summarize(requests: list[Request], makespan: float) -> dict:
    """Throughput and latency percentiles over the served requests (rejected
    ones are counted apart)."""
    served = [r for r in requests if r.error is None]
    lat = np.array([r.latency for r in served]) * 1e3 if served else np.zeros(1)
    return {"requests": len(served), "rejected": len(requests) - len(served), "makespan_s": makespan,
            "req_per_s": len(served) / makespan,
            "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "mean_ms": float(lat.mean()), "tokens": int(sum(r.seq_len for r in served))}
