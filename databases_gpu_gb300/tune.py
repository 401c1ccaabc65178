"""Autotuner for table sets.

A set serves tables of very different sizes with one launch sequence; the
parameters that serve a 2^8-key table best need not serve a 2^20-key one. For
each table-size class (floor(log2 keys)) the tuner builds a table of that
size, feeds it the class's own mixed workload (the batch size seen for the
class, 70 % find / 20 % insert / 10 % erase, half the finds on present keys)
through dyc_apply, and times every candidate of the search space:

    bucket_bytes   32 / 64 / 128 (the probe group width: bucket_bytes / 32 lanes)
    num_subtables  2 / 3 / 4 ...
    max_evictions  eviction bound

The fastest candidate wins; candidates within `tie` of it are decided by the
table's device bytes. A set uses one bucket size (its kernels are compiled
per bucket size), so `plan_set` takes the bucket size that wins for most of
the set's ops and, with it, each class's best subtable count and eviction
bound; `tune_launch` then picks the set's blocks-per-SM cap by timing whole
rounds. A class is tuned on one table in isolation, which is not how a set
round runs, so `validate` finally runs the tuned set and an untuned one on
the same held-out rounds and keeps the plan only if it wins. Everything runs
through the public API, on the device given.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

DEFAULT_SPACE = {"bucket_bytes": (64, 128), "num_subtables": (2, 3, 4),
                 "max_evictions": (16, 64, 256)}


def size_class(n: int) -> int:
    return max(0, int(n).bit_length() - 1)


@dataclass
class ClassResult:
    log2_size: int
    batch: int
    best: dict                      # winning parameters
    mops: float                     # its throughput on the class workload
    by_bucket: dict = field(default_factory=dict)  # bucket_bytes -> (params, mops)
    candidates: list = field(default_factory=list)


def _class_workload(torch, size, batch, rounds, seed, dev):
    from .workloads import perm32
    g = torch.Generator(device=dev)
    g.manual_seed(seed)
    idx = torch.arange(size, dtype=torch.int64, device=dev)
    pre_k = perm32(idx + 1)
    pre_v = (perm32(idx + 7) & 0x7FFFFFFF)
    out = []
    for _ in range(rounds):
        u = torch.rand(batch, generator=g, device=dev)
        ops = torch.where(u < 0.7, 0, torch.where(u < 0.9, 1, 2)).to(torch.uint8)
        hi = torch.where((ops == 0) & (torch.rand(batch, generator=g, device=dev) < 0.5),
                         size * 4, 0)
        j = (torch.rand(batch, generator=g, device=dev, dtype=torch.float64) *
             torch.where(ops == 1, 2 * size, size)).long() + hi
        k = perm32(j + 1)
        v = torch.randint(0, 1 << 31, (batch,), generator=g, device=dev, dtype=torch.int64)
        out.append((ops, _i32(torch, k), v.to(torch.int32)))
    return _i32(torch, pre_k), pre_v.to(torch.int32), out


def _i32(torch, k):
    return (k - ((k >> 31) << 32)).to(torch.int32)


def tune_class(log2_size: int, batch: int, space: dict | None = None, rounds: int = 4,
               tie: float = 0.03, seed: int = 10327, device: int = 0) -> ClassResult:
    """Time every candidate of `space` on a 2^log2_size-key u32 table fed
    batches of `batch` mixed ops (the first round is a warm-up)."""
    import torch

    from .table import DyCuckoo
    space = space or DEFAULT_SPACE
    dev = torch.device("cuda", device)
    size = 1 << log2_size
    pre_k, pre_v, work = _class_workload(torch, size, max(1, batch), rounds, seed + log2_size, dev)
    stream = torch.cuda.current_stream(dev)
    cands = []
    for sb in space["bucket_bytes"]:
        for d in space["num_subtables"]:
            for ev in space["max_evictions"]:
                t = DyCuckoo(size, bucket_bytes=sb, num_subtables=d, max_evictions=ev,
                             device=device)
                t.insert(pre_k, pre_v, unique=True, new_keys=True)
                times = []
                for r, (ops, k, v) in enumerate(work):
                    e0 = torch.cuda.Event(enable_timing=True)
                    e1 = torch.cuda.Event(enable_timing=True)
                    torch.cuda.synchronize(dev)
                    e0.record(stream)
                    t.apply(ops, k, v, stream=stream)
                    e1.record(stream)
                    torch.cuda.synchronize(dev)
                    if r:
                        times.append(e0.elapsed_time(e1))
                slot = 8
                nbytes = t.capacity * slot * sb // (sb - (slot if sb == 128 else 0))
                ms = float(np.median(times))
                cands.append({"bucket_bytes": sb, "num_subtables": d, "max_evictions": ev,
                              "ms": round(ms, 4), "mops": round(batch / ms / 1e3, 1),
                              "bytes": int(nbytes)})
                t.close()

    def pick(cs):
        fastest = min(c["ms"] for c in cs)
        near = [c for c in cs if c["ms"] <= fastest * (1 + tie)]
        return min(near, key=lambda c: (c["bytes"], c["ms"]))

    best = pick(cands)
    by_bucket = {}
    for sb in space["bucket_bytes"]:
        b = pick([c for c in cands if c["bucket_bytes"] == sb])
        by_bucket[sb] = ({k: b[k] for k in ("bucket_bytes", "num_subtables", "max_evictions")},
                         b["mops"])
    return ClassResult(log2_size, batch,
                       {k: best[k] for k in ("bucket_bytes", "num_subtables", "max_evictions")},
                       best["mops"], by_bucket, cands)


def tune_classes(sizes, batches, space=None, **kw) -> dict:
    """One ClassResult per size class present in `sizes`, each tuned at the
    mean batch size of its tables."""
    sizes = np.asarray(sizes)
    batches = np.asarray(batches)
    cls = np.array([size_class(s) for s in sizes])
    out = {}
    for c in sorted(set(cls.tolist())):
        b = int(round(float(np.mean(batches[cls == c]))))
        out[c] = tune_class(c, b, space, **kw)
    return out


def plan_set(sizes, batches, results: dict):
    """(bucket_bytes, per-table num_subtables, per-table max_evictions) for a
    set: the bucket size whose class winners carry the most ops, then each
    class's best parameters at that bucket size."""
    sizes = np.asarray(sizes)
    batches = np.asarray(batches)
    cls = np.array([size_class(s) for s in sizes])
    weight = {}
    for c, r in results.items():
        ops = float(batches[cls == c].sum())
        weight[r.best["bucket_bytes"]] = weight.get(r.best["bucket_bytes"], 0.0) + ops
    sb = max(weight, key=weight.get)
    d = np.array([results[c].by_bucket[sb][0]["num_subtables"] for c in cls], np.uint32)
    ev = np.array([results[c].by_bucket[sb][0]["max_evictions"] for c in cls], np.uint32)
    return sb, d, ev


def tune_launch(run_round, caps=(0, 2, 4, 8), repeats: int = 2, margin: float = 0.03) -> int:
    """The blocks-per-SM cap (0: as many as fit) with the shortest round;
    run_round(cap) runs one round with that cap and returns its time. A cap
    is taken over the uncapped launches only when it is faster by more than
    `margin` (round times vary by a few percent, and the random-access
    kernels are sized for uncapped grids)."""
    times = {cap: min(run_round(cap) for _ in range(repeats)) for cap in caps}
    best = min(times, key=times.get)
    if 0 in times and times[best] > times[0] * (1.0 - margin):
        return 0
    return best


def validate(run_plan, run_base, rounds: int = 4, margin: float = 0.03):
    """Held-out A/B of a tuned set against the untuned one: run_plan(i) and
    run_base(i) run held-out round i (the same ops for both) on their set and
    return its time; they alternate, so drifting clocks hit both. The plan is
    kept only when its median round is faster than the untuned median by
    more than `margin`. Returns (kept, plan_ms, base_ms)."""
    plan, base = [], []
    for i in range(rounds):
        plan.append(run_plan(i))
        base.append(run_base(i))
    pm, bm = float(np.median(plan)), float(np.median(base))
    return pm < bm * (1.0 - margin), pm, bm
