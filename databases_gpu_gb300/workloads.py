"""Seeded synthetic workloads with the shapes of the reference's benchmark
configurations (its datasets are not shipped; these stand in for them).

ResizeStream -- the dynamic resize stream: u64 keys / u64 values, batches of
mixed ops that first grow the table (60% insert / 30% find / 10% erase) and
then shrink it back (10% / 30% / 60%), with a share of in-batch duplicate keys
resolved by the batch-order rules. The live key set is always a window
[lo, hi) of a counter-indexed key sequence, so every batch's expected table
size, find hits and erase count are known exactly without a host-side map.

Keys are splitmix64 of a counter (a bijection, so distinct); keys that no
batch ever inserts come from counters at and above 2^40.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

_GOLD = 0x9E3779B97F4A7C15
_C1 = 0xBF58476D1CE4E5B9
_C2 = 0x94D049BB133111EB
_MISS_BASE = 1 << 40


def _s64(x: int) -> int:
    """The signed int64 with the same 64 bits as x."""
    x &= (1 << 64) - 1
    return x - (1 << 64) if x >> 63 else x


def _lsr(z, s: int):
    return (z >> s) & ((1 << (64 - s)) - 1)


def splitmix64(idx, seed: int):
    """splitmix64 finalizer of (idx + seed * golden) * golden, on int64 tensors
    (wrapping arithmetic; the bits are the uint64 result)."""
    z = (idx + _s64(seed * _GOLD)) * _s64(_GOLD)
    z = (z ^ _lsr(z, 30)) * _s64(_C1)
    z = (z ^ _lsr(z, 27)) * _s64(_C2)
    return z ^ _lsr(z, 31)


@dataclass
class StreamBatch:
    ops: object        # uint8 tensor
    keys: object       # int64 tensor (uint64 bits)
    vals: object       # int64 tensor
    size_after: int    # live keys after the batch
    find_ops: int      # finds in the batch (every one hits)
    erase_hits: int    # keys the batch's erases remove
    phase: str


class ResizeStream:
    """Grow batches then shrink batches over a key window.

    batch_ops    ops per batch (2^22 at full size)
    grow, shrink number of batches in each phase (256 + 256 at full size)
    start, peak  live keys before the first batch / after the grow phase
                 (2^20 and 2^27 at full size)
    dup          share of ops that repeat another op's key in the same batch
    """

    def __init__(self, batch_ops: int, grow: int, shrink: int, start: int, peak: int,
                 dup: float = 0.05, seed: int = 10327, device="cuda"):
        import torch
        self.torch = torch
        self.B, self.grow, self.shrink = batch_ops, grow, shrink
        self.start, self.peak, self.dup = start, peak, dup
        self.seed = seed
        self.device = torch.device(device)
        self.gen = torch.Generator(device=self.device)
        self.gen.manual_seed(seed)
        self.lo, self.hi = 0, start
        self.b = 0

    def key(self, idx):
        return splitmix64(idx, self.seed)

    def preload(self):
        """Keys and values of the initial window [0, start)."""
        t = self.torch
        idx = t.arange(0, self.start, dtype=t.int64, device=self.device)
        k = self.key(idx)
        assert not bool((k == 0).any())
        return k, self._vals(self.start)

    def _vals(self, n):
        t = self.torch
        return t.randint(0, 1 << 62, (n,), generator=self.gen, device=self.device, dtype=t.int64)

    def _rand_idx(self, n, lo, hi):
        t = self.torch
        return t.randint(lo, hi, (n,), generator=self.gen, device=self.device, dtype=t.int64)

    def __len__(self):
        return self.grow + self.shrink

    def next(self) -> StreamBatch:
        t = self.torch
        B = self.B
        growing = self.b < self.grow
        phase_b = self.b if growing else self.b - self.grow
        n_phase = self.grow if growing else self.shrink
        # net change this batch: spread (peak - start) evenly over the phase
        total = self.peak - self.start
        net = total * (phase_b + 1) // n_phase - total * phase_b // n_phase
        n_dup = int(round(self.dup * B))
        if growing:
            ins = int(round(0.6 * B))
            fnd = int(round(0.3 * B))
            dele = B - ins - fnd
            fresh = dele + net
            upd = ins - fresh
            assert 0 <= fresh and upd > n_dup, "batch too small for this growth rate"
            d_hit = dele
        else:
            ins = int(round(0.1 * B))
            fnd = int(round(0.3 * B))
            dele = B - ins - fnd
            fresh = ins
            upd = 0
            d_hit = fresh + net
            assert d_hit + n_dup <= dele, "batch too small for this shrink rate"
        lo, hi = self.lo, self.hi
        keep_lo = lo + d_hit  # keys [lo, keep_lo) are erased by this batch
        assert keep_lo < hi
        parts_k, parts_o = [], []
        # fresh inserts
        parts_k.append(t.arange(hi, hi + fresh, dtype=t.int64, device=self.device))
        parts_o.append(1)
        if growing:
            # updates of surviving keys; n_dup of them repeat another update's key
            u = self._rand_idx(upd - n_dup, keep_lo, hi)
            parts_k.append(u)
            parts_o.append(1)
            parts_k.append(u[self._rand_idx(n_dup, 0, u.numel())])
            parts_o.append(1)
            parts_k.append(t.arange(lo, keep_lo, dtype=t.int64, device=self.device))
            parts_o.append(2)
        else:
            e = t.arange(lo, keep_lo, dtype=t.int64, device=self.device)
            parts_k.append(e)
            parts_o.append(2)
            # repeated erases of keys this batch erases (the later one misses)
            parts_k.append(e[self._rand_idx(n_dup, 0, e.numel())])
            parts_o.append(2)
            miss = dele - d_hit - n_dup
            parts_k.append(self._rand_idx(miss, _MISS_BASE, _MISS_BASE + (1 << 40)))
            parts_o.append(2)
        parts_k.append(self._rand_idx(fnd, keep_lo, hi))
        parts_o.append(0)
        idx = t.cat(parts_k)
        ops = t.cat([t.full((p.numel(),), o, dtype=t.uint8, device=self.device)
                     for p, o in zip(parts_k, parts_o)])
        assert idx.numel() == B
        perm = t.randperm(B, generator=self.gen, device=self.device)
        idx, ops = idx[perm], ops[perm]
        keys = self.key(idx)
        vals = self._vals(B)
        self.lo, self.hi = keep_lo, hi + fresh
        self.b += 1
        return StreamBatch(ops.contiguous(), keys.contiguous(), vals, self.hi - self.lo, fnd,
                           d_hit, "grow" if growing else "shrink")


_M32 = 0xFFFFFFFF


def perm32(x):
    """A bijection of the 32-bit integers (odd multiplies and xorshifts), on
    int64 tensors holding values in [0, 2^32)."""
    x = (x ^ 0x5BD1E995) & _M32
    x = (x * 0x9E3779B1) & _M32
    x = x ^ (x >> 16)
    x = (x * 0x85EBCA6B) & _M32
    x = x ^ (x >> 13)
    x = (x * 0xC2B2AE35) & _M32
    return x ^ (x >> 16)


class MultiTableWorkload:
    """Many independent u32/u32 tables of log-uniform sizes, each receiving a
    mixed batch of log-uniform size per round.

    Table t's key of index j is perm32((j + t * 0x9E3779B9) mod 2^32) (distinct
    within a table; 0 is replaced by 2^32 - 1). It starts with indices
    [0, size_t). A round's ops for table t: `find` share (half on indices in
    [0, size_t), half on indices from 2^31, never inserted), `insert` share on
    indices in [0, 2 size_t) (about half update, half add), the rest erases on
    indices in [0, size_t). Everything is generated on the device.
    """

    def __init__(self, ntables: int, log2_size=(8, 20), log2_batch=(4, 16),
                 mix=(0.7, 0.2, 0.1), seed: int = 10327, device="cuda"):
        import torch
        self.torch = torch
        self.device = torch.device(device)
        self.gen = torch.Generator(device="cpu")
        self.gen.manual_seed(seed)
        self.dgen = torch.Generator(device=self.device)
        self.dgen.manual_seed(seed + 1)
        self.ntables = ntables
        u = torch.rand(ntables, generator=self.gen, dtype=torch.float64)
        self.sizes = torch.round(2.0 ** (log2_size[0] + u * (log2_size[1] - log2_size[0]))).long()
        u = torch.rand(ntables, generator=self.gen, dtype=torch.float64)
        self.batch = torch.round(2.0 ** (log2_batch[0] + u * (log2_batch[1] - log2_batch[0]))).long()
        self.mix = mix
        off = torch.zeros(ntables + 1, dtype=torch.int64)
        off[1:] = torch.cumsum(self.batch, 0)
        self.offsets_host = off.numpy().astype(np.uint32)
        self.offsets = torch.from_numpy(self.offsets_host.view(np.int32)).to(self.device)
        self.n_ops = int(off[-1])
        self._tid = torch.repeat_interleave(torch.arange(ntables, device=self.device),
                                            self.batch.to(self.device))
        self._size_dev = self.sizes.to(self.device)

    def key(self, t, j):
        """Keys of table t (int64 tensors), as int32 tensors (same 32 bits)."""
        k = perm32((j + t * 0x9E3779B9) & _M32)
        k = self.torch.where(k == 0, self.torch.full_like(k, _M32), k)
        return (k - ((k >> 31) << 32)).to(self.torch.int32)

    def preload(self, t: int):
        """Keys and values table t starts with (int32 CUDA tensors)."""
        torch = self.torch
        n = int(self.sizes[t])
        j = torch.arange(n, dtype=torch.int64, device=self.device)
        tt = torch.full_like(j, t)
        vals = (perm32(j ^ (tt << 20)) & 0x7FFFFFFF).to(torch.int32)
        return self.key(tt, j), vals

    def round(self):
        """One round: (ops uint8, keys int32, vals int32) over all tables, in
        table order (ranges given by self.offsets)."""
        torch = self.torch
        n = self.n_ops
        t = self._tid
        size = self._size_dev[t]
        u = torch.rand(n, generator=self.dgen, device=self.device)
        f, i = self.mix[0], self.mix[1]
        ops = torch.where(u < f, 0, torch.where(u < f + i, 1, 2)).to(torch.uint8)
        r = torch.rand(n, generator=self.dgen, device=self.device, dtype=torch.float64)
        hit = torch.rand(n, generator=self.dgen, device=self.device) < 0.5
        j_present = (r * size).long()
        j_insert = (r * 2 * size).long()
        j_miss = (1 << 31) + (r * (1 << 30)).long()
        j = torch.where(ops == 1, j_insert,
                        torch.where((ops == 0) & ~hit, j_miss, j_present))
        keys = self.key(t, j)
        vals = torch.randint(0, 1 << 31, (n,), generator=self.dgen, device=self.device,
                             dtype=torch.int64).to(torch.int32)
        return ops.contiguous(), keys.contiguous(), vals.contiguous()
