"""MC counting on several GPUs, one process per GPU.

The k-mer set partitions by minimizer bucket (every occurrence of a
canonical k-mer lies in a superkmer with the same minimizer, and the bucket
is a function of the minimizer), so the GPUs need one exchange and no other
communication:

1. split: every rank takes a share of the reads (cut at record boundaries);
2. route: each rank packs and scans its share on its GPU and groups the
   superkmers by destination rank = minimizer bucket mod world size
   (``mczi_route_superkmers``; the reference writes the same superkmers to
   per-partition files, src/lib.rs:4821-4925);
3. exchange: one all-to-all of the groups (sizes first, then bytes);
4. count: each rank counts the superkmers it received (``mczi_count``) and
   keeps records with count > x, exactly the records of its buckets;
5. gather (optional): the union of the ranks' records is the single-GPU
   result, record for record.

fof (presence) mode is the same plan with the dataset carried beside the
records: every rank takes a share of every dataset, routes each dataset's
share on its own, and the exchange sends a table of group sizes per
(destination, dataset) with the bytes, so the receiver rebuilds one input
per dataset and counts them in presence mode (``count_datasets_sharded``).
A k-mer's occurrences in one dataset all reach the same rank, so its
presence count there is its number of datasets, as on one GPU.

The exchange works over any ``torch.distributed`` process group: NCCL on
GPUs, gloo on the CPU (the tests run the plan with two gloo ranks and a CPU
stand-in for the routing step).
"""
from __future__ import annotations

import ctypes as C
from typing import Callable, Sequence

import numpy as np

from . import _native as N


def split_records(buf, parts: int) -> list[np.ndarray]:
    """`parts` contiguous slices of a FASTA (or four-line FASTQ) buffer, cut
    only at record starts, of about equal size."""
    a = np.frombuffer(buf, dtype=np.uint8) if not isinstance(buf, np.ndarray) else buf
    if parts <= 1 or a.size == 0:
        return [a] + [a[:0]] * max(0, parts - 1)
    if a[0] == ord("@"):
        # FASTQ: records are four lines; starts are the line starts 0, 4, 8, ...
        nl = np.flatnonzero(a == ord("\n"))
        starts = np.concatenate([[0], nl[3::4] + 1])
    else:
        starts = np.flatnonzero(a == ord(">"))
        starts = starts[(starts == 0) | (a[np.maximum(starts - 1, 0)] == ord("\n"))]
    starts = starts[starts < a.size]
    cuts = [0]
    for i in range(1, parts):
        target = a.size * i // parts
        j = int(np.searchsorted(starts, target))
        cuts.append(int(starts[j]) if j < len(starts) else a.size)
    cuts.append(a.size)
    return [a[cuts[i]:cuts[i + 1]] for i in range(parts)]


def route_superkmers(ctx, inputs: Sequence, config, world: int) -> list[np.ndarray]:
    """Step 2 on this rank's GPU: the superkmers of `inputs` as one-line FASTA
    records, one group per destination rank."""
    from .mc import _inputs_c
    lib = N.load()
    arr, keep = _inputs_c(list(inputs))
    sizes = (C.c_uint64 * world)()
    cc = config.c()
    ctx._ck(lib.mczi_route_superkmers(ctx.handle, C.byref(cc), arr, len(inputs), world, sizes))
    del keep
    out = []
    for d in range(world):
        g = np.empty(int(sizes[d]), dtype=np.uint8)
        ctx._ck(lib.mczi_route_copy(ctx.handle, d, g.ctypes.data if g.size else None, g.size))
        out.append(g)
    return out


def all_to_all_bytes(groups: Sequence[np.ndarray], group=None) -> list[np.ndarray]:
    """Step 3: rank r sends groups[d] to rank d and receives one byte array
    from every rank (sizes first, then the bytes, with all_to_all_single)."""
    import torch
    import torch.distributed as dist
    world = dist.get_world_size(group)
    backend = dist.get_backend(group)
    dev = torch.device("cuda", torch.cuda.current_device()) if backend == "nccl" else torch.device("cpu")
    send_sizes = torch.tensor([int(g.size) for g in groups], dtype=torch.int64, device=dev)
    recv_sizes = torch.empty(world, dtype=torch.int64, device=dev)
    dist.all_to_all_single(recv_sizes, send_sizes, group=group)
    ss, rs = send_sizes.tolist(), recv_sizes.tolist()
    payload = np.concatenate([np.asarray(g, dtype=np.uint8) for g in groups]) if sum(ss) else np.empty(0, np.uint8)
    send = torch.from_numpy(payload).to(dev)
    recv = torch.empty(sum(rs), dtype=torch.uint8, device=dev)
    dist.all_to_all_single(recv, send, output_split_sizes=rs, input_split_sizes=ss, group=group)
    r = recv.cpu().numpy()
    offs = np.concatenate([[0], np.cumsum(rs)]).astype(np.int64)
    return [r[offs[i]:offs[i + 1]] for i in range(world)]


def count_sharded(share: Sequence, config, group=None, ctx=None,
                  route: Callable | None = None, count: Callable | None = None):
    """Steps 2-4 on this rank: route its share of the reads, exchange, count
    the received superkmers.  Returns (lo, hi, counts) of this rank's buckets
    (hi None for k <= 32).  `route(share, world)` and `count(received)` replace
    the GPU steps (the CPU tests pass stand-ins)."""
    import torch.distributed as dist
    world = dist.get_world_size(group)
    if route is None:
        route = lambda s, w: route_superkmers(ctx, s, config, w)  # noqa: E731
    if count is None:
        def count(received):
            n = ctx.count(received, config)
            r = ctx.records(n, sorted=True)
            return r.lo, r.hi, r.count
    groups = route(share, world)
    received = [b for b in all_to_all_bytes(groups, group) if b.size]
    if not received:  # none of this rank's buckets occurs
        e = np.empty(0, dtype=np.uint64)
        return e, (e if config.k > 32 else None), e
    return count(received)


def _empty_groups(world: int) -> list[np.ndarray]:
    return [np.empty(0, dtype=np.uint8) for _ in range(world)]


def all_to_all_datasets(groups: Sequence[Sequence[np.ndarray]], group=None) -> list[np.ndarray]:
    """Step 3 in fof mode: groups[i][d] holds dataset i's records for rank d.
    One exchange of the size table (per destination, one size per dataset)
    and one of the bytes; returns, per dataset, the records this rank
    received from all ranks, concatenated."""
    import torch
    import torch.distributed as dist
    world = dist.get_world_size(group)
    n = len(groups)
    backend = dist.get_backend(group)
    dev = torch.device("cuda", torch.cuda.current_device()) if backend == "nccl" else torch.device("cpu")
    table = np.array([[int(groups[i][d].size) for i in range(n)] for d in range(world)], dtype=np.int64)
    send_tab = torch.from_numpy(table.reshape(-1).copy()).to(dev)
    recv_tab = torch.empty(world * n, dtype=torch.int64, device=dev)
    dist.all_to_all_single(recv_tab, send_tab, group=group)  # n sizes to and from every rank
    rtab = recv_tab.cpu().numpy().reshape(world, n)
    ss = [int(v) for v in table.sum(axis=1)]
    rs = [int(v) for v in rtab.sum(axis=1)]
    parts = [np.asarray(groups[i][d], dtype=np.uint8) for d in range(world) for i in range(n)]
    payload = np.concatenate(parts) if sum(ss) else np.empty(0, np.uint8)
    send = torch.from_numpy(payload).to(dev)
    recv = torch.empty(sum(rs), dtype=torch.uint8, device=dev)
    dist.all_to_all_single(recv, send, output_split_sizes=rs, input_split_sizes=ss, group=group)
    r = recv.cpu().numpy()
    per = [[] for _ in range(n)]
    off = 0
    for src in range(world):
        for i in range(n):
            ln = int(rtab[src, i])
            if ln:
                per[i].append(r[off:off + ln])
            off += ln
    return [np.concatenate(p) if p else np.empty(0, np.uint8) for p in per]


def count_datasets_sharded(shares: Sequence[Sequence], config, group=None, ctx=None,
                           route: Callable | None = None, count: Callable | None = None):
    """fof mode, steps 2-4 on this rank: shares[i] is this rank's share of
    dataset i (a list of buffers, possibly empty).  Each dataset's share is
    routed on its own; after the exchange this rank counts, in presence mode,
    one input per dataset that sent it records (a dataset with none here
    holds none of this rank's k-mers, so leaving it out changes no count).
    Returns (lo, hi, counts) of this rank's buckets (hi None for k <= 32).
    `route(share, world)` and `count(received_datasets)` replace the GPU
    steps (the CPU tests pass stand-ins)."""
    import torch.distributed as dist
    world = dist.get_world_size(group)
    if route is None:
        route = lambda s, w: route_superkmers(ctx, s, config, w)  # noqa: E731
    if count is None:
        def count(received):
            n = ctx.count(received, config, N.MODE_PRESENCE)
            r = ctx.records(n, sorted=True)
            return r.lo, r.hi, r.count
    groups = [route(list(share), world) if sum(len(b) for b in share) else _empty_groups(world) for share in shares]
    received = [b for b in all_to_all_datasets(groups, group) if b.size]
    if not received:
        e = np.empty(0, dtype=np.uint64)
        return e, (e if config.k > 32 else None), e
    return count(received)


def gather_records(lo, hi, cnt, group=None):
    """Step 5: every rank's records at rank 0, concatenated and sorted by
    canonical k-mer (other ranks get None)."""
    import torch.distributed as dist
    world = dist.get_world_size(group)
    parts = [None] * world
    dist.all_gather_object(parts, (lo, hi, cnt), group=group)
    if dist.get_rank(group) != 0:
        return None
    lo = np.concatenate([p[0] for p in parts]).astype(np.uint64)
    cnt = np.concatenate([p[2] for p in parts]).astype(np.uint64)
    if parts[0][1] is None:
        order = np.argsort(lo, kind="stable")
        return lo[order], None, cnt[order]
    hi = np.concatenate([p[1] for p in parts]).astype(np.uint64)
    order = np.lexsort((lo, hi))
    return lo[order], hi[order], cnt[order]
