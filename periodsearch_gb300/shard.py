"""Multi-GPU scans: one process per GPU, periods (or objects) sharded with
no data-path collective.

Periods are independent once the convexity weight is fixed
(period_search/period_search_BOINC.cpp:807-945), so a scan of [1, n_max]
splits into contiguous period ranges, one per rank.  Every rank runs the
deterministic convexity pre-pass itself (same conw_r everywhere), scans its
range and the rows are gathered on the host in index order; the best period
is the argmin of the concatenated rms column.  The only exchange is that
host-side gather of the rows (``torch.distributed.all_gather_object``; gloo
or NCCL process group), after the GPU work.

With ``refine`` every rank refits the minimum region of its own range with
the FP64 form (ps_scan_refined).  The global best row is some rank's local
best, and every row within ``refit_rel`` of the global best lies within
``refit_rel`` of its own range's best, so the union of the local refits
covers the global refit set except the +-``refit_halfwidth`` neighbours that
fall across a range boundary.

Objects of a multi-object run (many small work units) are balanced by
Ndata x periods with a longest-first greedy assignment.

    torchrun --nproc-per-node 8 --master-addr 127.0.0.1 -m periodsearch_gb300.shard \\
        period_search_in period_search_out [--form mixed] [--refine]
"""
from __future__ import annotations

import argparse
import heapq
import os
from typing import Callable, Sequence

import numpy as np


def period_shards(n_lo: int, n_hi: int, world: int) -> list[tuple[int, int]]:
    """Contiguous, balanced period ranges [lo, hi] (inclusive) per rank.  A
    rank gets an empty range (lo > hi) when there are fewer periods than
    ranks."""
    if world < 1 or n_hi < n_lo - 1:
        raise ValueError("bad shard request")
    n = n_hi - n_lo + 1
    base, extra = divmod(n, world)
    out, lo = [], n_lo
    for r in range(world):
        cnt = base + (1 if r < extra else 0)
        out.append((lo, lo + cnt - 1))
        lo += cnt
    return out


def object_shards(costs: Sequence[float], world: int) -> list[list[int]]:
    """Object ids per rank, balanced by cost (Ndata x periods): longest
    first, each to the least-loaded rank (ties: lowest rank)."""
    heap = [(0.0, r) for r in range(world)]
    out: list[list[int]] = [[] for _ in range(world)]
    for i in sorted(range(len(costs)), key=lambda i: (-costs[i], i)):
        load, r = heapq.heappop(heap)
        out[r].append(i)
        heapq.heappush(heap, (load + float(costs[i]), r))
    return [sorted(o) for o in out]


def gather_rows(local_rows: np.ndarray, group=None) -> np.ndarray:
    """Concatenates every rank's rows in rank order (host-side gather)."""
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()):
        return local_rows
    parts = [None] * dist.get_world_size(group)
    dist.all_gather_object(parts, local_rows, group=group)
    return np.concatenate(parts)


def scan_sharded(scan: Callable[[int, int], np.ndarray], n_lo: int, n_hi: int, group=None):
    """Scans this rank's share of [n_lo, n_hi] with scan(lo, hi) and gathers
    the rows of all ranks.  Returns (rows of the whole range, index of the
    best period)."""
    import torch.distributed as dist

    if dist.is_available() and dist.is_initialized():
        rank, world = dist.get_rank(group), dist.get_world_size(group)
    else:
        rank, world = 0, 1
    lo, hi = period_shards(n_lo, n_hi, world)[rank]
    if hi >= lo:
        local = scan(lo, hi)
    else:
        from . import ROW_DTYPE

        local = np.zeros(0, ROW_DTYPE)
    rows = gather_rows(local, group)
    if len(rows) != n_hi - n_lo + 1:
        raise RuntimeError("gathered %d rows for %d periods" % (len(rows), n_hi - n_lo + 1))
    return rows, n_lo + int(np.argmin(rows["rms"]))


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description="sharded period scan, one process per GPU")
    ap.add_argument("input")
    ap.add_argument("output")
    ap.add_argument("--form", choices=("fp64", "mixed"), default="fp64")
    ap.add_argument("--refine", action="store_true", help="FP64 refit of each range's minimum region")
    args = ap.parse_args(argv)
    import torch
    import torch.distributed as dist

    from . import Engine, PS_FORM_FP64, PS_FORM_MIXED, build, format_row, read_input

    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    build.build()
    form = PS_FORM_MIXED if args.form == "mixed" else PS_FORM_FP64
    with Engine(read_input(args.input), device=local_rank, form=form) as eng:
        conw_r, _ = eng.precalc_conw()          # deterministic: the same on every rank
        if args.refine:
            fn = lambda lo, hi: eng.scan_refined(conw_r, lo, hi)[0]   # noqa: E731
        else:
            fn = lambda lo, hi: eng.scan(conw_r, lo, hi)              # noqa: E731
        rows, best = scan_sharded(fn, 1, int(eng.info.n_max))
    if int(os.environ.get("RANK", "0")) == 0:
        with open(args.output, "w") as f:
            f.writelines(format_row(r) for r in rows)
        print("rows %d best period index %d (%.8f h)" % (len(rows), best, rows["period_h"][best - 1]))
    if world > 1:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
