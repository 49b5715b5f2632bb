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

With ``refine`` the minimum region is refitted with the plain FP64 form
over the GATHERED rows (``refine_sharded``), the rule of ps_scan_refined
applied to the whole range: every rank knows every row after the gather, so
all ranks compute the same refit set (the periods within ``refit_rel`` of
the global best row and the +-``refit_halfwidth`` periods around it, also
across range boundaries); each rank refits the part of the set in its own
range, the refitted rows are gathered, and the rounds repeat until the set
is closed.  The only exchanges are these host-side gathers.

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


def refine_sharded(rows: np.ndarray, refit: Callable[[list], np.ndarray], n_lo: int, rel: float = 0.01,
                   halfwidth: int = 2, group=None, max_rounds: int = 64):
    """FP64 refit of the minimum region of gathered rows (every rank holds
    the same rows).  Each round computes the refit set of the whole range --
    the periods not yet refitted whose row lies within ``rel`` of the best
    row, or within ``halfwidth`` periods of it -- refits this rank's share
    with ``refit(period_indices) -> rows`` and gathers the refitted rows.
    Returns (rows, index of the best period, periods refitted)."""
    import torch.distributed as dist

    if dist.is_available() and dist.is_initialized():
        rank, world = dist.get_rank(group), dist.get_world_size(group)
    else:
        rank, world = 0, 1
    rows = rows.copy()
    n = len(rows)
    shards = period_shards(n_lo, n_lo + n - 1, world)
    lo, hi = shards[rank]
    done = np.zeros(n, bool)
    for _ in range(max_rounds):
        best = int(np.argmin(rows["rms"]))
        lim = rows["rms"][best] * (1 + rel)
        idx = np.arange(n)
        want = ~done & ((np.abs(idx - best) <= halfwidth) | (rows["rms"] <= lim))
        if not want.any():
            break
        mine = [n_lo + int(i) for i in np.flatnonzero(want) if lo <= n_lo + i <= hi]
        local = (mine, refit(mine) if mine else None)
        if world > 1:
            parts = [None] * world
            dist.all_gather_object(parts, local, group=group)
        else:
            parts = [local]
        for per, new_rows in parts:
            if per:
                rows[np.asarray(per) - n_lo] = new_rows
        done |= want
    return rows, n_lo + int(np.argmin(rows["rms"])), int(done.sum())


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description="sharded period scan, one process per GPU")
    ap.add_argument("input")
    ap.add_argument("output")
    ap.add_argument("--form", choices=("fp64", "mixed"), default="fp64")
    ap.add_argument("--refine", action="store_true",
                    help="FP64 refit of the minimum region of the gathered rows (refine_sharded)")
    ap.add_argument("--backend", choices=("nccl", "gloo"), default=None,
                    help="process group backend (default: nccl with GPUs, else gloo)")
    args = ap.parse_args(argv)
    import torch
    import torch.distributed as dist

    from . import Engine, PS_FORM_FP64, PS_FORM_MIXED, build, format_row, read_input

    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        dist.init_process_group(args.backend or ("nccl" if torch.cuda.is_available() else "gloo"))
    build.build()
    form = PS_FORM_MIXED if args.form == "mixed" else PS_FORM_FP64
    data = read_input(args.input)
    with Engine(data, device=local_rank, form=form) as eng:
        conw_r, _ = eng.precalc_conw()          # deterministic: the same on every rank
        rows, best = scan_sharded(lambda lo, hi: eng.scan(conw_r, lo, hi), 1, int(eng.info.n_max))
        if args.refine and form != PS_FORM_FP64:
            with Engine(data, device=local_rank, form=PS_FORM_FP64) as eng64:
                rows, best, _ = refine_sharded(rows, lambda per: eng64.rows_of_periods(conw_r, per), 1)
    if int(os.environ.get("RANK", "0")) == 0:
        with open(args.output, "w") as f:
            f.writelines(format_row(r) for r in rows)
        print("rows %d best period index %d (%.8f h)" % (len(rows), best, rows["period_h"][best - 1]))
    if world > 1:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
