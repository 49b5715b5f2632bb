"""Sharding of a scan over ranks (one process per GPU): range and object
partitioning, and a world_size-2 gloo run on CPU in which each rank scans
its period range (with the oracle standing in for a rank's GPU) and the
gathered rows equal the single-process scan."""
from __future__ import annotations

import multiprocessing as mp
import socket

import numpy as np
import pytest

from conftest import GOLDEN


def test_period_shards_cover_the_range():
    from periodsearch_gb300.shard import period_shards

    for n_lo, n_hi, world in [(1, 40000, 8), (5, 17, 3), (1, 1, 4), (1, 7, 7), (3, 2, 2)]:
        sh = period_shards(n_lo, n_hi, world)
        assert len(sh) == world and sh[0][0] == n_lo
        for (a, b), (c, _) in zip(sh, sh[1:]):
            assert c == b + 1                                   # contiguous, in rank order
        assert sh[-1][1] == n_hi
        sizes = [b - a + 1 for a, b in sh]
        assert max(sizes) - min(sizes) <= 1 and min(sizes) >= 0
    with pytest.raises(ValueError):
        period_shards(1, 10, 0)


def test_object_shards_balance():
    from periodsearch_gb300.shard import object_shards

    rng = np.random.default_rng(3)
    costs = np.exp(rng.uniform(np.log(100), np.log(5000), 512)) * 1e4     # logU[100, 5000] Ndata x 1e4 periods
    sh = object_shards(costs, 8)
    assert sorted(i for s in sh for i in s) == list(range(512))
    loads = [costs[s].sum() for s in sh]
    assert max(loads) / min(loads) < 1.01
    assert object_shards(costs, 8) == sh                         # deterministic
    assert object_shards([5.0, 1.0, 1.0, 1.0, 1.0, 1.0], 2) == [[0], [1, 2, 3, 4, 5]]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, path, n_lo, n_hi, q):
    import sys

    sys.path.insert(0, str(GOLDEN.parent))
    try:
        import torch.distributed as dist

        import oracle_binding
        from periodsearch_gb300.shard import scan_sharded

        dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
        ora = oracle_binding.OracleProblem(path)
        conw_r, _ = ora.precalc_conw()                  # every rank runs the pre-pass: same conw_r
        ora.setup(conw_r)
        calls = []

        def scan(lo, hi):
            calls.append((lo, hi))
            return ora.scan(conw_r, lo, hi)

        rows, best = scan_sharded(scan, n_lo, n_hi)
        q.put((rank, calls, rows, best, conw_r))
        dist.destroy_process_group()
    except Exception as e:          # reported to the parent
        q.put((rank, repr(e), None, None, None))


def _run(world, path, n_lo, n_hi):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank_main, args=(r, world, port, str(path), n_lo, n_hi, q)) for r in range(world)]
    for p in ps:
        p.start()
    res = {}
    for _ in ps:
        rank, calls, rows, best, cw = q.get(timeout=300)
        res[rank] = (calls, rows, best, cw)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    return res


@pytest.mark.parametrize("case,n_lo,n_hi", [("tiny_cal", 1, 14), ("tiny_mix", 2, 3)])
def test_gloo_two_ranks_match_single_scan(oracle, case, n_lo, n_hi):
    path = GOLDEN / case / "period_search_in"
    res = _run(2, path, n_lo, n_hi)
    for r, (calls, rows, best, cw) in res.items():
        assert not isinstance(calls, str), calls
    (c0, rows0, best0, cw0), (c1, rows1, best1, cw1) = res[0], res[1]
    assert cw0 == cw1
    assert c0 and c1 and c0[0][0] == n_lo and c1[-1][1] == n_hi and c1[0][0] == c0[-1][1] + 1
    np.testing.assert_array_equal(rows0, rows1)            # every rank holds the gathered rows
    ora = oracle.OracleProblem(path)
    conw_r, _ = ora.precalc_conw()
    ora.setup(conw_r)
    single = ora.scan(conw_r, n_lo, n_hi)
    np.testing.assert_array_equal(rows0, single)
    assert best0 == best1 == n_lo + int(np.argmin(single["rms"]))


def test_gloo_rank_with_empty_range(oracle):
    """More ranks than periods: a rank scans nothing and still joins the gather."""
    path = GOLDEN / "tiny_cal" / "period_search_in"
    res = _run(2, path, 4, 4)
    assert res[0][0] == [(4, 4)] and res[1][0] == []
    assert len(res[1][1]) == 1 and res[0][2] == res[1][2] == 4


def _synthetic_rows(n, best):
    """Rows whose minimum lies at index best, with a near tie four periods
    away, and a refit that lowers every row by a period-dependent amount."""
    from periodsearch_gb300 import ROW_DTYPE

    rows = np.zeros(n, ROW_DTYPE)
    k = np.arange(n)
    rows["rms"] = 0.1 + 0.001 * np.abs(k - best) + 0.0002 * np.sin(k)
    rows["rms"][best + 4] = rows["rms"][best] * 1.004
    rows["period_h"] = 5.0 + 0.01 * k
    return rows


def _refit_rows(n_lo, base):
    def refit(per):
        out = base[np.asarray(per) - n_lo].copy()
        out["rms"] -= 1e-4 * (np.asarray(per) % 7)
        out["chi2"] = 1.0
        return out
    return refit


def _refine_rank(rank, world, port, n_lo, rows, q):
    try:
        import torch.distributed as dist

        from periodsearch_gb300.shard import refine_sharded

        dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
        calls = []
        base = _refit_rows(n_lo, rows)

        def refit(per):
            calls.append(list(per))
            return base(per)

        out, best, nref = refine_sharded(rows, refit, n_lo, rel=0.005, halfwidth=2)
        q.put((rank, calls, out, best, nref))
        dist.destroy_process_group()
    except Exception as e:          # reported to the parent
        q.put((rank, repr(e), None, None, None))


def test_gloo_refine_across_range_boundary():
    """The FP64 refit of the minimum region runs on the gathered rows: with
    the best period right at the boundary between two ranks' ranges, its
    neighbours on the other rank's side are refitted too, and the two ranks'
    result equals one process's."""
    from periodsearch_gb300.shard import period_shards, refine_sharded

    n_lo, n = 11, 20
    lo1 = period_shards(n_lo, n_lo + n - 1, 2)[1][0]
    best = lo1 - n_lo - 1                    # last period of rank 0's range
    rows = _synthetic_rows(n, best)
    want, want_best, want_n = refine_sharded(rows, _refit_rows(n_lo, rows), n_lo, rel=0.005, halfwidth=2)
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_refine_rank, args=(r, 2, port, n_lo, rows, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = {}
    for _ in ps:
        rank, calls, out, b, nref = q.get(timeout=300)
        assert not isinstance(calls, str), calls
        res[rank] = (calls, out, b, nref)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    refitted = sorted(i for r in res.values() for c in r[0] for i in c)
    assert refitted == sorted(set(refitted))                    # every period refitted once
    for k in (1, 2):
        assert n_lo + best + k in refitted                      # across the boundary (rank 1's range)
        assert n_lo + best - k in refitted
    assert all(i >= lo1 for c in res[1][0] for i in c) and all(i < lo1 for c in res[0][0] for i in c)
    for calls, out, b, nref in res.values():
        np.testing.assert_array_equal(out, want)
        assert b == want_best and nref == want_n
