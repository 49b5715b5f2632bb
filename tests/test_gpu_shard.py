"""The sharded scan through the engine: two ranks (gloo process group) on
one GPU, each scanning its period range in the mixed form and refitting its
share of the gathered minimum region in the FP64 form (shard.main with
--refine), give the same rows as one process running the same steps, and the
same best period as the single-process refined scan (ps_scan_refined)."""
from __future__ import annotations

import os
import socket
import subprocess
import sys

import numpy as np
import pytest

from conftest import GOLDEN, ROOT

pytestmark = pytest.mark.gpu


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


@pytest.mark.parametrize("case", ["tiny_cal", "tiny_mix"])
def test_two_ranks_on_one_gpu_match_single_process(engine_lib, tmp_path, case):
    from periodsearch_gb300 import PS_FORM_FP64, PS_FORM_MIXED, Engine, format_row, read_input
    from periodsearch_gb300.shard import refine_sharded

    inp = GOLDEN / case / "period_search_in"
    out = tmp_path / "period_search_out"
    port = _free_port()
    procs = []
    for rank in range(2):
        env = dict(os.environ, RANK=str(rank), WORLD_SIZE="2", LOCAL_RANK="0", MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, "-m", "periodsearch_gb300.shard", str(inp), str(out),
                                       "--form", "mixed", "--refine", "--backend", "gloo"],
                                      cwd=ROOT, env=env, stdout=subprocess.PIPE, stderr=subprocess.STDOUT,
                                      text=True))
    logs = [p.communicate(timeout=600)[0] for p in procs]
    for p, log in zip(procs, logs):
        assert p.returncode == 0, log

    data = read_input(inp)
    with Engine(data, form=PS_FORM_MIXED) as eng, Engine(data, form=PS_FORM_FP64) as eng64:
        conw_r, _ = eng.precalc_conw()
        n_max = int(eng.info.n_max)
        rows = eng.scan(conw_r, 1, n_max)
        single, best, nref = refine_sharded(rows, lambda per: eng64.rows_of_periods(conw_r, per), 1)
        _, st = eng.scan_refined(conw_r, 1, n_max)
        fp64_rows = eng64.scan(conw_r, 1, n_max)
    got = out.read_text().splitlines(keepends=True)
    assert got == [format_row(r) for r in single]
    assert nref >= 5
    assert best == int(st["best_index"])
    # the refitted rows carry the FP64 form's values
    np.testing.assert_array_equal(single["rms"][best - 1], fp64_rows["rms"][best - 1])
