"""Shared fixtures.  GPU tests carry @pytest.mark.gpu; everything else runs on
CPU.  The product library and the oracle are built in-tree on first use."""
from __future__ import annotations

import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))

GOLDEN = ROOT / "tests" / "golden"
SYNTH_CASES = ["tiny_cal", "tiny_rel", "tiny_mix", "tiny_stop", "c0_12"]
# four of the reference's real work units, cut to 12 periods (tests/golden/make_fixtures.py)
WU_CASES = ["wu_17979", "wu_4332", "wu_26380", "wu_2543"]


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs an sm_103 GPU (run with -m gpu)")


@pytest.fixture(scope="session")
def engine_lib():
    from periodsearch_gb300 import build

    build.build()
    from periodsearch_gb300 import _abi

    return _abi.lib()


@pytest.fixture(scope="session")
def oracle():
    import oracle_binding

    oracle_binding.build_oracle()
    return oracle_binding
