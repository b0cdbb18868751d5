"""The oracle against its committed golden values (tests/golden/oracle_trace.json,
written by tests/golden/make_oracle_golden.py): the cheap cases are re-run
here, so any change in the restatement's results shows as a failure."""
import json
import os
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_oracle_golden as G  # noqa: E402

FIXTURE = json.load(open(os.path.join(HERE, "golden", "oracle_trace.json"), encoding="utf-8"))


def test_fixture_lists_every_case():
    assert [c["name"] for c in FIXTURE["cases"]] == [c["name"] for c in G.CASES]


@pytest.mark.parametrize("case", [c for c in FIXTURE["cases"] if c["cheap"]], ids=lambda c: c["name"])
def test_oracle_reproduces_golden(case):
    assert G.run_oracle(case) == case["expect"]
