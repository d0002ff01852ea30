"""The oracle against outputs of the reference CPU engine itself, recorded
by tests/golden/make_golden.py (CPU)."""
import numpy as np
import pytest

import oracle as O
from common import load_golden, make_input, oracle_request

CASES = load_golden("reference_outputs.json")["cases"]


@pytest.mark.parametrize("case", CASES, ids=lambda c: c["name"])
def test_oracle_matches_reference_engine(case):
    h, v = O.Plan(oracle_request(case["horizontal"])), O.Plan(oracle_request(case["vertical"]))
    x = make_input(v.source_size, h.source_size, case["sample"], case["seed"])
    y = O.inverse_2d(h, v, x, case["conversion"])
    assert O.output_hash(y.astype(np.float32)) == case["output_hash"]
