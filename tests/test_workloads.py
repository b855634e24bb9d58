"""The seeded workload generators."""
import json

import numpy as np

from blochlib_gb300 import workloads as W
from helpers import GOLDEN


def test_zcw3_closed_form_matches_reference_powder_files():
    s = json.loads((GOLDEN / "zcw3_samples.json").read_text())
    for n, rec in s.items():
        a, b, g, w = W.zcw3(int(n))
        assert len(a) == rec["count"]
        got = np.stack([a, b, g, w], axis=1)[rec["index"]]
        np.testing.assert_allclose(got, np.array(rec["rows"]), rtol=0, atol=5e-12)


def test_configs_are_deterministic_and_shaped():
    for i in range(4):
        a, b = W.config(i), W.config(i)
        assert a["lines"] == b["lines"]
    assert W.config(0)["npts"] == 1024 and W.config(1)["npts"] == 2048 and W.config(2)["npts"] == 4096
    assert len(W.config(1)["powder"][0]) == 3722 and len(W.config(0)["powder"][0]) == 1154
    assert sum(l.startswith("D ") for l in W.config(2)["lines"]) == 28
