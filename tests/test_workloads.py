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


def test_repulsion_powder_sets():
    """c3/c4 draw the reference's repulsion sets (3 columns: gamma = 0, file weights)."""
    for n, count in [(100, 100), (144, 144), (320, 320), (678, 677)]:
        phi, theta, gamma, w = W.rep(n)
        assert len(phi) == len(theta) == len(gamma) == len(w) == count
        assert np.all(gamma == 0.0) and np.all(w > 0)
        assert np.all((theta >= 0) & (theta <= np.pi + 1e-9))
    sizes = {len(W.config(3, i)["powder"][0]) for i in range(40)}
    assert sizes <= {144, 320, 677, 1154} and len(sizes) >= 3
    big = W.config(4, 0)
    assert int(big["lines"][0].split()[1]) in (9, 10) and len(big["powder"][0]) == 100
