"""Hamiltonian blocks larger than 74 (9 or more like spins 1/2): the batched-product path.
Parity with the reference itself runs through the golden cases huge_9h and huge_9h_nonsym
(tests/test_gpu_parity.py::test_gpu_matches_reference_golden); these tests check the
properties that do not need a reference run: batch invariance (with a workspace chunk
boundary inside a crystallite range), a crystallite alone against the same crystallite in a
batch, and the mixed form against FP64."""
import numpy as np
import pytest

import blochlib_gb300 as bl
from blochlib_gb300 import workloads as W
from helpers import gpu_fid, load_golden, parse_job, rel

pytestmark = pytest.mark.gpu


def _job(count):
    job, _, _, _, _ = load_golden("huge_9h")
    cfg = W.config(0)
    rows = np.stack(cfg["powder"], axis=1)[:count]
    return job, rows


def test_huge_system_uses_blocks_above_74():
    job, _ = _job(1)
    lines, _ = parse_job(job)
    assert max(bl.SolidSys(lines).blocks()) == 126


def test_huge_batches_are_bitwise_identical():
    """128 crystallites x 12 steps: the exponential's workspace takes ~1200 items per launch,
    so a launch boundary falls inside a step; two crystallite batches against one."""
    job, rows = _job(128)
    one = gpu_fid(job, rows)
    small = bl.Context(0, hbm_budget=(1 << 30) + (4 << 30))  # 1 GiB workspace + ~4 GiB: two batches
    two = gpu_fid(job, rows, ctx=small)
    np.testing.assert_array_equal(one, two)


def test_huge_crystallite_alone_equals_in_batch():
    job, rows = _job(40)
    c = 23
    alone = gpu_fid(job, rows[c:c + 1])
    masked = rows.copy()
    masked[:, 3] = 0.0
    masked[c, 3] = rows[c, 3]
    np.testing.assert_array_equal(alone, gpu_fid(job, masked))


def test_huge_mixed_form_within_1e6():
    job, rows = _job(32)
    f64 = gpu_fid(job, rows)
    f32 = gpu_fid(job, rows, precision=1)
    assert rel(f32, f64) <= 1e-6, rel(f32, f64)
