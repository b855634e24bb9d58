"""HamiltonianGen operator expressions (bl_hamgen) against the reference's own HamiltonianGen.

Fixtures: tests/golden/hamgen.npz, written by `make_golden.py --hamgen` from the reference
(spin operators and tensors, spatial tensors at two angle sets, arithmetic and precedence,
functions on numbers and element by element on matrices, comparisons, variables, and the
reference's parser quirks).  Host-side only: no GPU."""
import json
from pathlib import Path

import numpy as np
import pytest

import blochlib_gb300 as bl

FIX = Path(__file__).parent / "golden" / "hamgen.npz"


def _fixtures():
    z = np.load(FIX)
    exprs = list(z["_exprs"])
    angles = z["_angles"]
    systems = json.loads(str(z["_systems"]))
    variables = {k: complex(*v) for k, v in json.loads(str(z["_vars"])).items()}
    cases = []
    for key in z.files:
        if key.startswith("_"):
            continue
        sname, ai, ei = key.split("|")
        cases.append((sname, systems[sname], tuple(angles[int(ai)]), str(exprs[int(ei)]), z[key]))
    return cases, variables


CASES, VARS = _fixtures()


@pytest.mark.parametrize("case", range(len(CASES)), ids=[f"{c[0]}:{c[3]}@{c[2][0]}" for c in CASES])
def test_hamgen_matches_reference(case):
    sname, lines, ang, expr, want = CASES[case]
    s = bl.SolidSys(lines)
    g = bl.HamiltonianGen()
    for k, v in VARS.items():
        g.addVar(k, v)
    got = g.Hamiltonian(s, expr, *ang)
    scale = max(1.0, float(np.max(np.abs(want))))
    assert got.shape == want.shape
    assert np.max(np.abs(got - want)) <= 1e-13 * scale, (expr, np.max(np.abs(got - want)))


def test_hamgen_covers_every_expression():
    seen = {c[3] for c in CASES}
    assert len(seen) >= 130 and len(CASES) >= 450


@pytest.mark.parametrize("expr", ["A20", "Iq_0", "Ix_0 +", "(Ix_0", "Iz_5", "T23_0", "2ex*Iz_0", "Ix_0 > Iz_0",
                                  "Iz_0 ^ Ix_0", "3", "Ix_0 / (Iz_0 - Iz_0)", "", "Ix_0 * _"])
def test_hamgen_errors(expr):
    """A numeric result, unknown names, syntax errors, spins out of range, tensor ranks/orders
    the reference rejects, comparisons of matrices, singular division: all fail cleanly."""
    s = bl.SolidSys(["numspin 2", "T 1H 0", "T 13C 1"])
    with pytest.raises(bl.BlochError):
        bl.HamiltonianGen().Hamiltonian(s, expr)


def test_hamgen_agrees_with_operator_names():
    """The engine's own operator syntax and HamiltonianGen's describe the same matrices."""
    s = bl.SolidSys(["numspin 3", "T 1H 0", "T 13C 1", "T 2H 2"])
    g = bl.HamiltonianGen()
    np.testing.assert_array_equal(g.Hamiltonian(s, "Ix"), s.op("Fx"))
    np.testing.assert_array_equal(g.Hamiltonian(s, "Iz_2"), s.op("Iz 2"))
    np.testing.assert_allclose(g.Hamiltonian(s, "Ix_0 + Iz_1"), s.op("Ix 0 + Iz 1"), atol=0)
