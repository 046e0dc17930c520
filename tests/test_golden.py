"""The oracle reproduces the committed golden fixtures (tests/golden/)."""
import os
import sys

import numpy as np
import pytest

from conftest import rel_l1

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_golden  # noqa: E402


@pytest.mark.parametrize("name", sorted(make_golden.GOLDEN))
def test_oracle_reproduces_golden(oracle_lib, name):
    g = np.load(os.path.join(HERE, "golden", name + ".npz"))
    case, x_cb, y_cb, q0, q1, steps, dt_final = make_golden.compute(name)
    assert np.array_equal(q0, g["q0"]), "initial condition changed"
    assert np.array_equal(x_cb, g["x_cb"])
    assert int(g["steps"]) == steps
    # bit-identical on the generating host; across hosts only libm (tanh in
    # the initial condition) may differ in the last bit
    assert rel_l1(q1, g["q"]).max() <= 1e-13
    assert dt_final == pytest.approx(float(g["dt_final"]), rel=1e-12, abs=1e-300)
