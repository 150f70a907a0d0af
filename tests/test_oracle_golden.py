"""Pin the oracle to the reference's golden outputs: relative L2 errors of the sine application
(applications/poisson/sine/tests/{cartesian,curvilinear}.output; fixture tests/golden/sine_errors.json)."""
import json
import os

import numpy as np
import pytest

import oracle as O

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "sine_errors.json")))


def sine_problem(k, curved):
    m = O.mesh_desc(8, lo=(-1, -1, -1), hi=(1, 1, 1), bc=(0, 1, 0, 0, 0, 0), deform_amp=0.15 if curved else 0.0,
                    deform_freq=2, deform_left=-1.0, deform_right=1.0, mapping_degree=3)
    return O.Problem(m, k)


@pytest.mark.parametrize("mesh", ["cartesian", "curvilinear"])
@pytest.mark.parametrize("k", [1, 2, 3, 4, 5, 6, 7])
def test_sine_golden_error(mesh, k):
    p = sine_problem(k, mesh == "curvilinear")
    b = p.rhs(O.FN_SINE, 3 * np.pi)
    x, r = p.solve(b, precond=2, rel_tol=1e-10, abs_tol=1e-20)
    assert r.converged
    err = p.error(x, O.FN_SINE, 3 * np.pi)
    gold = GOLD[mesh]["relative_l2_error"][k - 1]
    # the reference prints 6 significant digits
    assert abs(err - gold) <= 5e-6 * gold + 1e-12, (err, gold)
