"""Pins the CPU oracle (oracle/fv3d_oracle.c) to the reference itself.

The fixtures under tests/golden/ were produced by the reference's own FP64
headers (tests/golden/make_golden.py); the C restatement must reproduce them
bit for bit: every dt and every field after one and after several steps, and
the Riemann-solver known answers.
"""
import os

import numpy as np
import pytest

from _helpers import GOLDEN, golden_cases, load_case, params_from_dict
from oracle import pyoracle

CASES = [c["name"] for c in golden_cases()]


@pytest.mark.parametrize("name", CASES)
def test_oracle_reproduces_reference_bitwise(name):
    case = load_case(name)
    p = params_from_dict(case["params"])
    ora = pyoracle.Oracle(p)
    ora.set_prim(*case["qin"])
    got_q0 = np.stack(ora.get_prim())
    np.testing.assert_array_equal(got_q0, case["q0"])
    for k, dt_ref in enumerate(case["dts"]):
        dt = ora.compute_dt()
        assert dt == dt_ref, "step %d dt %r != reference %r" % (k, dt, dt_ref)
        ora.step(dt)
        if k == 0:
            np.testing.assert_array_equal(np.stack(ora.get_prim()), case["q1"])
    np.testing.assert_array_equal(np.stack(ora.get_prim()), case["qN"])


@pytest.mark.parametrize("solver,name", [(0, "hll"), (1, "hllc")])
@pytest.mark.parametrize("gamma", [1.4, 5.0 / 3.0])
def test_riemann_known_answers(solver, name, gamma):
    kat = np.load(os.path.join(GOLDEN, "riemann_kats.npz"))
    flux, pout = pyoracle.riemann(solver, gamma, kat["qL"], kat["qR"])
    np.testing.assert_array_equal(flux, kat["%s_%g_flux" % (name, gamma)])
    np.testing.assert_array_equal(pout, kat["%s_%g_pout" % (name, gamma)])


def test_oracle_thread_count_does_not_change_results():
    case = load_case("random_xy_tc_visc")
    p = params_from_dict(case["params"])
    outs = []
    for nt in (1, 3):
        pyoracle.set_threads(nt)
        ora = pyoracle.Oracle(p)
        ora.set_prim(*case["qin"])
        ora.step(ora.compute_dt())
        outs.append(np.stack(ora.get_prim()))
    pyoracle.set_threads(0)
    np.testing.assert_array_equal(outs[0], outs[1])


@pytest.mark.skipif(not pyoracle.reference_available(), reason="reference sources absent")
def test_oracle_matches_reference_longer_run():
    """Both CPU builds run the main.cpp loop to a final time on a blast."""
    import tempfile
    from fv3d_gb300 import problems
    pr = problems.sedov(64, tend=0.01)
    path = os.path.join(tempfile.mkdtemp(), "s.ini")
    with open(path, "w") as f:
        f.write(pr.ini)
    ref = pyoracle.RefOracle(path)
    ora = pyoracle.Oracle(pr.params)
    ref.set_prim(*pr.prim)
    ora.set_prim(*pr.prim)
    t1, n1 = ref.advance(pr.params.tend)
    t2, n2 = ora.advance(pr.params.tend)
    assert (t1, n1) == (t2, n2)
    np.testing.assert_array_equal(np.stack(ref.get_prim()), np.stack(ora.get_prim()))
