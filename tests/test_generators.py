"""The problem generators of Init.h (InitFunctor::init, Init.h:18-279) in the
CPU oracle, pinned to fixtures the reference's own Init.h produced
(tests/golden/generators.npz): the piecewise-constant generators bit for bit,
the cos / pow fields within a few units in the last place, and the H84 / C91
perturbations -- drawn here from the counter-based stream that replaces
Kokkos' XorShift64 pool -- by their amplitude and by the stream itself."""
import numpy as np
import pytest

from _helpers import GEN_RANDOM, assert_generated, generator_cases, load_generator
from fv3d_gb300 import problems
from oracle import pyoracle

CASES = generator_cases()


def _oracle(ini):
    p = pyoracle.parse_ini(ini)
    return p, pyoracle.Oracle(p)


@pytest.mark.parametrize("name", CASES)
def test_oracle_generators_match_reference(name):
    ini, want = load_generator(name)
    p, ora = _oracle(ini)
    got = ora.generate()
    assert_generated(got, want, name)
    # the state it sets is primToCons of the generated primitives, as set_prim's
    ref = pyoracle.Oracle(p)
    ref.set_prim(*got)
    for a, b in zip(ora.get_cons(), ref.get_cons()):
        np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("name", sorted(GEN_RANDOM))
def test_oracle_perturbations_follow_the_stream(name):
    ini, want = load_generator(name)
    p, ora = _oracle(ini)
    got = ora.generate()
    n = p.Nx * p.Ny * p.Nz
    if name.startswith("h84"):
        u = problems.uniform(p.seed, 31, n).reshape(got[3].shape)
        np.testing.assert_array_equal(got[3], p.h84_pert * (u - 0.5))
        assert np.abs(got[3]).max() <= 0.5 * p.h84_pert
    else:
        # p = T^(m1+1) (1 + pert): the perturbation relative to the
        # reference's unperturbed profile stays within its amplitude
        u = problems.uniform(p.seed, 32, n).reshape(got[4].shape)
        pert = p.c91_pert * (u - 0.5)
        z = p.zmin + (np.arange(p.Nz) + 0.5) * p.dz
        T = (1.0 + p.theta1 * z)[:, None, None]
        rel = got[4] / (T ** (p.m1 + 1.0)) - 1.0
        np.testing.assert_allclose(rel, pert, rtol=0, atol=1e-14)
        assert np.abs(want[4] / (T ** (p.m1 + 1.0)) - 1.0).max() <= 0.5 * p.c91_pert * (1 + 1e-12)


def test_unknown_problem_is_refused():
    ini, _ = load_generator("blast_3d")
    p, ora = _oracle(ini.replace("problem=blast", "problem=kelvin"))
    with pytest.raises(ValueError):
        ora.generate()
