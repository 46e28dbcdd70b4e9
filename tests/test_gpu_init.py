"""The problem generators of Init.h on the GPU (fv_init.cu): fvgpu_generate
into caller arrays, fvgpu_init_problem on a handle (FP64 and FP32-mixed) and
fvgpu_batch_init_problem, against the fixtures the reference's own Init.h
produced and against the oracle's restatement (the H84 / C91 perturbations
come from the same counter-based stream on both sides), then a step from the
generated state against the oracle's step from its own."""
import numpy as np
import pytest

import fv3d_gb300 as fv
from _helpers import (GEN_LIBM, GEN_MAX_ULP, GEN_RANDOM, assert_generated, assert_mixed, generator_cases,
                      load_generator)
from oracle import pyoracle

pytestmark = pytest.mark.gpu

CASES = generator_cases()


def _params(ini):
    return fv.parse_ini(ini)


@pytest.mark.parametrize("name", CASES)
def test_generate_matches_reference_and_oracle(name):
    ini, want = load_generator(name)
    p = _params(ini)
    got = fv.generate(p)
    assert_generated(got, want, name)
    ora = pyoracle.Oracle(p).generate()
    for v in GEN_RANDOM.get(name, ()):  # the stream: the same draws as the oracle's
        np.testing.assert_array_max_ulp(got[v], ora[v], maxulp=GEN_MAX_ULP)


@pytest.mark.parametrize("name", CASES)
def test_init_problem_then_step_matches_oracle(name):
    ini, _ = load_generator(name)
    p = _params(ini)
    sim = fv.Simulation(p)
    sim.init_problem()
    ora = pyoracle.Oracle(p)
    ora.generate()
    # the handle's state is primToCons of the GPU's generated primitives:
    # the same as set_prim of those arrays
    ref = fv.Simulation(p)
    ref.set_prim(*fv.generate(p))
    for a, b in zip(sim.get_cons(), ref.get_cons()):
        np.testing.assert_array_equal(a, b)
    exact = name not in GEN_LIBM and name not in GEN_RANDOM
    got = sim.get_prim()
    want = ora.get_prim()
    if exact:  # every field bit for bit: the steps are too
        for a, b in zip(got, want):
            np.testing.assert_array_equal(a, b)
        dt = sim.compute_dt()
        assert dt == ora.compute_dt()
        sim.step(dt)
        ora.step(dt)
        for a, b in zip(sim.get_prim(), ora.get_prim()):
            np.testing.assert_array_equal(a, b)
    else:
        for a, b in zip(got, want):
            np.testing.assert_allclose(a, b, rtol=1e-14, atol=1e-300)


@pytest.mark.parametrize("name", ["blast_xy", "rt_xz", "diffusion_3d", "c91_3d"])
def test_mixed_handle_and_batch_init_problem(name):
    ini, _ = load_generator(name)
    p = _params(ini)
    m = p.copy()
    m.precision = fv._abi.FV_PREC_FP32_MIXED
    sm = fv.Simulation(m)
    sm.init_problem()
    s64 = fv.Simulation(p)
    s64.init_problem()
    assert_mixed(sm.get_prim(), s64.get_prim(), p.gamma0, name)
    b = fv.Batch([p, p])
    b.set_prim(0, *fv.generate(p))
    b.init_problem(1)
    for a, c in zip(b.get_prim(0), b.get_prim(1)):
        np.testing.assert_array_equal(a, c)


def test_init_problem_refuses_unknown_problem():
    ini, _ = load_generator("blast_3d")
    p = _params(ini.replace("problem=blast", "problem=kelvin"))
    sim = fv.Simulation(p)
    with pytest.raises(fv.FvError) as e:
        sim.init_problem()
    assert e.value.status == 1  # FV_ERR_PARAM
    with pytest.raises(fv.FvError):
        fv.generate(p)
