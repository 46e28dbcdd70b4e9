"""FP64 batches at the benchmark sizes against the oracle.

The two batch configurations are built in full -- 512 Sod / Sedov instances
with sides 64-256 and 64 Rayleigh-Taylor instances from 256 x 768 to
1024 x 3072 with conduction and viscosity -- and advanced by the persistent
batch kernels, each instance with its own CFL dt.  A seeded sample of the
instances (the smallest, the largest, one of median size and five drawn at
random) is advanced by the oracle from the same initial state for the same
number of steps (the main.cpp loop with its own CFL dt each step): times and
fields must agree to the per-step bound times the step count -- in fact bit
for bit, since the FP64 path rounds like the reference.
"""
import numpy as np
import pytest

import fv3d_gb300 as fv
from fv3d_gb300 import problems
from _helpers import REL_L1_STEP, rel_l1_fields
from oracle import pyoracle

pytestmark = pytest.mark.gpu


def sample(probs, seed, n_random=5):
    cells = np.array([p.cells for p in probs])
    order = np.argsort(cells, kind="stable")
    pick = [int(order[0]), int(order[-1]), int(order[len(order) // 2])]
    rng = problems.uniform(seed, 41, 4 * n_random)
    for u in rng:
        i = min(int(u * len(probs)), len(probs) - 1)
        if i not in pick:
            pick.append(i)
        if len(pick) == 3 + n_random:
            break
    return pick


def check_batch_against_oracle(probs, nsteps, seed):
    b = fv.Batch([p.params for p in probs])
    for i, pr in enumerate(probs):
        b.set_prim(i, *pr.prim)
    b.run(nsteps)
    t = b.times()
    pyoracle.set_threads(0)
    for i in sample(probs, seed):
        pr = probs[i]
        ora = pyoracle.Oracle(pr.params)
        ora.set_prim(*pr.prim)
        t_o, n_o = ora.advance(1.0e30, max_steps=nsteps)
        assert n_o == nsteps
        assert t[i] == t_o, (i, pr.name, t[i], t_o)
        got, want = b.get_prim(i), ora.get_prim()
        errs = rel_l1_fields(got, want)
        assert max(errs) <= nsteps * REL_L1_STEP, (i, pr.name, pr.shape, errs)
        for k in range(5):
            np.testing.assert_array_equal(got[k], want[k], err_msg="instance %d (%s) field %d" % (i, pr.name, k))
        ora.close()
    b.close()


def test_batch512_sod_sedov_fp64_vs_oracle():
    check_batch_against_oracle(problems.batch_sod_sedov(512), nsteps=4, seed=512)


def test_batch64_rt_fp64_vs_oracle():
    check_batch_against_oracle(problems.batch_rt(64), nsteps=3, seed=64)
