"""Handles and batches on a caller's stream.  The step-loop kernels are
launched with programmatic dependent launch, so consecutive kernels of
different handles on one stream must still see each other's completed
work; results equal the same runs on the handles' own streams, bit for
bit, whatever the interleaving (and across a switch back to the own stream,
which drops the captured graphs)."""
import numpy as np
import pytest

import fv3d_gb300 as fv
from fv3d_gb300 import problems

pytestmark = pytest.mark.gpu


def _alone(pr, n):
    s = fv.Simulation(pr.params)
    s.set_prim(*pr.prim)
    s.enqueue_steps(n)
    return s.get_prim()


def test_handles_share_a_caller_stream():
    torch = pytest.importorskip("torch")
    prs = [problems.sedov(64), problems.rayleigh_taylor(64, 192), problems.blast(24, nz=20)]
    want = [_alone(p, 12) for p in prs]
    st = torch.cuda.Stream()
    sims = []
    for p in prs:
        s = fv.Simulation(p.params)
        s.set_prim(*p.prim)
        s.set_stream(st.cuda_stream)
        sims.append(s)
    for n in (3, 4, 5):  # interleaved on one stream
        for s in sims:
            s.enqueue_steps(n)
    for s, w in zip(sims, want):
        s.set_stream(0)  # back to the handle's own stream (waits for the caller's)
        for a, b in zip(s.get_prim(), w):
            np.testing.assert_array_equal(a, b)


def test_batch_and_handle_share_a_caller_stream():
    torch = pytest.importorskip("torch")
    sod = problems.sod(64, "x", nx_other=32)
    sed = problems.sedov(48, tend=1.0e30)
    ref = fv.Batch([sod.params])
    ref.set_prim(0, *sod.prim)
    ref.run(6)
    want_b = ref.get_prim(0)
    want_s = _alone(sed, 6)
    st = torch.cuda.Stream()
    b = fv.Batch([sod.params])
    b.set_prim(0, *sod.prim)
    s = fv.Simulation(sed.params)
    s.set_prim(*sed.prim)
    b.set_stream(st.cuda_stream)
    s.set_stream(st.cuda_stream)
    for _ in range(3):
        b.run(2)
        s.enqueue_steps(2)
    st.synchronize()
    for a, w in zip(b.get_prim(0), want_b):
        np.testing.assert_array_equal(a, w)
    for a, w in zip(s.get_prim(), want_s):
        np.testing.assert_array_equal(a, w)
