"""The failure path of the tensor-core kernels, exercised without a GPU fault
(GPU required): every mbarrier wait in them is bounded; a wait that runs out
ends the kernel with a status word the host reads, and the context stays
usable.  Here a self-test kernel waits, with the same bounded wait, on a phase
that nothing completes."""
import numpy as np
import pytest

import anime4kcpp_gb300 as ac
import oracle
from anime4kcpp_gb300 import synthetic

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    from anime4kcpp_gb300 import build
    build.build()
    oracle.build()


@pytest.mark.parametrize("limit_ms", [20, 200])
def test_bounded_wait_gives_up_and_reports(limit_ms):
    rc, status, ms = ac.wait_selftest(limit_ms)
    assert rc == 0
    assert status == 1  # the wait gave up (2 would mean the phase completed)
    assert limit_ms * 0.9 <= ms <= limit_ms + 500


def test_context_usable_after_a_timed_out_wait():
    assert ac.wait_selftest(50)[1] == 1
    p = ac.Processor("cuda", 0, "acnet-legacy-hdn0", precision="fp16")
    x = synthetic.rgb_u8(37, 41, seed=3)
    out = p.process(x, 2.0)
    assert p.ok(), p.error()
    d = np.abs(out.astype(int) - oracle.process(x, 2.0, "acnet-legacy-hdn0").astype(int))
    assert d.max() <= 6


@pytest.mark.parametrize("form,factor,c", [("fp16", 2.0, 3), ("fp16", 4.0, 3), ("fp32", 2.0, 1), ("fp16", 2.0, 1)])
def test_injected_allocation_failure_is_reported_and_recoverable(form, factor, c):
    """Host-side fault injection: the first device allocation of a fresh
    processor's call fails as if the device were out of memory.  The call
    reports it through ok() / error() without touching the GPU, and the next
    call on the same processor succeeds with the right result."""
    x = synthetic.rgb_u8(53, 71, seed=4) if c == 3 else synthetic.luma(53, 71, np.uint8, seed=4)
    p = ac.Processor("cuda", 0, "acnet-legacy-hdn1", precision=form)
    assert p.ok(), p.error()
    ac.debug_fail_alloc(1)
    try:
        p.process(x, factor)
        assert not p.ok()
        assert "allocation" in p.error(), p.error()
    finally:
        ac.debug_fail_alloc(0)
    out = p.process(x, factor)
    assert p.ok(), p.error()
    want = oracle.process(x, factor, "acnet-legacy-hdn1")
    assert np.abs(out.astype(int) - want.astype(int)).max() <= (1 if form == "fp32" else 2)


def test_injected_allocation_failure_in_the_serving_loop():
    """A job whose buffer allocation fails completes with status -1 and the
    error; the server keeps serving the jobs after it."""
    import torch
    x = synthetic.rgb_u8(45, 61, seed=8)
    src = torch.from_numpy(x).pin_memory().numpy()
    outs = [torch.empty((90, 122, 3), dtype=torch.uint8).pin_memory().numpy() for _ in range(2)]
    srv = ac.Server(0, "fp16", hbm_budget_gb=1.0, workers=2)
    try:
        ac.debug_fail_alloc(1)
        r = srv.wait(srv.submit(src, outs[0], "acnet-legacy-hdn0", 2.0))
        ac.debug_fail_alloc(0)
        assert r["status"] == -1 and "allocation" in r["error"], r
        r = srv.wait(srv.submit(src, outs[1], "acnet-legacy-hdn0", 2.0))
        assert r["status"] == 0, r
        want = oracle.process(x, 2.0, "acnet-legacy-hdn0")
        assert np.abs(outs[1].astype(int) - want.astype(int)).max() <= 2
    finally:
        ac.debug_fail_alloc(0)
        srv.close()
