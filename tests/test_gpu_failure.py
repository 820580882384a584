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
