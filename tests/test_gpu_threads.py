"""One processor shared by several host threads (the reference CLI's and
benchmark's pattern; reference CUDAProcessor.cpp:374-386 keeps scratch, error
state and stream per calling thread), for every kernel family's path: each
thread's results equal the single-threaded ones, and an error on one thread
leaves the others' state alone (GPU required)."""
import threading

import numpy as np
import pytest

import anime4kcpp_gb300 as ac
from anime4kcpp_gb300 import synthetic

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    from anime4kcpp_gb300 import build
    build.build()


@pytest.mark.parametrize("model", ["acnet-f8b8-hdn", "artcnn-c4f16", "artcnn-c4f32", "fsrcnnx-f8", "arnet-b8"])
def test_threads_share_one_processor(model):
    p = ac.Processor("cuda", 0, model, precision="fp16")
    imgs = [synthetic.rgb_u8(40 + 9 * i, 52 + 7 * i, seed=i) if i % 2 else synthetic.luma(40 + 9 * i, 52 + 7 * i, seed=i)
            for i in range(6)]
    want = [p.process(im, 2.0) for im in imgs]
    assert p.ok(), p.error()
    got = [None] * len(imgs)
    errors = []

    def work(i):
        for _ in range(3):
            out = p.process(imgs[i], 2.0)
            if not p.ok():
                errors.append(p.error())
            got[i] = out

    ts = [threading.Thread(target=work, args=(i,)) for i in range(len(imgs))]
    [t.start() for t in ts]
    [t.join() for t in ts]
    assert not errors, errors
    for a, b in zip(got, want):
        assert np.array_equal(a, b)


def test_error_state_is_per_thread():
    p = ac.Processor("cuda", 0, "acnet-legacy-hdn0", precision="fp16")
    x = synthetic.rgb_u8(48, 64, seed=2)
    want = p.process(x, 2.0)
    start = threading.Barrier(2)
    res = {}

    def bad():
        start.wait()
        for _ in range(5):
            p.process(x, -1.0, dst=np.zeros((96, 128, 3), np.uint8))
        res["bad"] = (p.ok(), p.error())

    def good():
        start.wait()
        outs = [p.process(x, 2.0) for _ in range(5)]
        res["good"] = (p.ok(), all(np.array_equal(o, want) for o in outs))

    ts = [threading.Thread(target=bad), threading.Thread(target=good)]
    [t.start() for t in ts]
    [t.join() for t in ts]
    assert res["bad"][0] is False and "factor" in res["bad"][1]
    assert res["good"] == (True, True)
