"""The serving loop (ac_gb300_server_*): continuous batching and HBM-budget
admission over a mix of resolutions, factors, models and formats (GPU
required).  Each job's result must be the same alone and in the mix: the jobs
run through the same processors and kernels as ac_processor_process, and
every tile shape and batch composition gives identical bytes, so the
tolerance is zero."""
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


def _jobs():
    rng = np.random.default_rng(5)
    jobs = []
    models = ["acnet-legacy-hdn0", "acnet-legacy-hdn1", "acnet-legacy-hdn2", "acnet-legacy-hdn3", "arnet-b8"]
    for i in range(18):
        h, w = int(rng.integers(40, 260)), int(rng.integers(40, 300))
        model = models[i % 5] if i % 3 else "acnet-legacy-hdn1"  # every third job batches with its peers
        factor = 4.0 if i % 7 == 3 else 2.0
        if i % 5 == 4 and model != "arnet-b8":
            y = synthetic.luma(h - h % 2, w - w % 2, np.uint16, seed=i, noise=4.0, bits=10)
            u = synthetic.luma(y.shape[0] // 2, y.shape[1] // 2, np.uint16, seed=i + 50, bits=10)
            v = synthetic.luma(y.shape[0] // 2, y.shape[1] // 2, np.uint16, seed=i + 90, bits=10)
            jobs.append(("yuv", model, factor, (y, u, v)))
        else:
            jobs.append(("rgb", model, factor, synthetic.rgb_u8(h, w, seed=i)))
    return jobs


def _outs(kind, factor, x):
    f = int(factor)
    if kind == "rgb":
        return np.zeros((f * x.shape[0], f * x.shape[1], 3), np.uint8)
    return tuple(np.zeros((f * p.shape[0], f * p.shape[1]), np.uint16) for p in x)


def _alone(kind, model, factor, x, form):
    torch = pytest.importorskip("torch")
    p = ac.Processor("cuda", 0, model, precision=form)
    if kind == "rgb":
        out = p.process(x, factor)
        assert p.ok(), p.error()
        return out
    src = [tuple(torch.from_numpy(pl).cuda() for pl in x)]
    dst = [tuple(torch.empty((int(factor) * pl.shape[0], int(factor) * pl.shape[1]), dtype=torch.uint16, device="cuda")
                 for pl in x)]
    p.process_yuv_device(src, dst, factor, 6)
    return tuple(d.cpu().numpy() for d in dst[0])


@pytest.mark.parametrize("form", ["fp16", "fp32"])
def test_results_are_the_same_alone_and_in_the_mix(form):
    jobs = _jobs()
    srv = ac.Server(0, form, hbm_budget_gb=8.0, workers=3)
    outs, tickets = [], []
    for kind, model, factor, x in jobs:  # all submitted at once: admitted, batched and overlapped together
        o = _outs(kind, factor, x)
        outs.append(o)
        tickets.append(srv.submit(x, o, model, factor, shift=6 if kind == "yuv" else 0))
    results = [srv.wait(t) for t in tickets]
    for r in results:
        assert r["status"] == 0, r["error"]
        assert r["latency_ms"] >= r["device_ms"] >= 0.0
        # the GPU-timed parts (CUDA events on the worker's stream) lie inside the device span
        parts = (r["h2d_ms"], r["compute_ms"], r["d2h_ms"])
        assert min(parts) >= 0.0 and r["compute_ms"] > 0.0
        assert sum(parts) <= r["device_ms"] + 0.05
    st = srv.stats()
    assert st["completed"] == len(jobs) and st["failed"] == 0
    if form == "fp16":
        assert max(r["batch"] for r in results) > 1  # continuous batching merged ready jobs
    srv.close()
    for (kind, model, factor, x), o in zip(jobs, outs):
        want = _alone(kind, model, factor, x, form)
        if kind == "rgb":
            assert np.array_equal(o, want), (model, factor, x.shape)
        else:
            for a, b in zip(o, want):
                assert np.array_equal(a, b), (model, factor, x[0].shape)


def test_budget_admission_and_rejection():
    frames = [synthetic.rgb_u8(540, 960, seed=i) for i in range(6)]
    budget = 40e6  # one 960x540 x2 job needs ~9 MB of frame buffers plus 1 MB of tables
    srv = ac.Server(0, "fp16", hbm_budget_gb=budget / 1e9, workers=2)
    outs = [np.zeros((1080, 1920, 3), np.uint8) for _ in frames]
    tickets = [srv.submit(x, o, "acnet-legacy-hdn0", 2.0) for x, o in zip(frames, outs)]
    big = synthetic.rgb_u8(1080, 1920, seed=9)
    big_out = np.zeros((4320, 7680, 3), np.uint8)
    t_big = srv.submit(big, big_out, "acnet-legacy-hdn0", 4.0)  # ~300 MB: can never fit
    for t in tickets:
        assert srv.wait(t)["status"] == 0
    r = srv.wait(t_big)
    assert r["status"] == -2 and "HBM budget" in r["error"]
    st = srv.stats()
    assert 0 < st["peak_bytes"] <= budget and st["pool_bytes"] <= budget
    srv.close()
    p = ac.Processor("cuda", 0, "acnet-legacy-hdn0", precision="fp16")
    for x, o in zip(frames, outs):
        assert np.array_equal(o, p.process(x, 2.0))


def test_malformed_jobs_are_rejected():
    srv = ac.Server(0, "fp16", hbm_budget_gb=1.0, workers=1)
    x = synthetic.rgb_u8(32, 32, seed=1)
    # every family of the reference is served (here ArtCNN, FP32 pipeline):
    # the job gives the ordinary processor's bytes
    out = np.zeros((64, 64, 3), np.uint8)
    t = srv.submit(x, out, "artcnn-c4f16", 2.0)
    r = srv.wait(t)
    assert r["status"] == 0, r["error"]
    assert np.array_equal(out, ac.Processor("cuda", 0, "artcnn-c4f16", precision="fp16").process(x, 2.0))
    t = srv.submit(x, np.zeros((64, 64, 3), np.uint16), "acnet-legacy-hdn0", 2.0)
    r = srv.wait(t)
    assert r["status"] == -2 and "differ" in r["error"]
    srv.close()


def test_cli_default_model_jobs_batched():
    """Jobs of the reference CLI's default model (ACNet<8> B8 HDN, RGB) and of
    ACNet<8> B4 (gray), submitted together: the server batches them through
    the quad kernel, and each gets the ordinary processor's bytes."""
    srv = ac.Server(0, "fp16", hbm_budget_gb=4.0, workers=2)
    jobs = [("acnet-f8b8-hdn", synthetic.rgb_u8(90 + 7 * i, 130 + 11 * i, seed=30 + i)) for i in range(5)]
    jobs.append(("acnet-f8b4", synthetic.luma(70, 90, np.uint8, seed=9)))
    outs, tickets = [], []
    for model, x in jobs:
        o = np.zeros((2 * x.shape[0], 2 * x.shape[1]) + x.shape[2:], np.uint8)
        outs.append(o)
        tickets.append(srv.submit(x, o, model, 2.0))
    for t in tickets:
        r = srv.wait(t)
        assert r["status"] == 0, r["error"]
    srv.close()
    for (model, x), o in zip(jobs, outs):
        assert np.array_equal(o, ac.Processor("cuda", 0, model, precision="fp16").process(x, 2.0)), model
