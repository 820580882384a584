"""Batched persistent launches over a shared tile queue, the tile-shape
variants, the autotuner and CUDA-graph replay (GPU required).

Every tile shape computes each output pixel from the same window with the
same arithmetic, so all of them, the batched launch and the per-image path
must give identical bytes.
"""
import numpy as np
import pytest

import anime4kcpp_gb300 as ac
import oracle
from anime4kcpp_gb300 import synthetic

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module", autouse=True)
def built():
    from anime4kcpp_gb300 import build
    build.build()
    oracle.build()


def _frames():
    rng = np.random.default_rng(11)
    imgs = []
    for i in range(7):
        h, w = int(rng.integers(40, 300)), int(rng.integers(40, 400))
        imgs.append(synthetic.rgb_u8(h, w, seed=100 + i))
    for i in range(3):
        imgs.append(synthetic.luma(int(rng.integers(20, 200)), int(rng.integers(20, 200)), np.uint8, seed=200 + i))
    for i in range(2):
        imgs.append(synthetic.rgb_u8(int(rng.integers(30, 120)), int(rng.integers(30, 120)), seed=300 + i, alpha=True))
    return imgs


def _out_like(s):
    return torch.empty((2 * s.shape[0], 2 * s.shape[1]) + tuple(s.shape[2:]), dtype=s.dtype, device="cuda")


def _per_image(p, srcs):
    outs = []
    for s in srcs:
        d = _out_like(s)
        p.process_device(s, d, 2.0)
        outs.append(d.cpu().numpy())
    return outs


@pytest.mark.parametrize("kernel", ["3", "4"])
@pytest.mark.parametrize("form", ["fp16", "bf16"])
def test_batch_matches_per_image_and_replays_graphs(form, kernel, monkeypatch):
    monkeypatch.setenv("AC_GB300_TC_KERNEL", kernel)
    frames = _frames()
    p = ac.Processor("cuda", 0, "acnet-legacy-hdn1", precision=form)
    srcs = [torch.from_numpy(f).cuda() for f in frames]
    want = _per_image(p, srcs)
    dsts = [_out_like(s) for s in srcs]
    groups = 3  # RGB, gray and RGBA images form one launch each
    for call in range(4):
        for d in dsts:
            d.zero_()
        before = ac.graph_replays()
        p.process_batch_device(srcs, dsts, 2.0)
        for d, w in zip(dsts, want):
            assert np.array_equal(d.cpu().numpy(), w)
        replays = ac.graph_replays() - before
        # call 0 measures the plan (autotuner), call 1 launches directly,
        # calls 2 and 3 capture once and replay the graph
        assert replays == (groups if call >= 2 else 0)
    ref = oracle.process(frames[0], 2.0, "acnet-legacy-hdn1").astype(int)
    d = np.abs(want[0].astype(int) - ref)
    assert (d <= 1).mean() >= 0.99


@pytest.mark.parametrize("kernel", ["3", "4"])
@pytest.mark.parametrize("c", [1, 3, 4])
def test_tile_shapes_and_cta_caps_give_identical_bytes(c, kernel, monkeypatch):
    """Each persistent kernel's three tile shapes and CTA caps."""
    monkeypatch.setenv("AC_GB300_TC_KERNEL", kernel)
    if c == 1:
        x = synthetic.luma(131, 150, np.uint16, seed=9)
    else:
        x = synthetic.rgb_u8(131, 150, seed=9, alpha=(c == 4))
    src = torch.from_numpy(x).cuda()
    outs = []
    for shape in ("0", "1", "2"):
        for per_sm in ("1", "2"):
            monkeypatch.setenv("AC_GB300_TC3_SHAPE", shape)
            monkeypatch.setenv("AC_GB300_TC3_PER_SM", per_sm)
            p = ac.Processor("cuda", 0, "acnet-legacy-hdn2", precision="fp16")
            d = _out_like(src)
            p.process_device(src, d, 2.0)
            outs.append(d.cpu().numpy())
            plan = p.last_plan()
            assert plan["kernel"] == ("quad" if kernel == "4" else "pair")
            assert plan["ctas_per_sm"] == int(per_sm)
    for o in outs[1:]:
        assert np.array_equal(o, outs[0])


def _source(h, w, c, dtype, seed):
    x = synthetic.rgb_u8(h, w, seed=seed, alpha=(c == 4)) if c > 1 else synthetic.luma(h, w, np.uint8, seed=seed)
    if dtype == "uint16":
        return (x.astype(np.uint16) * 257).astype(np.uint16)
    if dtype == "float32":
        return (x.astype(np.float32) / 255.0).astype(np.float32)
    return x


@pytest.mark.parametrize("form", ["fp16", "bf16"])
@pytest.mark.parametrize("dtype", ["uint8", "uint16", "float32"])
@pytest.mark.parametrize("c", [1, 3, 4])
def test_split_network_gives_identical_bytes(c, dtype, form, monkeypatch):
    """The quad kernel's network split in two launches (layers 0-4 writing
    a 16-bit activation map, layers 5-8 and the colour merge reading it)
    against the whole network in one launch: the same bytes, for one image
    and for a batch of images of several sizes (tiles at every edge, images
    smaller than a tile)."""
    monkeypatch.setenv("AC_GB300_TC_KERNEL", "4")
    imgs = [_source(h, w, c, dtype, seed=h * 3 + w) for h, w in [(131, 150), (1, 1), (7, 93), (54, 54), (200, 49)]]
    srcs = [torch.from_numpy(x).cuda() for x in imgs]
    outs = {}
    for depth in ("9", "5"):
        monkeypatch.setenv("AC_GB300_FUSION_DEPTH", depth)
        p = ac.Processor("cuda", 0, "acnet-legacy-hdn2", precision=form)
        single = _out_like(srcs[0])
        p.process_device(srcs[0], single, 2.0)
        assert p.ok(), p.error()
        assert p.last_plan()["fusion_depth"] == int(depth)
        dsts = [_out_like(s) for s in srcs]
        p.process_batch_device(srcs, dsts, 2.0)
        assert p.ok(), p.error()
        assert p.last_plan()["fusion_depth"] == int(depth)
        outs[depth] = [single.cpu().numpy()] + [d.cpu().numpy() for d in dsts]
    for a, b in zip(outs["9"], outs["5"]):
        assert np.array_equal(a, b)
    assert np.array_equal(outs["5"][0], outs["5"][1])


@pytest.mark.parametrize("depth", ["9", "5"])
def test_async_calls_on_several_streams_from_one_thread(depth, monkeypatch):
    """x2 calls queued with sync=0 on four streams from one host thread run
    at the same time; each stream has its own tile counters and (split
    network) its own activation maps, so every result equals the result of
    a synchronous call."""
    monkeypatch.setenv("AC_GB300_TC_KERNEL", "4")
    monkeypatch.setenv("AC_GB300_FUSION_DEPTH", depth)
    imgs = [synthetic.rgb_u8(360 + 40 * k, 640 - 32 * k, seed=50 + k) for k in range(4)]
    srcs = [torch.from_numpy(x).cuda() for x in imgs]
    p = ac.Processor("cuda", 0, "acnet-legacy-hdn3", precision="fp16")
    want = []
    for s in srcs:
        d = _out_like(s)
        p.process_device(s, d, 2.0)
        want.append(d.cpu().numpy())
    streams = [torch.cuda.Stream() for _ in srcs]
    for rep in range(3):
        dsts = [_out_like(s) for s in srcs]
        torch.cuda.synchronize()
        for k in range(4):  # each stream: one frame, then a batch of the other three
            p.process_device(srcs[k], dsts[k], 2.0, stream=streams[k].cuda_stream, sync=False)
        bd = [[_out_like(srcs[j]) for j in range(4) if j != k] for k in range(4)]
        for k in range(4):
            p.process_batch_device([srcs[j] for j in range(4) if j != k], bd[k], 2.0, stream=streams[k].cuda_stream,
                                   sync=False)
        torch.cuda.synchronize()
        assert p.ok(), p.error()
        for k in range(4):
            assert np.array_equal(dsts[k].cpu().numpy(), want[k])
            others = [j for j in range(4) if j != k]
            for d, j in zip(bd[k], others):
                assert np.array_equal(d.cpu().numpy(), want[j])
    assert p.last_plan()["fusion_depth"] == int(depth)


@pytest.mark.parametrize("kernel", ["3", "4"])
@pytest.mark.parametrize("batch", [False, True])
def test_autotuned_equals_untuned(kernel, batch, monkeypatch):
    """The autotuner of each persistent kernel (the quad kernel is the
    default) picks a plan -- tile shape and CTAs per SM, measured once per
    batch class -- without changing the bytes."""
    monkeypatch.setenv("AC_GB300_TC_KERNEL", kernel)
    imgs = [synthetic.rgb_u8(300, 500, seed=21)] + ([synthetic.rgb_u8(h, w, seed=h) for h, w in
                                                     [(257, 1031), (700, 333), (64, 64)]] if batch else [])
    srcs = [torch.from_numpy(x).cuda() for x in imgs]
    outs, plans = [], []
    for tune in ("1", "0"):
        monkeypatch.setenv("AC_GB300_AUTOTUNE", tune)
        p = ac.Processor("cuda", 0, "acnet-legacy-hdn0", precision="fp16")
        dsts = [_out_like(s) for s in srcs]
        for _ in range(2):  # the measuring call, then the tuned plan's own launch
            if batch:
                p.process_batch_device(srcs, dsts, 2.0)
            else:
                p.process_device(srcs[0], dsts[0], 2.0)
        outs.append([d.cpu().numpy() for d in dsts])
        plans.append(p.last_plan())
    for a, b in zip(outs[0], outs[1]):
        assert np.array_equal(a, b)
    assert plans[0]["kernel"] == plans[1]["kernel"] == ("quad" if kernel == "4" else "pair")
    assert plans[0]["tile"][0] > 0 and plans[0]["ctas_per_sm"] in (1, 2)
    assert plans[1]["ctas_per_sm"] == 2  # untuned: the default plan
    # the quad kernel's candidates include the network split in two launches
    assert plans[0]["fusion_depth"] in ((9, 5) if kernel == "4" else (9,))
    assert plans[1]["fusion_depth"] == 9


@pytest.mark.parametrize("form,factor", [("fp32", 2.0), ("fp16", 4.0)])
def test_batch_falls_back_per_image(form, factor):
    frames = [synthetic.rgb_u8(41, 67, seed=1), synthetic.luma(33, 29, np.uint8, seed=2)]
    p = ac.Processor("cuda", 0, "acnet-legacy-hdn0", precision=form)
    srcs = [torch.from_numpy(f).cuda() for f in frames]
    want = []
    dsts = []
    for s in srcs:
        f = int(factor)
        d = torch.empty((f * s.shape[0], f * s.shape[1]) + tuple(s.shape[2:]), dtype=s.dtype, device="cuda")
        p.process_device(s, d, factor)
        want.append(d.cpu().numpy())
        dsts.append(torch.empty_like(d))
    p.process_batch_device(srcs, dsts, factor)
    for d, w in zip(dsts, want):
        assert np.array_equal(d.cpu().numpy(), w)
