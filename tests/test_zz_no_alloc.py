"""The allocation-free batch entry ac_gb300_process_device_noalloc, through
the C ABI (GPU required).

Its results are compared with the ordinary device entry
(ac_gb300_process_device) on the same processor: both run the persistent
tensor-core kernel, so the bytes must agree exactly, on two calls in a row.
The file is collected last and also passes alone in a fresh process (its
first ordinary call is the set-up the entry requires).
"""
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


def _ordinary(p, torch, srcs):
    outs = []
    for s in srcs:
        shape = (2 * s.shape[0], 2 * s.shape[1]) + tuple(s.shape[2:])
        d = torch.empty(shape, dtype=s.dtype, device="cuda")
        p.process_device(s, d, 2.0)
        outs.append(d)
    return outs


@pytest.mark.parametrize("form", ["fp16", "bf16"])
def test_noalloc_matches_device_entry_on_two_calls(form):
    torch = pytest.importorskip("torch")
    p = ac.Processor("cuda", 0, "acnet-legacy-hdn0", precision=form)
    frames = [synthetic.rgb_u8(180, 320, seed=1), synthetic.rgb_u8(180, 320, seed=2), synthetic.rgb_u8(97, 131, seed=3)]
    srcs = [torch.from_numpy(f).cuda() for f in frames]
    want = [d.cpu().numpy() for d in _ordinary(p, torch, srcs)]  # also uploads the weights
    dsts = [torch.zeros((2 * f.shape[0], 2 * f.shape[1], 3), dtype=torch.uint8, device="cuda") for f in frames]
    stream = torch.cuda.current_stream().cuda_stream
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info()[0]
    for _ in range(2):
        for d in dsts:
            d.zero_()
        rc = p.process_device_noalloc(srcs, dsts, stream=stream, sync=True)
        assert rc == ac.AC_SUCCESS, p.error()
        assert p.ok()
        for d, w in zip(dsts, want):
            assert np.array_equal(d.cpu().numpy(), w)
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free_before
    ref = oracle.process(frames[2], 2.0, "acnet-legacy-hdn0").astype(int)
    diff = np.abs(want[2].astype(int) - ref)
    assert (diff <= 1).mean() >= 0.99 and diff.max() <= (6 if form == "fp16" else 16)


def test_noalloc_luma_u16_batch_of_mixed_sizes():
    torch = pytest.importorskip("torch")
    p = ac.Processor("cuda", 0, "acnet-legacy-hdn2", precision="fp16")
    frames = [synthetic.luma(h, w, np.uint16, seed=h + w) for h, w in ((70, 97), (45, 1), (128, 64))]
    srcs = [torch.from_numpy(f).cuda() for f in frames]
    want = [d.cpu().numpy() for d in _ordinary(p, torch, srcs)]
    dsts = [torch.empty((2 * f.shape[0], 2 * f.shape[1]), dtype=torch.uint16, device="cuda") for f in frames]
    for _ in range(2):
        rc = p.process_device_noalloc(srcs, dsts, sync=True)
        assert rc == ac.AC_SUCCESS, p.error()
        for d, w in zip(dsts, want):
            assert np.array_equal(d.cpu().numpy(), w)


def test_noalloc_rejects_what_it_cannot_do():
    torch = pytest.importorskip("torch")
    src = torch.from_numpy(synthetic.rgb_u8(32, 48, seed=4)).cuda()
    dst = torch.zeros((64, 96, 3), dtype=torch.uint8, device="cuda")
    # the plain FP32 form has no allocation-free entry
    p32 = ac.Processor("cuda", 0, "acnet-legacy-hdn0", precision="fp32")
    assert p32.process_device_noalloc([src], [dst]) != ac.AC_SUCCESS
    assert "FP16 or BF16" in p32.error()
    # weights not yet resident: no ordinary call in this precision so far
    p = ac.Processor("cuda", 0, "acnet-legacy-hdn0", precision="fp16")
    assert p.process_device_noalloc([src], [dst]) != ac.AC_SUCCESS
    assert "ordinary process call" in p.error()
    _ordinary(p, torch, [src])
    # batches beyond the scratch's 64 images, wrong output shape, mixed types
    assert p.process_device_noalloc([src] * 65, [dst] * 65) != ac.AC_SUCCESS
    assert "1 to 64" in p.error()
    bad = torch.zeros((64, 95, 3), dtype=torch.uint8, device="cuda")
    assert p.process_device_noalloc([src], [bad]) != ac.AC_SUCCESS
    assert "2x" in p.error()
    gray = torch.zeros((32, 48), dtype=torch.uint8, device="cuda")
    assert p.process_device_noalloc([src, gray], [dst, dst]) != ac.AC_SUCCESS
    # and a good call afterwards succeeds and clears the error
    assert p.process_device_noalloc([src], [dst], sync=True) == ac.AC_SUCCESS
    assert p.ok()
