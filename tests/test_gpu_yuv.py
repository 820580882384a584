"""Planar YUV frames through the device path: the reference CLI's video
recipe (cli/src/Main.cpp:183-206) -- Y shifted left, upscaled, shifted back;
chroma planes resized to their destination size with Catmull-Rom -- checked
against the oracle, and the batched x4 luma chain against the per-image path
(GPU required)."""
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


def _frame10(h, w, seed):
    """10-bit 4:2:0 planes stored LSB-aligned in u16."""
    y = synthetic.luma(h, w, np.uint16, seed=seed, noise=4.0, bits=10)
    u = synthetic.luma(h // 2, w // 2, np.uint16, seed=seed + 1, noise=4.0, bits=10)
    v = synthetic.luma(h // 2, w // 2, np.uint16, seed=seed + 2, noise=4.0, bits=10)
    return y, u, v


def _dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _run(p, frames, factor, shift):
    f = int(factor)
    src = [tuple(_dev(pl) for pl in fr) for fr in frames]
    outs = [tuple(torch.empty((f * pl.shape[0], f * pl.shape[1]) + tuple(pl.shape[2:]), dtype=pl.dtype, device="cuda")
                  for pl in fr) for fr in src]
    p.process_yuv_device(src, outs, factor, shift)
    return [tuple(o.cpu().numpy() for o in fr) for fr in outs]


def _oracle_frame(fr, factor, model, shift):
    y, planes = fr[0], fr[1:]
    ys = (y.astype(np.uint32) << shift).astype(np.uint16)
    oy = oracle.process(ys, factor, model) >> shift
    oc = [oracle.resize(pl, int(factor) * pl.shape[1], int(factor) * pl.shape[0], oracle.RESIZE_CATMULL_ROM) for pl in planes]
    return [oy] + oc


@pytest.mark.parametrize("model,factor", [("arnet-b8", 4.0), ("acnet-legacy-hdn0", 2.0)])
def test_yuv420_10bit_fp32_vs_oracle(model, factor):
    frames = [_frame10(68, 120, seed=5), _frame10(34, 46, seed=9)]
    p = ac.Processor("cuda", 0, model, precision="fp32")
    got = _run(p, frames, factor, 6)
    for fr, g in zip(frames, got):
        want = _oracle_frame(fr, factor, model, 6)
        d = np.abs(g[0].astype(int) - want[0].astype(int))
        assert d.max() <= 1
        for gc, wc in zip(g[1:], want[1:]):
            assert np.array_equal(gc, wc)


def test_yuv_nv12_fp16_batch_of_frames():
    """Y plus an interleaved UV plane, eight frames in one call, FP16 form."""
    frames = []
    for i in range(8):
        y, u, v = _frame10(90, 160, seed=20 + i)
        frames.append((y, np.ascontiguousarray(np.stack([u, v], axis=2))))
    p = ac.Processor("cuda", 0, "acnet-legacy-hdn0", precision="fp16")
    got = _run(p, frames, 2.0, 6)
    for fr, g in zip(frames, got):
        want = _oracle_frame(fr, 2.0, "acnet-legacy-hdn0", 6)
        d = np.abs(g[0].astype(int) - want[0].astype(int))
        assert (d <= 1).mean() >= 0.99 and d.max() <= 8
        assert np.array_equal(g[1], want[1])


def test_batched_x4_chain_equals_per_image():
    imgs = [synthetic.luma(h, w, np.uint16, seed=h + w) for h, w in ((70, 97), (128, 64), (45, 1))]
    p = ac.Processor("cuda", 0, "acnet-legacy-hdn3", precision="fp16")
    srcs = [_dev(x) for x in imgs]
    want = []
    dsts = []
    for s in srcs:
        d = torch.empty((4 * s.shape[0], 4 * s.shape[1]), dtype=s.dtype, device="cuda")
        p.process_device(s, d, 4.0)
        want.append(d.cpu().numpy())
        dsts.append(torch.empty_like(d))
    for call in range(2):
        launches = ac.launch_count()
        p.process_batch_device(srcs, dsts, 4.0)
        if call == 1:  # the first call also measured the plans of both passes
            assert ac.launch_count() - launches == 2  # two batched x2 passes
        for d, w in zip(dsts, want):
            assert np.array_equal(d.cpu().numpy(), w)


def test_yuv_rejects_bad_planes():
    y = _dev(synthetic.luma(32, 32, np.uint16, seed=1))
    uv = _dev(synthetic.luma(16, 16, np.uint16, seed=2))
    p = ac.Processor("cuda", 0, "acnet-legacy-hdn0", precision="fp16")
    rgb = _dev(synthetic.rgb_u8(32, 32, seed=3))
    with pytest.raises(RuntimeError, match="one channel"):
        p.process_yuv_device([(rgb, uv)], [(torch.empty((64, 64, 3), dtype=torch.uint8, device="cuda"),
                                            torch.empty((32, 32), dtype=torch.uint16, device="cuda"))], 2.0, 0)
    f32 = _dev(synthetic.f32_luma_uniform(32, 32, seed=4))
    with pytest.raises(RuntimeError, match="shift"):
        p.process_yuv_device([(f32,)], [(torch.empty((64, 64), dtype=torch.float32, device="cuda"),)], 2.0, 6)
    del y


def test_video_config_full_size():
    """The video workload at its full size: 8 frames of 1920x1080 10-bit 4:2:0
    in one call, x4 with ARNet-B8, FP16 form.  Two frames are checked: their
    chroma planes whole, their luma in two windows against the oracle on the
    input crop with a 32-pixel margin (the two x2 passes see 18 + 9 pixels):
    never more than 1 LSB of the 10-bit value off, >= 95 % exact (the exact
    fraction depends on the content: 97.6 % on these frames)."""
    H, W, n, M = 1080, 1920, 96, 32
    frames = [_frame10(H, W, seed=300 + 3 * i) for i in range(8)]
    p = ac.Processor("cuda", 0, "arnet-b8", precision="fp16")
    got = _run(p, frames, 4.0, 6)
    assert p.ok(), p.error()
    for i in (0, 5):
        y, u, v = frames[i]
        gy, gu, gv = got[i]
        assert gy.shape == (4 * H, 4 * W) and gu.shape == (2 * H, 2 * W)
        for pl, g in ((u, gu), (v, gv)):
            assert np.array_equal(g, oracle.resize(pl, 4 * pl.shape[1], 4 * pl.shape[0], oracle.RESIZE_CATMULL_ROM))
        for wy, wx in ((0, 0), (H // 2 - n // 2, W // 2 - n // 2)):
            y0, x0 = max(0, wy - M), max(0, wx - M)
            y1, x1 = min(H, wy + n + M), min(W, wx + n + M)
            crop = (y[y0:y1, x0:x1].astype(np.uint32) << 6).astype(np.uint16)
            want = oracle.process(np.ascontiguousarray(crop), 4.0, "arnet-b8") >> 6
            oy, ox = 4 * (wy - y0), 4 * (wx - x0)
            d = np.abs(gy[4 * wy:4 * (wy + n), 4 * wx:4 * (wx + n)].astype(int) -
                       want[oy:oy + 4 * n, ox:ox + 4 * n].astype(int))
            assert d.max() <= 1 and (d == 0).mean() >= 0.95, (d.max(), (d == 0).mean())


@pytest.mark.parametrize("bits,shift", [(10, 6), (12, 4)])
def test_yuv_shift_any_row_layout(bits, shift):
    """The shl / shr of Y with padded, 16-byte-aligned row strides (the
    16-byte-per-thread path, rows whose last chunk is partial) and with tight
    odd strides (element by element): the same bytes, nothing written past
    a row."""
    h, w = 37, 51
    y = synthetic.luma(h, w, np.uint16, seed=bits, noise=4.0, bits=bits)
    u = synthetic.luma(h // 2, w // 2, np.uint16, seed=bits + 1, noise=4.0, bits=bits)
    p = ac.Processor("cuda", 0, "acnet-legacy-hdn0", precision="fp16")
    outs = []
    for pad in (False, True):
        stride_in = 256 if pad else 2 * w
        stride_out = 512 if pad else 2 * 2 * w
        ybuf = torch.full((h * stride_in // 2,), 0xFFFF, dtype=torch.uint16, device="cuda")
        ybuf.view(h, stride_in // 2)[:, :w] = torch.from_numpy(y).cuda()
        obuf = torch.full((2 * h * stride_out // 2,), 0xA5A5, dtype=torch.uint16, device="cuda")
        src_y = (ybuf.data_ptr(), w, h, 1, stride_in, ac.UINT16)
        dst_y = (obuf.data_ptr(), 2 * w, 2 * h, 1, stride_out, ac.UINT16)
        su = _dev(u)
        du = torch.empty((2 * (h // 2), 2 * (w // 2)), dtype=torch.uint16, device="cuda")
        p.process_yuv_device([(src_y, su)], [(dst_y, du)], 2.0, shift)
        assert p.ok(), p.error()
        o = obuf.view(2 * h, stride_out // 2).cpu().numpy()
        assert np.all(o[:, 2 * w:] == 0xA5A5)  # padding untouched
        outs.append(o[:, :2 * w].copy())
        # the source plane is left as it was
        assert np.array_equal(ybuf.view(h, stride_in // 2)[:, :w].cpu().numpy(), y)
    assert np.array_equal(outs[0], outs[1])
    want = _oracle_frame((y, u), 2.0, "acnet-legacy-hdn0", shift)[0]
    d = np.abs(outs[0].astype(int) - want.astype(int))
    # FP16 keeps 11 significant bits: within 1 LSB of a 10-bit output, a few
    # LSB of a 12-bit one
    lsb = 1 << (bits - 10)
    assert (d <= lsb).mean() >= 0.99 and d.max() <= 8 * lsb
