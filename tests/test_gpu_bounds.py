"""Bounds of the device entry points (GPU required).

``compute-sanitizer`` is not available on the GPU pool, so out-of-bounds
writes are caught with canary guard bands: every destination image sits in a
larger device buffer filled with a canary byte pattern -- a guard before the
first row, padding after every row (a row stride wider than the row) and a
guard after the last row -- and after the call every byte outside the image
must still hold the canary.  Row strides are multiples of 256 bytes, as in
the library's own device buffers.  Odd sizes (1x1, 3x5, 17x33, 47x93, widths that
are not multiples of any tile) in every element type, channel count and
arithmetic form.

Argument checks: a zero, negative or too-small row stride is rejected by
every device entry point before anything is launched."""
import numpy as np
import pytest

import anime4kcpp_gb300 as ac
from anime4kcpp_gb300 import synthetic

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

CANARY = 0xA5
GUARD = 4096  # bytes before the first and after the last row
PAD = 96      # at least this many bytes of canary after every row

TYPES = {"uint8": (torch.uint8, ac.UINT8, 1), "uint16": (torch.uint16, ac.UINT16, 2), "float32": (torch.float32, ac.FLOAT32, 4)}


@pytest.fixture(scope="module", autouse=True)
def built():
    from anime4kcpp_gb300 import build
    build.build()


def source(h, w, c, dtype, seed):
    x = synthetic.rgb_u8(h, w, seed=seed, alpha=(c == 4)) if c > 1 else synthetic.luma(h, w, np.uint8, seed=seed)
    if dtype == "uint16":
        return (x.astype(np.uint16) * 257).astype(np.uint16)
    if dtype == "float32":
        return (x.astype(np.float32) / 255.0).astype(np.float32)
    return x


class Guarded:
    """A (h, w, c) destination inside a canary-filled byte buffer."""

    def __init__(self, h, w, c, dtype):
        tdt, self.etype, self.es = TYPES[dtype]
        self.h, self.w, self.c, self.dtype = h, w, c, dtype
        self.row = w * c * self.es
        # a 256-byte multiple, as the library's own buffers (the kernels see
        # the pitch alignment they see on the host-buffer path)
        self.stride = (self.row + PAD + 255) // 256 * 256
        self.buf = torch.full((2 * GUARD + self.stride * h,), CANARY, dtype=torch.uint8, device="cuda")

    def image(self):
        return (self.buf.data_ptr() + GUARD, self.w, self.h, self.c, self.stride, self.etype)

    def check(self):
        host = self.buf.cpu().numpy()
        body = host[GUARD:GUARD + self.stride * self.h].reshape(self.h, self.stride)
        outside = np.concatenate([host[:GUARD], host[GUARD + self.stride * self.h:], body[:, self.row:].ravel()])
        bad = np.flatnonzero(outside != CANARY)
        assert bad.size == 0, "%d guard bytes overwritten" % bad.size
        return np.ascontiguousarray(body[:, :self.row]).view(np.dtype(self.dtype)).reshape(self.h, self.w, self.c)


@pytest.mark.parametrize("form", ["fp32", "fp16", "bf16"])
@pytest.mark.parametrize("c", [1, 3, 4])
@pytest.mark.parametrize("dtype", ["uint8", "uint16", "float32"])
@pytest.mark.parametrize("shape", [(1, 1), (3, 5), (17, 33), (47, 93)])
def test_dst_guard_bands_x2(form, c, dtype, shape):
    h, w = shape
    x = source(h, w, c, dtype, seed=h * 7 + w)
    p = ac.Processor("cuda", 0, "acnet-legacy-hdn1", precision=form)
    want = p.process(x, 2.0)
    assert p.ok(), p.error()
    src = torch.from_numpy(np.ascontiguousarray(x)).cuda()
    g = Guarded(2 * h, 2 * w, c, dtype)
    p.process_device(src, g.image(), 2.0)
    assert p.ok(), p.error()
    got = g.check()
    assert np.array_equal(got.reshape(want.shape), want)


@pytest.mark.parametrize("c", [1, 3, 4])
@pytest.mark.parametrize("dtype", ["uint8", "uint16", "float32"])
def test_dst_guard_bands_split_network(c, dtype, monkeypatch):
    """The network split in two launches (AC_GB300_FUSION_DEPTH=5), one
    image and a batch, against the whole-network launch's bytes."""
    monkeypatch.setenv("AC_GB300_TC_KERNEL", "4")
    sizes = [(1, 1), (3, 5), (17, 33), (47, 93), (55, 109)]
    imgs = [source(h, w, c, dtype, seed=h + 2 * w) for h, w in sizes]
    monkeypatch.setenv("AC_GB300_FUSION_DEPTH", "9")
    p9 = ac.Processor("cuda", 0, "acnet-legacy-hdn1", precision="fp16")
    want = [p9.process(x, 2.0) for x in imgs]
    assert p9.ok(), p9.error()
    monkeypatch.setenv("AC_GB300_FUSION_DEPTH", "5")
    p = ac.Processor("cuda", 0, "acnet-legacy-hdn1", precision="fp16")
    srcs = [torch.from_numpy(np.ascontiguousarray(x)).cuda() for x in imgs]
    for s, (h, w), wv in zip(srcs, sizes, want):
        g = Guarded(2 * h, 2 * w, c, dtype)
        p.process_device(s, g.image(), 2.0)
        assert p.ok(), p.error()
        assert np.array_equal(g.check().reshape(wv.shape), wv)
    gs = [Guarded(2 * h, 2 * w, c, dtype) for h, w in sizes]
    p.process_batch_device(srcs, [g.image() for g in gs], 2.0)
    assert p.ok(), p.error()
    assert p.last_plan()["fusion_depth"] == 5
    for g, wv in zip(gs, want):
        assert np.array_equal(g.check().reshape(wv.shape), wv)


@pytest.mark.parametrize("form", ["fp32", "fp16"])
@pytest.mark.parametrize("model,factor", [("acnet-legacy-hdn0", 4.0), ("acnet-legacy-hdn0", 3.0), ("arnet-b8", 2.0),
                                          ("acnet-f8b8-hdn", 2.0), ("artcnn-c4f16", 2.0), ("fsrcnnx-f8", 2.0)])
@pytest.mark.parametrize("c", [1, 3])
def test_dst_guard_bands_other_paths(form, model, factor, c):
    h, w = 17, 33
    x = source(h, w, c, "uint8", seed=5)
    p = ac.Processor("cuda", 0, model, precision=form)
    want = p.process(x, factor)
    assert p.ok(), p.error()
    src = torch.from_numpy(np.ascontiguousarray(x)).cuda()
    g = Guarded(want.shape[0], want.shape[1], c, "uint8")
    p.process_device(src, g.image(), factor)
    assert p.ok(), p.error()
    assert np.array_equal(g.check().reshape(want.shape), want)


@pytest.mark.parametrize("form", ["fp16", "bf16"])
def test_dst_guard_bands_batch(form):
    sizes = [(1, 1), (3, 5), (17, 33), (47, 93), (46, 46)]
    imgs = [source(h, w, 3, "uint8", seed=h + w) for h, w in sizes]
    p = ac.Processor("cuda", 0, "acnet-legacy-hdn2", precision=form)
    want = [p.process(x, 2.0) for x in imgs]
    srcs = [torch.from_numpy(x).cuda() for x in imgs]
    gs = [Guarded(2 * h, 2 * w, 3, "uint8") for h, w in sizes]
    p.process_batch_device(srcs, [g.image() for g in gs], 2.0)
    assert p.ok(), p.error()
    for g, wv in zip(gs, want):
        assert np.array_equal(g.check(), wv)


def bad_images(src_t, w, h, c):
    """(src, dst) device-image tuples whose strides are invalid."""
    dst = torch.empty((2 * h, 2 * w, c), dtype=torch.uint8, device="cuda")
    good_s = (src_t.data_ptr(), w, h, c, w * c, ac.UINT8)
    good_d = (dst.data_ptr(), 2 * w, 2 * h, c, 2 * w * c, ac.UINT8)
    cases = []
    for stride in (0, -w * c, w * c - 1):
        cases.append(((src_t.data_ptr(), w, h, c, stride, ac.UINT8), good_d))
        cases.append((good_s, (dst.data_ptr(), 2 * w, 2 * h, c, stride * 2 if stride > 0 else stride, ac.UINT8)))
    return dst, cases


@pytest.mark.parametrize("entry", ["device", "batch", "noalloc"])
def test_bad_strides_rejected_before_launch(entry):
    h, w, c = 20, 30, 3
    x = source(h, w, c, "uint8", seed=1)
    src = torch.from_numpy(x).cuda()
    p = ac.Processor("cuda", 0, "acnet-legacy-hdn0", precision="fp16")
    p.process(x, 2.0)  # weights resident (the allocation-free entry needs them)
    assert p.ok(), p.error()
    dst, cases = bad_images(src, w, h, c)
    for s, d in cases:
        n0 = ac.launch_count()
        if entry == "device":
            with pytest.raises(RuntimeError):
                p.process_device(s, d, 2.0)
        elif entry == "batch":
            with pytest.raises(RuntimeError):
                p.process_batch_device([s], [d], 2.0)
        else:
            rc = p.process_device_noalloc([s], [d])
            assert rc != 0 and not p.ok()
        assert "stride" in p.error() or "row" in p.error(), p.error()
        assert ac.launch_count() == n0
    # the processor still works afterwards
    p.process_device(src, dst, 2.0)
    assert p.ok(), p.error()


def test_bad_strides_rejected_yuv():
    h, w = 20, 30
    y = torch.from_numpy(synthetic.luma(h, w, np.uint16, seed=2, bits=10)).cuda()
    u = torch.from_numpy(synthetic.luma(h // 2, w // 2, np.uint16, seed=3, bits=10)).cuda()
    oy = torch.empty((2 * h, 2 * w), dtype=torch.uint16, device="cuda")
    ou = torch.empty((h, w), dtype=torch.uint16, device="cuda")
    p = ac.Processor("cuda", 0, "acnet-legacy-hdn0", precision="fp16")
    bad_y = (y.data_ptr(), w, h, 1, 0, ac.UINT16)
    bad_u = (u.data_ptr(), w // 2, h // 2, 1, w // 2 * 2 - 2, ac.UINT16)
    for frame in ((bad_y, u, u), (y, bad_u, u)):
        n0 = ac.launch_count()
        with pytest.raises(RuntimeError):
            p.process_yuv_device([frame], [(oy, ou, ou)], 2.0, 6)
        assert "stride" in p.error() or "row" in p.error(), p.error()
        assert ac.launch_count() == n0
