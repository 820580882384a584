"""TMA staging of the quad kernel's input window (GPU required).

For u8 images of 1 or 3 channels whose base and row pitch are 16-byte
aligned, the quad kernel loads each tile's haloed input window with one TMA
box load into shared memory (issued during the previous tile's last layer)
and computes the layer-0 slots and the chroma region from there; other
images load the window straight from global memory.  Both paths compute
every pixel from the same clamped window, so the bytes must agree exactly:
every tile shape, ACNet<8> B4 / B8, images smaller than one window, odd
sizes, and pitches that are not 16-byte aligned (which fall back)."""
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


def _image(h, w, c, seed):
    return synthetic.rgb_u8(h, w, seed=seed, alpha=(c == 4)) if c > 1 else synthetic.luma(h, w, np.uint8, seed=seed)


def _run(model, srcs, form, tma, monkeypatch, shape=None):
    monkeypatch.setenv("AC_GB300_TMA_IN", "1" if tma else "0")
    if shape is not None:
        monkeypatch.setenv("AC_GB300_TC3_SHAPE", str(shape))
    p = ac.Processor("cuda", 0, model, precision=form)
    dsts = [torch.empty((2 * s.shape[0], 2 * s.shape[1]) + tuple(s.shape[2:]), dtype=torch.uint8, device="cuda")
            for s in srcs]
    if len(srcs) == 1:
        p.process_device(srcs[0], dsts[0], 2.0)
    else:
        p.process_batch_device(srcs, dsts, 2.0)
    assert p.ok(), p.error()
    return [d.cpu().numpy() for d in dsts]


@pytest.mark.parametrize("form", ["fp16", "bf16"])
@pytest.mark.parametrize("shape", [0, 1, 2])
@pytest.mark.parametrize("c", [1, 3, 4])
def test_staged_equals_direct_every_shape(form, shape, c, monkeypatch):
    sizes = [(131, 150), (7, 9), (1, 1), (46, 46), (64, 200), (200, 48)]
    srcs = [torch.from_numpy(_image(h, w, c, seed=h + 3 * w)).cuda() for h, w in sizes]
    a = _run("acnet-legacy-hdn1", srcs, form, True, monkeypatch, shape)
    b = _run("acnet-legacy-hdn1", srcs, form, False, monkeypatch, shape)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


@pytest.mark.parametrize("model", ["acnet-f8b4", "acnet-f8b8-hdn"])
@pytest.mark.parametrize("c", [1, 3])
def test_staged_equals_direct_acnet8(model, c, monkeypatch):
    srcs = [torch.from_numpy(_image(h, w, c, seed=h)).cuda() for h, w in [(97, 143), (5, 3), (60, 52)]]
    a = _run(model, srcs, "fp16", True, monkeypatch)
    b = _run(model, srcs, "fp16", False, monkeypatch)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


def test_unaligned_pitch_falls_back(monkeypatch):
    """A 61-pixel-wide RGB view of a wider buffer has a 16-byte aligned base
    but a 183-byte pitch: not stageable, loaded directly, same bytes as a
    packed copy of it; mixed with stageable images in one batch."""
    big = torch.from_numpy(synthetic.rgb_u8(90, 61, seed=4)).cuda()   # pitch 183 bytes
    aligned = torch.from_numpy(synthetic.rgb_u8(90, 64, seed=5)).cuda()  # pitch 192 bytes
    a = _run("acnet-legacy-hdn0", [big, aligned], "fp16", True, monkeypatch)
    b = _run("acnet-legacy-hdn0", [big, aligned], "fp16", False, monkeypatch)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    want = oracle.process(big.cpu().numpy(), 2.0, "acnet-legacy-hdn0")
    assert np.abs(a[0].astype(int) - want.astype(int)).max() <= 2
