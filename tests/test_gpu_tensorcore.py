"""Tensor-core (tcgen05) form: building-block self-test and network accuracy
(GPU required).

The FP16/BF16 forms round the 8-channel activations and the 8->8 weights to
16 bits; they are held to the precision targets of the headline workload:
PSNR >= 50 dB against the FP64 oracle on u8 outputs and agreement with the
reference CPU processor within +-1 LSB on >= 99.99 % of u8 pixels (FP16;
measured at 1080p RGB: all of them), BF16 within +-1 LSB on >= 99.5 %.
tests/test_gpu_precision.py holds the headline configuration itself.
"""
import json
import os

import numpy as np
import pytest

import anime4kcpp_gb300 as ac
import oracle
from anime4kcpp_gb300 import synthetic

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = np.load(os.path.join(HERE, "golden", "golden.npz"))
META = json.load(open(os.path.join(HERE, "golden", "golden.json")))["cases"]


@pytest.fixture(scope="module", autouse=True)
def built():
    from anime4kcpp_gb300 import build
    build.build()
    oracle.build()


def to_bits(a, bf16):
    a = np.asarray(a, np.float32)
    if bf16:
        u = a.view(np.uint32)
        return ((u + 0x7FFF + ((u >> 16) & 1)) >> 16).astype(np.uint16)
    return a.astype(np.float16).view(np.uint16)


def from_bits(b, bf16):
    if bf16:
        return (b.astype(np.uint32) << 16).view(np.float32)
    return b.view(np.float16).astype(np.float32)


@pytest.mark.parametrize("bf16", [False, True])
@pytest.mark.parametrize("shift,k", [(128, 32), (1, 16), (37, 32), (64, 64)])
def test_tcgen05_tile_selftest(shift, k, bf16):
    rng = np.random.default_rng(shift * 7 + k)
    px = 128 + (k // 8 - 1) * shift + 8
    x = to_bits(rng.uniform(-1, 1, size=(px, 8)), bf16)
    b = to_bits(rng.uniform(-1, 1, size=(16, k)), bf16)
    rc, d = ac.tc_selftest(x, b, shift, bf16)
    assert rc == 0
    xf, bf = from_bits(x, bf16).astype(np.float64), from_bits(b, bf16).astype(np.float64)
    a = np.zeros((128, k))
    for kk in range(k):
        a[:, kk] = xf[np.arange(128) + (kk // 8) * shift, kk % 8]
    want = a @ bf.T
    assert np.abs(d - want).max() <= 1e-4 * max(1.0, np.abs(want).max())


def psnr(got_u8, ref_f64):
    err = got_u8.astype(np.float64) / 255.0 - np.clip(ref_f64, 0.0, 1.0)
    mse = np.mean(err * err)
    return 99.0 if mse == 0 else 10 * np.log10(1.0 / mse)


@pytest.mark.parametrize("kernel", ["3", "4"])
@pytest.mark.parametrize("form", ["fp16", "bf16"])
@pytest.mark.parametrize("shape", [(67, 95), (46, 46), (47, 93), (1, 30), (30, 1), (140, 200), (45, 49), (89, 97)])
def test_tc_luma_vs_fp64_oracle(form, shape, kernel, monkeypatch):
    """kernel "3": persistent warp-specialised pipeline over pixel pairs;
    "4" (default): its quad form (four pixels per GEMM row, B matrices
    streamed per layer)."""
    monkeypatch.setenv("AC_GB300_TC_KERNEL", kernel)
    h, w = shape
    x = synthetic.luma(h, w, np.uint8, seed=h * 131 + w)
    ref64 = oracle.process_f64(x, "acnet-legacy-hdn1")
    ref32 = oracle.process(x, 2.0, "acnet-legacy-hdn1")
    p = ac.Processor("cuda", 0, "acnet-legacy-hdn1", precision=form)
    got = p.process(x, 2.0)
    assert p.ok(), p.error()
    d = np.abs(got.astype(int) - ref32.astype(int))
    if form == "fp16":
        assert psnr(got, ref64) >= 50.0
        assert (d <= 1).mean() >= 0.99
        assert d.max() <= 4
    else:
        assert psnr(got, ref64) >= 40.0
        assert d.max() <= 16


@pytest.mark.parametrize("kernel", ["3", "4"])
@pytest.mark.parametrize("form", ["fp16", "bf16"])
def test_tc_rgb_full_hd(form, kernel, monkeypatch):
    monkeypatch.setenv("AC_GB300_TC_KERNEL", kernel)
    x = synthetic.rgb_u8(1080, 1920, cells=64, seed=2024)
    ref32 = oracle.process(x, 2.0, "acnet-legacy-hdn0")
    p = ac.Processor("cuda", 0, "acnet-legacy-hdn0", precision=form)
    got = p.process(x, 2.0)
    assert p.ok(), p.error()
    d = np.abs(got.astype(int) - ref32.astype(int))
    if form == "fp16":
        # measured on this configuration: every sample within 1 LSB
        assert (d <= 1).mean() >= 0.9999
        assert d.max() <= 2
    else:
        assert (d <= 1).mean() >= 0.995 and d.max() <= 8


@pytest.mark.parametrize("kernel", ["3", "4"])
@pytest.mark.parametrize("case", [c for c in META if "arnet" not in c["model"]], ids=lambda c: c["name"])
def test_tc_golden_fp16(case, kernel, monkeypatch):
    monkeypatch.setenv("AC_GB300_TC_KERNEL", kernel)
    x = GOLD[case["name"] + "/in"]
    want = GOLD[case["name"] + "/generic"]
    p = ac.Processor("cuda", 0, case["model"], precision="fp16")
    got = p.process(x, case["factor"])
    assert p.ok(), p.error()
    d = np.abs(got.astype(np.float64) - want.astype(np.float64))
    if x.dtype == np.float32:
        assert d.max() <= 5e-3
    elif x.dtype == np.uint16:
        assert d.max() <= 6 * 257
    else:
        assert d.max() <= 6


@pytest.mark.parametrize("kernel", ["3", "4"])
@pytest.mark.parametrize("form", ["fp32", "fp16", "bf16"])
@pytest.mark.parametrize("c", [3, 4])
@pytest.mark.parametrize("dtype", ["uint8", "uint16", "float32"])
def test_fused_colour_path_matches_unfused(form, c, dtype, kernel, monkeypatch):
    """RGB(A) x2 runs split + CNN + chroma resample + merge in one kernel; the
    result must equal the separate split / CNN / merge kernels bit for bit."""
    if form == "fp32" and kernel == "4":
        pytest.skip("the FP32 form has one kernel")
    monkeypatch.setenv("AC_GB300_TC_KERNEL", kernel)
    x = synthetic.rgb_u8(61, 83, seed=5, alpha=(c == 4))
    if dtype == "uint16":
        x = (x.astype(np.uint16) * 257).astype(np.uint16)
    elif dtype == "float32":
        x = (x.astype(np.float32) / 255.0).astype(np.float32)
    outs = []
    for fused in ("1", "0"):
        monkeypatch.setenv("AC_GB300_FUSED", fused)
        p = ac.Processor("cuda", 0, "acnet-legacy-hdn2", precision=form)
        outs.append(p.process(x, 2.0))
        assert p.ok(), p.error()
    assert np.array_equal(outs[0], outs[1])


@pytest.mark.parametrize("kernel", ["3", "4"])
@pytest.mark.parametrize("c", [1, 3])
def test_persistent_kernel_independent_of_cta_count(c, kernel, monkeypatch):
    """The persistent kernel's tile queue: any number of CTAs, each taking a
    varying number of tiles (3 x 4 tiles here), gives the same bytes."""
    monkeypatch.setenv("AC_GB300_TC_KERNEL", kernel)
    if c == 1:
        x = synthetic.luma(131, 150, np.uint8, seed=17)
    else:
        x = synthetic.rgb_u8(131, 150, seed=17)
    outs = []
    for ctas in ("1", "2", "5", "0"):
        monkeypatch.setenv("AC_GB300_TC3_CTAS", ctas)
        p = ac.Processor("cuda", 0, "acnet-legacy-hdn1", precision="fp16")
        outs.append(p.process(x, 2.0))
        assert p.ok(), p.error()
    for o in outs[1:]:
        assert np.array_equal(o, outs[0])
    ref32 = oracle.process(x, 2.0, "acnet-legacy-hdn1")
    d = np.abs(outs[0].astype(int) - ref32.astype(int))
    assert (d <= 1).mean() >= 0.99 and d.max() <= 6


@pytest.mark.parametrize("form", ["fp16", "bf16"])
@pytest.mark.parametrize("c", [1, 3, 4])
def test_quad_kernel_batch_equals_single(form, c, monkeypatch):
    """The quad persistent kernel over a batch of uneven images (one launch)
    gives each image the bytes of its own launch."""
    import torch
    monkeypatch.setenv("AC_GB300_TC_KERNEL", "4")
    sizes = [(37, 53), (64, 64), (95, 140), (1, 7), (46, 46), (47, 93)]
    imgs = [synthetic.luma(h, w, np.uint8, seed=h + w) if c == 1 else synthetic.rgb_u8(h, w, seed=h + w, alpha=(c == 4))
            for h, w in sizes]
    p = ac.Processor("cuda", 0, "acnet-legacy-hdn2", precision=form)
    singles = [p.process(x, 2.0) for x in imgs]
    assert p.ok(), p.error()
    srcs = [torch.from_numpy(np.ascontiguousarray(x)).cuda() for x in imgs]
    dsts = [torch.empty((2 * x.shape[0], 2 * x.shape[1]) + x.shape[2:], dtype=torch.uint8, device="cuda") for x in imgs]
    for _ in range(3):  # direct launch, graph capture, graph replay
        p.process_batch_device(srcs, dsts, 2.0)
        assert p.ok(), p.error()
        for d, want in zip(dsts, singles):
            assert np.array_equal(d.cpu().numpy(), want)
