"""Precision of every arithmetic form on the headline and precision workloads,
against the FP64 oracle of the same path (GPU required).

The oracle (``oracle.pipeline_f64``) runs the luma network in FP64 and every
other step at the reference's own rounding points
(core/src/processor/Processor.cpp:199-276): rgb2yuv quantised to the source
type, Catmull-Rom chroma, the FP64 luma through fromFloat, yuv2rgb.  Its
``quantised`` output is what the reference would return with exact network
arithmetic; ``exact`` skips the two final roundings (PSNR reference).

Targets (the FP16 tensor-core form of the headline workload): PSNR >= 50 dB
against the FP64 oracle and +-1 LSB u8 agreement on >= 99.99 % of samples,
both against the FP64 oracle's quantised output and against the reference
CPU processor's own output (the oracle's bit-exact Generic restatement).
The BF16 form (8 mantissa bits) is held to the reference's own
cross-backend bar, PSNR > 48 dB (tests/core/src/ProcessorTest.cpp:113-217).
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


@pytest.fixture(scope="module")
def headline():
    """1920x1080 RGB u8, 64 Voronoi cells (the headline workload's frames)."""
    x = synthetic.rgb_u8(1080, 1920, cells=64, seed=2024)
    exact, quant = oracle.pipeline_f64(x, "acnet-legacy-hdn0")
    ref32 = oracle.process(x, 2.0, "acnet-legacy-hdn0")
    return x, exact, quant, ref32


def report(tag, st, extra=""):
    print("\n%s: max_abs %.6f psnr %.2f dB max_lsb %g within_1lsb %.7f %s"
          % (tag, st["max_abs"], st["psnr_db"], st["max_lsb"], st["frac_within_1lsb"], extra))


@pytest.mark.parametrize("form", ["fp16", "bf16", "fp32"])
def test_headline_1080p_rgb_vs_fp64(headline, form):
    x, exact, quant, ref32 = headline
    p = ac.Processor("cuda", 0, "acnet-legacy-hdn0", precision=form)
    got = p.process(x, 2.0)
    assert p.ok(), p.error()
    st = oracle.error_stats(got, exact, quant)
    d32 = np.abs(got.astype(int) - ref32.astype(int))
    report("1080p RGB HDN0 " + form, st, "vs reference CPU: max %d within_1 %.7f" % (d32.max(), (d32 <= 1).mean()))
    if form == "bf16":
        assert st["psnr_db"] > 48.0, st
        return
    assert st["psnr_db"] >= 50.0, st
    assert st["frac_within_1lsb"] >= 0.9999, st
    assert (d32 <= 1).mean() >= 0.9999, (d32.max(), (d32 <= 1).mean())
    assert st["max_lsb"] <= 2 and d32.max() <= 2, (st, d32.max())
    if form == "fp32":
        assert d32.max() <= 1


@pytest.mark.parametrize("form", ["fp16", "bf16", "fp32"])
def test_batched_launch_precision_equals_single(headline, form):
    """The bench's value launches 8 frames at once through the batch entry
    point; each frame's bytes equal its own launch's, so the statistics above
    hold for the batched headline too."""
    import torch
    x = headline[0]
    p = ac.Processor("cuda", 0, "acnet-legacy-hdn0", precision=form)
    single = p.process(x, 2.0)
    src = torch.from_numpy(x).cuda()
    frames = [src, torch.roll(src, shifts=(5, 7), dims=(0, 1)).contiguous()]
    dsts = [torch.empty((2160, 3840, 3), dtype=torch.uint8, device="cuda") for _ in frames]
    p.process_batch_device(frames, dsts, 2.0)
    assert p.ok(), p.error()
    assert np.array_equal(dsts[0].cpu().numpy(), single)


@pytest.mark.parametrize("form", ["fp16", "bf16", "fp32"])
def test_f32_luma_1080p_vs_fp64(form):
    """The precision workload's 1920x1080 f32 single-channel luma (uniform
    [0, 1] plus edge structure): f32 output against the FP64 network."""
    x = synthetic.f32_luma_uniform(1080, 1920, seed=1081)
    exact, quant = oracle.pipeline_f64(x, "acnet-legacy-hdn3")
    p = ac.Processor("cuda", 0, "acnet-legacy-hdn3", precision=form)
    got = p.process(x, 2.0)
    assert p.ok(), p.error()
    st = oracle.error_stats(got, exact, quant)
    report("1080p f32 luma HDN3 " + form, st)
    tol = {"fp32": 1e-4, "fp16": 2e-3, "bf16": 2e-2}[form]
    assert st["max_abs"] <= tol, st
