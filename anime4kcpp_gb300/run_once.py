"""Run one upscale of a seeded synthetic frame through the device-pointer
entry point, a fixed number of times (used for kernel profiling); with
--batch N, N such frames per call through the batch entry point (one
persistent launch per call in the tensor-core forms); with --yuv, one planar
10-bit YUV 4:2:0 frame in u16 through the planar entry point (Y shifted by
6 bits around the network, chroma resized).

    python -m anime4kcpp_gb300.run_once --form fp16 --size 1920x1080 --channels 3 --repeat 2
    python -m anime4kcpp_gb300.run_once --form fp16 --size 1920x1080 --channels 3 --batch 8 --repeat 2
    python -m anime4kcpp_gb300.run_once --form fp16 --model arnet-b8 --size 1920x1080 --yuv --factor 4 --repeat 2

--fusion-depth 9 or 5 forces the quad kernel's plan (the whole network in
one launch, or split in two launches) instead of the autotuner's choice.
"""
import argparse
import os

import numpy as np


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--form", default="fp16", choices=["fp32", "fp16", "bf16"])
    ap.add_argument("--model", default="acnet-legacy-hdn0")
    ap.add_argument("--size", default="1920x1080")
    ap.add_argument("--channels", type=int, default=3, choices=[1, 3, 4])
    ap.add_argument("--factor", type=float, default=2.0)
    ap.add_argument("--repeat", type=int, default=2)
    ap.add_argument("--batch", type=int, default=0, help="frames per call through the batch entry point (0: single)")
    ap.add_argument("--yuv", action="store_true", help="one planar 10-bit YUV 4:2:0 u16 frame (shift 6)")
    ap.add_argument("--fusion-depth", type=int, default=0, choices=[0, 5, 9],
                    help="quad kernel: 9 = one launch, 5 = split in two launches (0: autotuned)")
    a = ap.parse_args()
    if a.fusion_depth:
        os.environ["AC_GB300_FUSION_DEPTH"] = str(a.fusion_depth)
    import torch

    import anime4kcpp_gb300 as ac
    from anime4kcpp_gb300 import build, synthetic
    build.build()
    w, h = (int(v) for v in a.size.split("x"))
    if a.yuv:
        f = int(a.factor)
        planes = [synthetic.luma(h, w, np.uint16, seed=1, bits=10)] + \
                 [synthetic.luma(h // 2, w // 2, np.uint16, seed=2 + k, bits=10) for k in range(2)]
        frame = [torch.from_numpy(pl).cuda() for pl in planes]
        out = [torch.empty((f * pl.shape[0], f * pl.shape[1]), dtype=torch.uint16, device="cuda") for pl in planes]
        p = ac.Processor("cuda", 0, a.model, precision=a.form)
        for _ in range(a.repeat):
            p.process_yuv_device([frame], [out], a.factor, 6)
        torch.cuda.synchronize()
        print("ok yuv", a.form, a.size, "launches", ac.launch_count())
        return
    if a.channels == 1:
        x = synthetic.luma(h, w, np.uint8, seed=1)
    else:
        x = synthetic.rgb_u8(h, w, seed=1, alpha=a.channels == 4)
    ow, oh = ac.output_shape(w, h, a.channels, a.factor)
    n = max(1, a.batch)
    srcs = [torch.from_numpy(np.roll(x, 7 * i, axis=1).copy()).cuda() for i in range(n)]
    dsts = [torch.empty((oh, ow) + ((a.channels,) if a.channels > 1 else ()), dtype=torch.uint8, device="cuda")
            for _ in range(n)]
    p = ac.Processor("cuda", 0, a.model, precision=a.form)
    for _ in range(a.repeat):
        if a.batch:
            p.process_batch_device(srcs, dsts, a.factor)
        else:
            p.process_device(srcs[0], dsts[0], a.factor)
    torch.cuda.synchronize()
    print("ok", a.form, a.size, a.channels, "launches", ac.launch_count())


if __name__ == "__main__":
    main()
