"""Run one upscale of a seeded synthetic frame through the device-pointer
entry point, a fixed number of times (used for kernel profiling); with
--batch N, N such frames per call through the batch entry point (one
persistent launch per call in the tensor-core forms).

    python -m anime4kcpp_gb300.run_once --form fp16 --size 1920x1080 --channels 3 --repeat 2
    python -m anime4kcpp_gb300.run_once --form fp16 --size 1920x1080 --channels 3 --batch 8 --repeat 2
"""
import argparse

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
    a = ap.parse_args()
    import torch

    import anime4kcpp_gb300 as ac
    from anime4kcpp_gb300 import build, synthetic
    build.build()
    w, h = (int(v) for v in a.size.split("x"))
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
