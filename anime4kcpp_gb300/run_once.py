"""Run one upscale of a seeded synthetic frame through the device-pointer
entry point, a fixed number of times (used for kernel profiling).

    python -m anime4kcpp_gb300.run_once --form fp16 --size 1920x1080 --channels 3 --repeat 2
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
    src = torch.from_numpy(x).cuda()
    dst = torch.empty((oh, ow) + ((a.channels,) if a.channels > 1 else ()), dtype=torch.uint8, device="cuda")
    p = ac.Processor("cuda", 0, a.model, precision=a.form)
    for _ in range(a.repeat):
        p.process_device(src, dst, a.factor)
    torch.cuda.synchronize()
    print("ok", a.form, a.size, a.channels, "launches", ac.launch_count())


if __name__ == "__main__":
    main()
