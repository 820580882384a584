"""Generate golden vectors from the reference's own CPU processor.

Runs where the Anime4KCPP sources were compiled into ``oracle/_ref`` (``make -C
oracle ref``).  Every case feeds a seeded synthetic input to the reference's
``ac::core::Processor`` (CPU, Generic backend = arch 1, and its automatic ISA
choice = arch 0) and stores input and outputs in ``golden.npz`` with the case
list in ``golden.json``.  ACNetLegacy, ACNet<8>, ArtCNN and FSRCNNX cases use
the reference's trained parameters.  The reference's ARNet parameters are absent, so the
ARNet cases use the seeded synthetic ARNet parameters of ``oracle``; the chroma
resize inside the reference build is this project's restatement (the
reference's stb_image_resize2 is not vendored), so RGB cases pin the
colour conversion and luma path, not stb's resampler.

Usage: python tests/golden/make_golden.py
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from anime4kcpp_gb300 import synthetic  # noqa: E402

CASES = [
    # name, kind, shape (h, w[, c]), dtype, model, factor, seed
    ("gray_u8_hdn0_x2", "luma", (23, 37), "uint8", "acnet-legacy-hdn0", 2.0, 11),
    ("gray_u16_hdn1_x2", "luma", (17, 31), "uint16", "acnet-legacy-hdn1", 2.0, 12),
    ("gray_f32_hdn2_x2", "luma", (20, 24), "float32", "acnet-legacy-hdn2", 2.0, 13),
    ("gray_u8_hdn3_x2", "luma", (33, 40), "uint8", "acnet-legacy-hdn3", 2.0, 14),
    ("gray_u8_gan_x2", "luma", (16, 16), "uint8", "acnet-legacy-gan", 2.0, 15),
    ("gray_u8_hdn0_x4", "luma", (13, 21), "uint8", "acnet-legacy-hdn0", 4.0, 16),
    ("gray_u8_hdn0_x3", "luma", (13, 21), "uint8", "acnet-legacy-hdn0", 3.0, 17),
    ("gray_u8_1x1_x2", "luma", (1, 1), "uint8", "acnet-legacy-hdn0", 2.0, 18),
    ("gray_u8_1x5_x2", "luma", (1, 5), "uint8", "acnet-legacy-hdn0", 2.0, 19),
    ("gray_u8_7x1_x2", "luma", (7, 1), "uint8", "acnet-legacy-hdn0", 2.0, 20),
    ("gray_u8_2x2_x2", "luma", (2, 2), "uint8", "acnet-legacy-hdn0", 2.0, 21),
    ("rgb_u8_hdn0_x2", "rgb", (24, 36), "uint8", "acnet-legacy-hdn0", 2.0, 22),
    ("rgba_u8_hdn3_x2", "rgba", (16, 20), "uint8", "acnet-legacy-hdn3", 2.0, 23),
    ("rgb_u8_gan_x4", "rgb", (12, 16), "uint8", "acnet-legacy-gan", 4.0, 24),
    ("rgb_u16_hdn1_x2", "rgb", (14, 20), "uint16", "acnet-legacy-hdn1", 2.0, 25),
    ("rgb_f32_hdn2_x2", "rgb", (10, 12), "float32", "acnet-legacy-hdn2", 2.0, 26),
    ("gray_u16_arnet_b8_x2", "luma10", (19, 25), "uint16", "arnet-b8", 2.0, 27),
    ("gray_u16_arnet_b8_x4", "luma10", (11, 13), "uint16", "arnet-b8", 4.0, 28),
    ("gray_u8_arnet_hdn_b16_x2", "luma", (15, 18), "uint8", "arnet-hdn-b16", 2.0, 29),
    ("rgb_u8_arnet_b8_x2", "rgb", (12, 14), "uint8", "arnet-b8", 2.0, 30),
    ("gray_u8_acnet_f8b4_x2", "luma", (21, 29), "uint8", "acnet-f8b4", 2.0, 31),
    ("gray_u8_acnet_f8b8_hdn_x2", "luma", (18, 23), "uint8", "acnet-f8b8-hdn", 2.0, 32),
    ("gray_u16_acnet_f8b18_box_x2", "luma10", (13, 17), "uint16", "acnet-f8b18-box", 2.0, 33),
    ("gray_f32_acnet_box_hdn_x2", "luma", (11, 19), "float32", "acnet-box-hdn", 2.0, 34),
    ("gray_u8_acnet_f8b8_x4", "luma", (9, 14), "uint8", "acnet-f8b8", 4.0, 35),
    ("rgb_u8_acnet_f8b8_hdn_x2", "rgb", (14, 18), "uint8", "acnet-f8b8-hdn", 2.0, 36),
    ("gray_u8_acnet_1x3_x2", "luma", (1, 3), "uint8", "acnet-f8b4-hdn", 2.0, 37),
    ("gray_u8_artcnn_c4f16_x2", "luma", (21, 29), "uint8", "artcnn-c4f16", 2.0, 38),
    ("gray_f32_artcnn_c4f32_ds_x2", "luma", (11, 17), "float32", "artcnn-c4f32-ds", 2.0, 39),
    ("gray_u16_artcnn_c4f16_dn_x2", "luma10", (13, 15), "uint16", "artcnn-c4f16-dn", 2.0, 40),
    ("rgb_u8_artcnn_c4f32_x2", "rgb", (12, 14), "uint8", "artcnn-c4f32", 2.0, 41),
    ("gray_u8_fsrcnnx_f8_x2", "luma", (19, 23), "uint8", "fsrcnnx-f8", 2.0, 42),
    ("gray_u16_fsrcnnx_f16_dp_x2", "luma10", (13, 17), "uint16", "fsrcnnx-f16-dp", 2.0, 43),
    ("gray_u8_fsrcnnx_f8_x4", "luma", (9, 11), "uint8", "fsrcnnx-f8-distort", 4.0, 44),
    ("gray_u8_fsrcnnx_2x3_x2", "luma", (2, 3), "uint8", "fsrcnnx-f16", 2.0, 45),
]


def make_input(kind, shape, dtype, seed):
    h, w = shape
    if kind == "rgb":
        img = synthetic.rgb_u8(h, w, seed=seed)
        if dtype == "uint16":
            return (img.astype(np.uint16) * 257).astype(np.uint16)
        if dtype == "float32":
            return (img.astype(np.float32) / 255.0).astype(np.float32)
        return img
    if kind == "rgba":
        return synthetic.rgb_u8(h, w, seed=seed, alpha=True)
    if kind == "luma10":
        # 10-bit content shifted up by 6 as the reference CLI does for video.
        return (synthetic.luma(h, w, np.uint16, seed=seed, noise=4.0, bits=10) << 6).astype(np.uint16)
    if dtype == "float32":
        return synthetic.f32_luma_uniform(h, w, seed=seed)
    return synthetic.luma(h, w, np.dtype(dtype), seed=seed)


def main():
    if not oracle.ref_available():
        raise SystemExit("oracle/_ref/libacref.so missing: run `make -C oracle ref` where the reference sources exist")
    arrays, meta = {}, []
    for name, kind, shape, dtype, model, factor, seed in CASES:
        x = make_input(kind, shape, dtype, seed)
        generic = oracle.ref_process(x, factor, model, arch=1)
        auto = oracle.ref_process(x, factor, model, arch=0)
        arrays[name + "/in"] = x
        arrays[name + "/generic"] = generic
        arrays[name + "/auto"] = auto
        meta.append({"name": name, "model": model, "factor": factor, "dtype": dtype, "shape": list(x.shape),
                     "auto_backend": oracle.ref().acref_name(model.encode(), 0).decode()})
    np.savez_compressed(os.path.join(HERE, "golden.npz"), **arrays)
    with open(os.path.join(HERE, "golden.json"), "w") as fh:
        json.dump({"generator": "reference CPU processor built by oracle/Makefile (g++ -O3 -ffp-contract=off)",
                   "cases": meta}, fh, indent=1)
    print("wrote", len(meta), "cases")


if __name__ == "__main__":
    main()
