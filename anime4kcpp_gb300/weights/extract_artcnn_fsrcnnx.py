"""Extract the trained ArtCNN and FSRCNNX parameters from an Anime4KCPP source tree.

The reference ships its trained weights as generated C++ arrays
(core/internal/AC/Core/Internal/Model/Param/ArtCNN.p, FSRCNNX.p).  This script
compiles a tiny dumper that includes those files, so every value is rounded
to float32 by a C++ compiler exactly as in the reference build, and writes
the values to ``artcnn_fsrcnnx.bin`` beside this script.

Blob layout (little endian):
    8 bytes   magic  b"ACGBW9F1"
    uint32    variant count (10)
    then for each variant (order below):
        uint32 family (1 ArtCNN, 2 FSRCNNX), uint32 F, uint32 blocks,
        uint32 kind, uint32 kernel floats, uint32 bias floats, uint32 alpha floats
        float32 kernels[], biases[], alphas[]   (reference NHWC layout:
        core/include/AC/Core/Model/ArtCNN.hpp:28-56, FSRCNNX.hpp:28-66)

Variants: ArtCNN F16 C4 {normal, DN, DS}, ArtCNN F32 C4 {normal, DN, DS},
FSRCNNX F8 {normal, DistortPlus}, FSRCNNX F16 {normal, DistortPlus}; kind is
the index within each group (core/src/Model.cpp ArtCNN / FSRCNNX ctors).

Usage: python extract_artcnn_fsrcnnx.py /path/to/Anime4KCPP
"""
import os
import struct
import subprocess
import sys
import tempfile

BLOCKS = 4
VARIANTS = [
    (1, 16, 0, "ArtCNN_C4F16"), (1, 16, 1, "ArtCNN_C4F16_DN"), (1, 16, 2, "ArtCNN_C4F16_DS"),
    (1, 32, 0, "ArtCNN_C4F32"), (1, 32, 1, "ArtCNN_C4F32_DN"), (1, 32, 2, "ArtCNN_C4F32_DS"),
    (2, 8, 0, "FSRCNNX_F8"), (2, 8, 1, "FSRCNNX_F8_DistortPlus"),
    (2, 16, 0, "FSRCNNX_F16"), (2, 16, 1, "FSRCNNX_F16_DistortPlus"),
]


def sizes(family, F, B=BLOCKS):
    if family == 1:  # ArtCNN.hpp:28-31
        return F * 9 + F * F * 9 * (B + 1) + F * 4 * 9, F + F * (B + 1) + 4, 0
    # FSRCNNX.hpp:28-33
    return F * 25 + F * F * 9 * B + F * F + F * 4 * 9, F + F * (B + 1) + 4, F * (B + 1)


def dumper():
    lines = ["#include <cstdio>", "#include <cstdint>", "#define AC_CORE_PARAM_ALIGN 64", "namespace p {",
             '#include "AC/Core/Internal/Model/Param/ArtCNN.p"', '#include "AC/Core/Internal/Model/Param/FSRCNNX.p"', "}",
             "static void put(std::FILE* f, const float* v, unsigned n) { std::fwrite(v, 4, n, f); }",
             "int main(int argc, char** argv)", "{", "    std::FILE* f = std::fopen(argv[1], \"wb\");",
             "    if (!f) return 1;"]
    for family, F, kind, name in VARIANTS:
        nk, nb, na = sizes(family, F)
        pre = "p::%s_NHWC_" % name
        lines += ["    static_assert(sizeof(%skernels) == %d * 4, \"kernels\");" % (pre, nk),
                  "    static_assert(sizeof(%sbiases) == %d * 4, \"biases\");" % (pre, nb),
                  "    { uint32_t h[7] = {%d, %d, %d, %d, %d, %d, %d}; std::fwrite(h, 4, 7, f); }"
                  % (family, F, BLOCKS, kind, nk, nb, na),
                  "    put(f, %skernels, %d); put(f, %sbiases, %d);" % (pre, nk, pre, nb)]
        if na:
            lines += ["    static_assert(sizeof(%salphas) == %d * 4, \"alphas\");" % (pre, na),
                      "    put(f, %salphas, %d);" % (pre, na)]
    lines += ["    std::fclose(f);", "    return 0;", "}", ""]
    return "\n".join(lines)


def main(ref_root):
    here = os.path.dirname(os.path.abspath(__file__))
    out = os.path.join(here, "artcnn_fsrcnnx.bin")
    with tempfile.TemporaryDirectory() as tmp:
        src = os.path.join(tmp, "dump.cpp")
        exe = os.path.join(tmp, "dump")
        raw = os.path.join(tmp, "raw.bin")
        with open(src, "w") as fh:
            fh.write(dumper())
        subprocess.check_call(["g++", "-std=c++17", "-O0", "-I", os.path.join(ref_root, "core", "internal"), "-o", exe, src])
        subprocess.check_call([exe, raw])
        with open(raw, "rb") as fh:
            payload = fh.read()
    want = sum(28 + 4 * sum(sizes(fa, F)) for fa, F, _, _ in VARIANTS)
    assert len(payload) == want, (len(payload), want)
    with open(out, "wb") as fh:
        fh.write(b"ACGBW9F1")
        fh.write(struct.pack("<I", len(VARIANTS)))
        fh.write(payload)
    print("wrote", out, os.path.getsize(out), "bytes")


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("AC_REFERENCE_ROOT")
    if not root:
        sys.exit("usage: %s REFERENCE_ROOT (or set AC_REFERENCE_ROOT)" % sys.argv[0])
    main(root)
