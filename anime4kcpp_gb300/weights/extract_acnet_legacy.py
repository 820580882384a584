"""Extract the trained ACNetLegacy parameters from an Anime4KCPP source tree.

The reference ships its trained weights as generated C++ arrays
(core/internal/AC/Core/Internal/Model/Param/ACNet.p, arrays
ACNetLegacy_{GAN,HDN0..3}_NHWC_{kernels,biases}).  This script compiles a tiny
dumper that includes that file, so every value is rounded to float32 by a C++
compiler exactly as in the reference build, and writes the values to
``acnet_legacy.bin`` beside this script.

Blob layout (little endian):
    8 bytes   magic  b"ACGBW001"
    uint32    variant count (5)
    uint32    kernel floats per variant (4712)
    uint32    bias floats per variant (72)
    then for each variant in the order GAN, HDN0, HDN1, HDN2, HDN3:
        float32[4712] kernels, float32[72] biases   (reference NHWC layout,
        core/include/AC/Core/Model/ACNet.hpp:34-60)

Usage: python extract_acnet_legacy.py /path/to/Anime4KCPP
"""
import os
import struct
import subprocess
import sys
import tempfile

VARIANTS = ("GAN", "HDN0", "HDN1", "HDN2", "HDN3")
KERNELS = 8 * 9 + 8 * 8 * 9 * 8 + 8 * 4
BIASES = 8 + 8 * 8

DUMPER = r"""
#include <cstdio>
#define AC_CORE_PARAM_ALIGN 64
namespace p {
#include "AC/Core/Internal/Model/Param/ACNet.p"
}
#define DUMP(V) \
    static_assert(sizeof(p::ACNetLegacy_##V##_NHWC_kernels) == %(k)d * 4, "kernel size"); \
    static_assert(sizeof(p::ACNetLegacy_##V##_NHWC_biases) == %(b)d * 4, "bias size"); \
    std::fwrite(p::ACNetLegacy_##V##_NHWC_kernels, 4, %(k)d, f); \
    std::fwrite(p::ACNetLegacy_##V##_NHWC_biases, 4, %(b)d, f);
int main(int argc, char** argv)
{
    std::FILE* f = std::fopen(argv[1], "wb");
    if (!f) return 1;
    DUMP(GAN) DUMP(HDN0) DUMP(HDN1) DUMP(HDN2) DUMP(HDN3)
    std::fclose(f);
    return 0;
}
""" % {"k": KERNELS, "b": BIASES}


def main(ref_root):
    here = os.path.dirname(os.path.abspath(__file__))
    out = os.path.join(here, "acnet_legacy.bin")
    with tempfile.TemporaryDirectory() as tmp:
        src = os.path.join(tmp, "dump.cpp")
        exe = os.path.join(tmp, "dump")
        raw = os.path.join(tmp, "raw.bin")
        with open(src, "w") as fh:
            fh.write(DUMPER)
        subprocess.check_call(["g++", "-std=c++17", "-O0", "-I", os.path.join(ref_root, "core", "internal"), "-o", exe, src])
        subprocess.check_call([exe, raw])
        with open(raw, "rb") as fh:
            payload = fh.read()
    assert len(payload) == len(VARIANTS) * (KERNELS + BIASES) * 4
    with open(out, "wb") as fh:
        fh.write(b"ACGBW001")
        fh.write(struct.pack("<III", len(VARIANTS), KERNELS, BIASES))
        fh.write(payload)
    print("wrote", out, os.path.getsize(out), "bytes")


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("AC_REFERENCE_ROOT")
    if not root:
        sys.exit("usage: %s REFERENCE_ROOT (or set AC_REFERENCE_ROOT)" % sys.argv[0])
    main(root)
