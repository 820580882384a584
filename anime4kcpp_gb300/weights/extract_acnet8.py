"""Extract the trained ACNet<8> parameters from an Anime4KCPP source tree.

The reference ships its trained weights as generated C++ arrays
(core/internal/AC/Core/Internal/Model/Param/ACNet.p, arrays
ACNet_F8B{4,8,18}{,_HDN,_Box,_Box_HDN}_NHWC_{kernels,biases,alphas}).  This
script compiles a tiny dumper that includes that file, so every value is
rounded to float32 by a C++ compiler exactly as in the reference build, and
writes the values to ``acnet8.bin`` beside this script.

Blob layout (little endian):
    8 bytes   magic  b"ACGBW8F1"
    uint32    variant count (12)
    then for each variant, blocks 4, 8, 18 in turn and within each the kinds
    normal, HDN, Box, Box-HDN:
        uint32 blocks, uint32 kernel floats, uint32 bias floats, uint32 alpha floats
        float32 kernels[], biases[], alphas[]   (reference NHWC layout,
        core/include/AC/Core/Model/ACNet.hpp:63-116: kernels 8*9 + 576*B + 8*4*9,
        biases 8 + 8*B + 4, alphas 8*(B + 1))

Usage: python extract_acnet8.py /path/to/Anime4KCPP
"""
import os
import struct
import subprocess
import sys
import tempfile

BLOCKS = (4, 8, 18)
KINDS = ("", "_HDN", "_Box", "_Box_HDN")


def sizes(b):
    return 8 * 9 + 576 * b + 8 * 4 * 9, 8 + 8 * b + 4, 8 * (b + 1)


def dumper():
    lines = ["#include <cstdio>", "#include <cstdint>", "#define AC_CORE_PARAM_ALIGN 64", "namespace p {",
             '#include "AC/Core/Internal/Model/Param/ACNet.p"', "}",
             "static void put(std::FILE* f, const float* v, unsigned n) { std::fwrite(v, 4, n, f); }",
             "static void hdr(std::FILE* f, uint32_t b, uint32_t k, uint32_t c, uint32_t a)",
             "{ uint32_t h[4] = {b, k, c, a}; std::fwrite(h, 4, 4, f); }",
             "int main(int argc, char** argv)", "{", "    std::FILE* f = std::fopen(argv[1], \"wb\");",
             "    if (!f) return 1;"]
    for b in BLOCKS:
        nk, nb, na = sizes(b)
        for kind in KINDS:
            name = "p::ACNet_F8B%d%s_NHWC_" % (b, kind)
            lines += ["    static_assert(sizeof(%skernels) == %d * 4, \"kernels\");" % (name, nk),
                      "    static_assert(sizeof(%sbiases) == %d * 4, \"biases\");" % (name, nb),
                      "    static_assert(sizeof(%salphas) == %d * 4, \"alphas\");" % (name, na),
                      "    hdr(f, %d, %d, %d, %d);" % (b, nk, nb, na),
                      "    put(f, %skernels, %d); put(f, %sbiases, %d); put(f, %salphas, %d);" % (name, nk, name, nb, name, na)]
    lines += ["    std::fclose(f);", "    return 0;", "}", ""]
    return "\n".join(lines)


def main(ref_root):
    here = os.path.dirname(os.path.abspath(__file__))
    out = os.path.join(here, "acnet8.bin")
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
    want = sum(16 + 4 * sum(sizes(b)) for b in BLOCKS for _ in KINDS)
    assert len(payload) == want, (len(payload), want)
    with open(out, "wb") as fh:
        fh.write(b"ACGBW8F1")
        fh.write(struct.pack("<I", len(BLOCKS) * len(KINDS)))
        fh.write(payload)
    print("wrote", out, os.path.getsize(out), "bytes")


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("AC_REFERENCE_ROOT")
    if not root:
        sys.exit("usage: %s REFERENCE_ROOT (or set AC_REFERENCE_ROOT)" % sys.argv[0])
    main(root)
