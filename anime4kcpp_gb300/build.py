"""Build the native library ``libac_gb300.so`` in-tree with nvcc.

Every CUDA translation unit is compiled for sm_103a only
(``-gencode arch=compute_103a,code=sm_103a``); host translation units go
through nvcc to g++.  The ACNetLegacy, ACNet<8>, ArtCNN and FSRCNNX
parameters are embedded from the blobs in ``weights/`` through generated C++
sources.  Object files
are compiled in parallel and reused when newer than every source and header.

Usage: python -m anime4kcpp_gb300.build [--force] [--jobs N]
"""
import argparse
import concurrent.futures
import glob
import os
import struct
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libac_gb300.so")
NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

COMMON = ["-O3", "-std=c++17", "-lineinfo", "-I" + INCLUDE, "-I" + CSRC,
          "-Xcompiler", "-fPIC,-fvisibility=hidden,-ffp-contract=off"]


def _gen_weights():
    """weights/acnet_legacy.bin -> _build/weights_acnet_legacy.cpp."""
    src = os.path.join(HERE, "weights", "acnet_legacy.bin")
    out = os.path.join(BUILD, "weights_acnet_legacy.cpp")
    if os.path.exists(out) and os.path.getmtime(out) >= os.path.getmtime(src):
        return out
    raw = open(src, "rb").read()
    if raw[:8] != b"ACGBW001":
        raise RuntimeError("bad weight blob " + src)
    n, nk, nb = struct.unpack("<III", raw[8:20])
    words = struct.unpack("<%dI" % ((len(raw) - 20) // 4), raw[20:])
    assert len(words) == n * (nk + nb)
    lines = ["// Generated by anime4kcpp_gb300/build.py from weights/acnet_legacy.bin. Do not edit.",
             "#include <cstdint>", "namespace acgb {",
             "extern const int kAcnetLegacyVariants = %d;" % n,
             "extern const int kAcnetLegacyKernels = %d;" % nk,
             "extern const int kAcnetLegacyBiases = %d;" % nb,
             "extern const uint32_t kAcnetLegacyBlob[] = {"]
    for i in range(0, len(words), 8):
        lines.append("    " + ", ".join("0x%08xu" % w for w in words[i:i + 8]) + ",")
    lines += ["};", "}  // namespace acgb", ""]
    with open(out, "w") as fh:
        fh.write("\n".join(lines))
    return out


def _gen_blob_words(name, magic, symbol):
    """weights/<name>.bin -> _build/weights_<name>.cpp (the blob's words after
    the magic as one array; models.cpp walks its per-variant headers)."""
    src = os.path.join(HERE, "weights", name + ".bin")
    out = os.path.join(BUILD, "weights_%s.cpp" % name)
    if os.path.exists(out) and os.path.getmtime(out) >= os.path.getmtime(src):
        return out
    raw = open(src, "rb").read()
    if raw[:8] != magic:
        raise RuntimeError("bad weight blob " + src)
    words = struct.unpack("<%dI" % ((len(raw) - 8) // 4), raw[8:])
    lines = ["// Generated by anime4kcpp_gb300/build.py from weights/%s.bin. Do not edit." % name,
             "#include <cstdint>", "namespace acgb {",
             "extern const int %sWords = %d;" % (symbol, len(words)),
             "extern const uint32_t %sBlob[] = {" % symbol]
    for i in range(0, len(words), 8):
        lines.append("    " + ", ".join("0x%08xu" % w for w in words[i:i + 8]) + ",")
    lines += ["};", "}  // namespace acgb", ""]
    with open(out, "w") as fh:
        fh.write("\n".join(lines))
    return out


def _gen_weights_acnet8():
    return _gen_blob_words("acnet8", b"ACGBW8F1", "kAcnet8")


def _gen_weights_f3():
    return _gen_blob_words("artcnn_fsrcnnx", b"ACGBW9F1", "kArtFsr")


def _sources():
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))
    return srcs + [_gen_weights(), _gen_weights_acnet8(), _gen_weights_f3()]


def _headers():
    return glob.glob(os.path.join(CSRC, "*.hpp")) + glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(INCLUDE, "*.h"))


def _compile(src, force):
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    newest = max([os.path.getmtime(src)] + [os.path.getmtime(h) for h in _headers()] + [os.path.getmtime(__file__)])
    if not force and os.path.exists(obj) and os.path.getmtime(obj) >= newest:
        return obj, None
    cmd = [NVCC] + ARCH + COMMON
    if src.endswith(".cu"):
        cmd += ["-Xptxas", "-warn-spills"]
    cmd += ["-c", src, "-o", obj]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), res.stdout + res.stderr))
    return obj, (res.stdout + res.stderr).strip() or None


def build(force=False, jobs=None, verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    srcs = _sources()
    jobs = jobs or min(len(srcs), os.cpu_count() or 4)
    with concurrent.futures.ThreadPoolExecutor(max_workers=jobs) as ex:
        results = list(ex.map(lambda s: _compile(s, force), srcs))
    objs = [o for o, _ in results]
    for o, log in results:
        if log and verbose:
            print(os.path.basename(o), log, file=sys.stderr)
    newest_obj = max(os.path.getmtime(o) for o in objs)
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < newest_obj:
        tmp = LIB + ".tmp"
        # -Bsymbolic: the library's own calls bind to its own definitions, so it
        # can be loaded (RTLD_LOCAL) next to another library that exports the
        # ac::core C++ symbols (the reference core with this library as backend)
        cmd = [NVCC] + ARCH + ["-shared", "-cudart", "static", "-Xlinker", "-Bsymbolic", "-o", tmp] + objs + \
            ["-lpthread", "-ldl", "-lrt"]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), res.stdout + res.stderr))
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--jobs", type=int, default=None)
    ap.add_argument("-v", "--verbose", action="store_true")
    a = ap.parse_args()
    print(build(a.force, a.jobs, a.verbose))
