"""The C++ drop-in boundary: a small C++ program written the way a caller of
the reference's core writes it (core/include/AC/Core/Processor.hpp:15-48,
Image.hpp:359-419), compiled against this repository's include/ and linked
with libac_gb300.so.

CPU: the Image contract (stride rule, mapping without ownership, shared
copies and views, deep clones, copy in / out), and processor creation by
string and by the create<CUDA, Model> hook: never null, ok() false without
a GPU, with the reason in error(); CPU / OpenCL types give no fallback.

GPU: the same program upscales images through both factories and the
output is checked against the oracle (bit-identical to the Python / C-ABI
path of the same processor, within 1 LSB of the reference CPU processor in
the FP32 form)."""
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIBDIR = os.path.join(ROOT, "anime4kcpp_gb300")

PROGRAM = r"""
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

#include "AC/Core.hpp"

using ac::core::Image;
using ac::core::Processor;
namespace model = ac::core::model;

static int failures = 0;
#define CHECK(c) do { if (!(c)) { std::printf("FAIL %s:%d %s\n", __FILE__, __LINE__, #c); failures++; } } while (0)

static void image_contract()
{
    Image a(5, 3, 3, Image::UInt8);                 // row 15 bytes -> stride 16
    CHECK(a.width() == 5 && a.height() == 3 && a.channels() == 3 && a.stride() == 16);
    CHECK(a.elementSize() == 1 && a.pixelSize() == 3 && a.size() == 48 && a.ownership() && !a.empty());
    CHECK(a.isUint() && !a.isFloat());
    Image wide(5, 3, 3, Image::UInt8, 40);          // an explicit stride that holds a row is kept
    CHECK(wide.stride() == 40);
    Image f(7, 2, 1, Image::Float32);
    CHECK(f.stride() == 28 && f.isFloat() && f.elementSize() == 4);
    for (int y = 0; y < 3; y++)
        for (int x = 0; x < 15; x++) a.line(y)[x] = static_cast<unsigned char>(16 * y + x);
    Image b = a;                                    // copies share pixels
    CHECK(b == a && b.ptr() == a.ptr());
    Image v = a.view(1, 1, 10, 10);                 // clipped to the image, sharing
    CHECK(v.width() == 4 && v.height() == 2 && v.stride() == a.stride() && v.pixel(0, 0) == a.pixel(1, 1));
    CHECK(v.ownership() && v == a);
    CHECK(a.view(10, 10, 2, 2).empty());
    Image c = a.clone();                            // deep copy
    CHECK(c != a && c.stride() == 16 && std::memcmp(c.line(2), a.line(2), 15) == 0);
    std::vector<unsigned char> host(3 * 20, 0xEE);
    a.to(host.data(), 20);                          // rows 20 bytes apart
    CHECK(host[20] == 16 && host[34] == 30 && host[35] == 0xEE);
    Image m;
    m.map(5, 3, 3, Image::UInt8, host.data(), 20);  // no ownership, caller stride
    CHECK(!m.ownership() && m.stride() == 20 && m.ptr() == host.data());
    Image g;
    g.from(5, 3, 3, Image::UInt8, host.data(), 20); // copy in, own stride
    CHECK(g.ownership() && g.stride() == 16 && g.line(1)[0] == 16);
    Image keep = g;
    keep.create(0, 3, 1, Image::UInt8);             // invalid sizes leave the image unchanged
    CHECK(keep == g && keep.width() == 5);
    m.map(4, 4, 1, Image::UInt8, nullptr);
    CHECK(m.width() == 5);
}

static void processors_without_gpu()
{
    auto p = Processor::create("cuda", 0, "acnet-legacy-hdn0");
    CHECK(p != nullptr && p->type() == Processor::CUDA && std::string(p->typeName()) == "CUDA");
    CHECK(!p->ok() && std::strlen(p->error()) > 0);
    auto q = Processor::create<Processor::CUDA>(0, model::ACNetLegacy(model::ACNetLegacy::Variant::HDN0));
    CHECK(q != nullptr && q->type() == Processor::CUDA && !q->ok());
    auto cpu = Processor::create("cpu", 0, "acnet-legacy-hdn0");
    CHECK(cpu != nullptr && cpu->type() == Processor::CPU && !cpu->ok() && std::strlen(cpu->error()) > 0);
    auto ocl = Processor::create("opencl", 0, "acnet-legacy-hdn0");
    CHECK(ocl != nullptr && ocl->type() == Processor::OpenCL && !ocl->ok());
    Image src(8, 8, 3, Image::UInt8);
    Image out = p->process(src, 2.0);              // fails loudly, writes nothing
    CHECK(!p->ok() && out.empty());
    CHECK(std::strlen(Processor::info<Processor::CPU>()) > 0 && std::strlen(Processor::listInfo()) > 0);
}

static std::vector<unsigned char> read_file(const char* path)
{
    std::ifstream f(path, std::ios::binary);
    return std::vector<unsigned char>((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
}

// gpu <factory> <in.raw> <w> <h> <c> <factor> <out.raw>: u8 image upscale.
static int upscale(int argc, char** argv)
{
    if (argc < 9) return 2;
    const std::string factory = argv[2];
    const int w = std::atoi(argv[4]), h = std::atoi(argv[5]), c = std::atoi(argv[6]);
    const double factor = std::atof(argv[7]);
    std::vector<unsigned char> in = read_file(argv[3]);
    if (static_cast<int>(in.size()) != w * h * c) return 3;
    Image src;
    src.map(w, h, c, Image::UInt8, in.data());
    std::shared_ptr<Processor> p;
    if (factory == "hdn0") p = Processor::create<Processor::CUDA>(0, model::ACNetLegacy(model::ACNetLegacy::Variant::HDN0));
    else if (factory == "acnet8") p = Processor::create<Processor::CUDA>(0, model::ACNet<8>(model::ACNet<8>::Variant::B8_HDN));
    else if (factory == "arnet") p = Processor::create<Processor::CUDA>(0, model::ARNet<8>(model::ARNet<8>::Variant::B8_NORMAL));
    else if (factory == "artcnn") p = Processor::create<Processor::CUDA>(0, model::ArtCNN<16>(model::ArtCNN<16>::Variant::C4_NORMAL));
    else if (factory == "fsrcnnx") p = Processor::create<Processor::CUDA>(0, model::FSRCNNX<8>(model::FSRCNNX<8>::Variant::B4_NORMAL));
    else p = Processor::create("cuda", 0, factory.c_str());
    if (!p->ok()) { std::printf("create: %s\n", p->error()); return 4; }
    Image dst = p->process(src, factor);
    if (!p->ok()) { std::printf("process: %s\n", p->error()); return 5; }
    // a preallocated dst of the right shape is filled in place
    Image pre(dst.width(), dst.height(), dst.channels(), dst.type());
    p->process(src, pre, factor);
    if (!p->ok()) { std::printf("process into dst: %s\n", p->error()); return 6; }
    Image bad(dst.width() + 1, dst.height(), dst.channels(), dst.type());
    p->process(src, bad, factor);
    if (p->ok()) { std::printf("a dst of the wrong shape was accepted\n"); return 7; }
    std::vector<unsigned char> out(static_cast<size_t>(dst.width()) * dst.height() * dst.channels());
    dst.to(out.data());
    std::vector<unsigned char> out2(out.size());
    pre.to(out2.data());
    if (out != out2) { std::printf("preallocated dst differs\n"); return 8; }
    std::ofstream(argv[8], std::ios::binary).write(reinterpret_cast<const char*>(out.data()), out.size());
    std::printf("%d %d %d %s\n", dst.width(), dst.height(), dst.channels(), p->name());
    return 0;
}

int main(int argc, char** argv)
{
    if (argc > 1 && std::string(argv[1]) == "gpu") return upscale(argc, argv);
    image_contract();
    processors_without_gpu();
    std::printf("%d failures\n", failures);
    return failures ? 1 : 0;
}
"""


@pytest.fixture(scope="module")
def program(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("needs g++")
    from anime4kcpp_gb300 import build
    build.build()
    d = tmp_path_factory.mktemp("cxx")
    src, exe = d / "caller.cpp", d / "caller"
    src.write_text(PROGRAM)
    subprocess.check_call(["g++", "-std=c++17", "-O1", "-I" + os.path.join(ROOT, "include"), str(src), "-o", str(exe),
                           "-L" + LIBDIR, "-lac_gb300", "-Wl,-rpath," + LIBDIR])
    return exe


def test_cxx_program_without_gpu(program):
    """Runs with no GPU visible (CUDA_VISIBLE_DEVICES empty), so the
    processor must report failure instead of computing anything."""
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="")
    r = subprocess.run([str(program)], capture_output=True, text=True, env=env, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "0 failures" in r.stdout


@pytest.mark.gpu
@pytest.mark.parametrize("factory,model,factor,c", [
    ("hdn0", "acnet-legacy-hdn0", 2.0, 3), ("hdn0", "acnet-legacy-hdn0", 4.0, 1), ("acnet-legacy-hdn2", "acnet-legacy-hdn2", 2.0, 4),
    ("acnet8", "acnet-f8b8-hdn", 2.0, 3), ("arnet", "arnet-b8", 2.0, 1), ("artcnn", "artcnn-c4f16", 2.0, 1),
    ("fsrcnnx", "fsrcnnx-f8", 2.0, 3)])
def test_cxx_program_upscales_on_gpu(program, tmp_path, factory, model, factor, c):
    import anime4kcpp_gb300 as ac
    import oracle
    from anime4kcpp_gb300 import synthetic
    h, w = 61, 90
    x = synthetic.rgb_u8(h, w, seed=7, alpha=(c == 4)) if c > 1 else synthetic.luma(h, w, np.uint8, seed=7)
    (tmp_path / "in.raw").write_bytes(np.ascontiguousarray(x).tobytes())
    r = subprocess.run([str(program), "gpu", factory, str(tmp_path / "in.raw"), str(w), str(h), str(c), str(factor),
                        str(tmp_path / "out.raw")], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    ow, oh, oc = (int(v) for v in r.stdout.split()[:3])
    got = np.frombuffer((tmp_path / "out.raw").read_bytes(), np.uint8).reshape((oh, ow, oc) if c > 1 else (oh, ow))
    # the C++ processor is the one the C ABI and Python wrap: same bytes
    p = ac.Processor("cuda", 0, model)
    want = p.process(x, factor)
    assert p.ok(), p.error()
    assert np.array_equal(got, want.reshape(got.shape))
    ref = oracle.process(x, factor, model)
    assert np.abs(got.astype(int) - ref.astype(int)).max() <= 1
