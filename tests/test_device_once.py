"""Host logic of the per-device one-time launch set-up (``device_once`` in
anime4kcpp_gb300/csrc/kernels.hpp), without a GPU: a small C++ program
includes the header, supplies its own ``cudaGetDevice`` (a thread-local
device index) and calls one set-up site from many threads on several
"devices".  Each device's set-up must run exactly once and every caller on
that device must get that device's result; an index beyond the table runs
the set-up on every call; a set-up that fails is not cached (device 5's
first two attempts fail, the third succeeds and is kept)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "anime4kcpp_gb300", "csrc")
CUDA_INC = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")

PROGRAM = r"""
#include <atomic>
#include <cstdio>
#include <thread>
#include <vector>

#include "kernels.hpp"

static thread_local int tls_dev = 0;
extern "C" cudaError_t cudaGetDevice(int* d)
{
    *d = tls_dev;
    return cudaSuccess;
}

static std::atomic<int> runs[128];

static acgb::LaunchSetup site()
{
    return acgb::device_once([] {
        const int n = ++runs[tls_dev];
        std::this_thread::yield();
        if (tls_dev == 5 && n <= 2) return acgb::LaunchSetup{cudaErrorInvalidValue, 0, 0};
        return acgb::LaunchSetup{cudaSuccess, 10 * tls_dev + 1, tls_dev};
    });
}

int main()
{
    std::atomic<int> bad{0};
    std::vector<std::thread> ts;
    for (int t = 0; t < 8; t++)
        ts.emplace_back([&, t] {
            for (int i = 0; i < 2000; i++)
            {
                tls_dev = (t + i) % 4;
                const acgb::LaunchSetup s = site();
                if (s.err != cudaSuccess || s.per_sm != 10 * tls_dev + 1 || s.sms != tls_dev) bad++;
            }
        });
    for (auto& t : ts) t.join();
    // beyond the table: no caching, the set-up runs every time
    tls_dev = 100;
    for (int i = 0; i < 3; i++)
        if (site().sms != 100) bad++;
    // a failing set-up is retried on the next call, a success then kept
    tls_dev = 5;
    int fails = 0;
    for (int i = 0; i < 6; i++)
    {
        const acgb::LaunchSetup s = site();
        if (s.err != cudaSuccess) fails++;
        else if (s.per_sm != 51) bad++;
    }
    std::printf("%d %d %d %d %d %d %d %d\n", bad.load(), runs[0].load(), runs[1].load(), runs[2].load(), runs[3].load(),
                runs[100].load(), runs[5].load(), fails);
    return 0;
}
"""


@pytest.mark.skipif(shutil.which("g++") is None or not os.path.isfile(os.path.join(CUDA_INC, "cuda_runtime.h")),
                    reason="needs g++ and the CUDA headers")
def test_device_once_runs_once_per_device(tmp_path):
    src = tmp_path / "device_once.cpp"
    exe = tmp_path / "device_once"
    src.write_text(PROGRAM)
    subprocess.check_call(["g++", "-std=c++17", "-O1", "-pthread", "-I" + CSRC, "-I" + CUDA_INC, str(src), "-o", str(exe)])
    out = subprocess.check_output([str(exe)], text=True).split()
    bad, r0, r1, r2, r3, r100, r5, fails5 = map(int, out)
    assert bad == 0
    assert (r0, r1, r2, r3) == (1, 1, 1, 1)
    assert r100 == 3
    assert (r5, fails5) == (3, 2)
