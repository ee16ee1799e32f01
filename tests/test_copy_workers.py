"""The server pool's resident host copy threads (SgCopyWorkers in
sagesim_gb300/csrc/sg_batch.h) on the CPU: every copy is exact and every part
of a split job runs once, with 0 to 7 workers and many jobs back to back. The
header is compiled into a small test program with the host C++ compiler."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "sagesim_gb300", "csrc")

PROGRAM = r"""
#include "sg_batch.h"
#include <atomic>
#include <cstdio>
#include <random>
int main()
{
    std::mt19937_64 rng(7);
    for (unsigned nw : {0u, 1u, 3u, 7u}) {
        SgCopyWorkers w(nw);
        std::vector<char> src(4 << 20), dst(4 << 20);
        for (auto &c : src) c = (char)rng();
        for (int it = 0; it < 200; ++it) {
            const size_t off = rng() % 64, len = rng() % (src.size() - off);
            std::fill(dst.begin(), dst.end(), 0);
            w.copy(dst.data() + off, src.data() + off, len);
            if (memcmp(dst.data() + off, src.data() + off, len) != 0) return 1;
            if (len + off < dst.size() && dst[len + off] != 0) return 2;
            const unsigned parts = 1 + (unsigned)(rng() % 20);
            std::vector<int> hit(parts, 0);
            w.run_parts(parts, [&](unsigned k) { hit[k]++; });
            for (int h : hit)
                if (h != 1) return 3;
        }
    }
    std::puts("ok");
    return 0;
}
"""


def _cuda_include():
    for cand in (os.environ.get("CUDA_HOME", ""), "/usr/local/cuda"):
        inc = os.path.join(cand, "include")
        if cand and os.path.exists(os.path.join(inc, "cuda_runtime.h")):
            return inc
    nvcc = shutil.which("nvcc")
    if nvcc:
        inc = os.path.join(os.path.dirname(os.path.dirname(nvcc)), "include")
        if os.path.exists(os.path.join(inc, "cuda_runtime.h")):
            return inc
    return None


def test_copy_workers_exact_and_each_part_once(tmp_path):
    cxx = shutil.which("g++")
    inc = _cuda_include()
    if not cxx or not inc:
        pytest.skip("needs g++ and the CUDA headers")
    src = tmp_path / "cw.cpp"
    src.write_text(PROGRAM)
    exe = tmp_path / "cw"
    subprocess.run([cxx, "-O2", "-std=c++17", "-pthread", "-I" + inc, "-I" + CSRC, str(src), "-o", str(exe)],
                   check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0 and out.stdout.strip() == "ok", (out.returncode, out.stdout, out.stderr)
