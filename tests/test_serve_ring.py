"""The serving rings (bepuphysics1_gb300/csrc/ring.h) under concurrent
producers and consumers: every value arrives exactly once, pushes fail only
when full and pops only when empty.  Compiled here with the host compiler."""
import os
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]

PROGRAM = r"""
#include "ring.h"
#include <atomic>
#include <cstdio>
#include <thread>
#include <vector>
int main() {
    using bepugpu::Ring;
    Ring<int> small(4);
    for (int i = 0; i < 4; i++) if (!small.Push(i)) return 1;
    if (small.Push(9)) return 2;              // full
    int v;
    for (int i = 0; i < 4; i++) if (!small.Pop(v) || v != i) return 3;  // FIFO
    if (small.Pop(v)) return 4;               // empty
    const int P = 4, C = 4, N = 200000;
    Ring<int> q(1024);
    std::vector<std::atomic<int>> seen(P * N);
    for (auto& s : seen) s.store(0);
    std::atomic<int> got{0};
    std::vector<std::thread> ts;
    for (int p = 0; p < P; p++)
        ts.emplace_back([&, p] { for (int i = 0; i < N; i++) while (!q.Push(p * N + i)) std::this_thread::yield(); });
    for (int c = 0; c < C; c++)
        ts.emplace_back([&] { int x; while (got.load() < P * N) if (q.Pop(x)) { seen[x]++; got++; } else std::this_thread::yield(); });
    for (auto& t : ts) t.join();
    for (auto& s : seen) if (s.load() != 1) return 5;
    std::puts("ok");
    return 0;
}
"""


@pytest.mark.skipif(shutil.which(os.environ.get("CXX", "g++")) is None, reason="no host C++ compiler")
def test_ring_concurrent(tmp_path):
    src = tmp_path / "ring_test.cpp"
    src.write_text(PROGRAM)
    exe = tmp_path / "ring_test"
    cxx = os.environ.get("CXX", "g++")
    subprocess.run([cxx, "-O2", "-std=c++17", "-pthread", "-I", str(ROOT / "bepuphysics1_gb300" / "csrc"), str(src),
                    "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == "ok", (r.returncode, r.stdout, r.stderr)
