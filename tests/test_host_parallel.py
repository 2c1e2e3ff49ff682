"""The host worker pool behind the scene upload's parallel loops (host_parallel.h): every item
of every range is visited exactly once, for many sizes and grains, and calls from several
host threads at once run one after another without losing work."""
import os
import shutil
import subprocess

import pytest

CSRC = os.path.join(os.path.dirname(__file__), "..", "narvalengine_gb300", "csrc")

PROGRAM = r"""
#include "host_parallel.h"
#include <atomic>
#include <cstdio>
#include <numeric>
#include <thread>
#include <vector>
int main() {
  std::atomic<int> bad{0};
  auto body = [&](int seed) {
    for (int it = 0; it < 300; it++) {
      const size_t n = 1 + (size_t)((it + seed) * 7919) % 150000;
      const size_t grain = 1 + (size_t)(it % 7) * 997;
      std::vector<int> v(n, 0);
      nehost::parallelFor(n, grain, [&](size_t b, size_t e) {
        for (size_t i = b; i < e; i++) v[i] += 1;
      });
      for (size_t i = 0; i < n; i++)
        if (v[i] != 1) { bad++; break; }
    }
  };
  body(0);
  std::thread a(body, 1), b(body, 2), c(body, 3);
  a.join(); b.join(); c.join();
  nehost::parallelFor(0, 10, [&](size_t, size_t) { bad++; });
  std::printf("%s\n", bad ? "bad" : "ok");
  return bad ? 1 : 0;
}
"""


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_worker_pool(tmp_path):
    src = tmp_path / "pool.cpp"
    src.write_text(PROGRAM)
    exe = tmp_path / "pool"
    subprocess.run(["g++", "-O2", "-std=c++17", "-pthread", "-I", CSRC, str(src), "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stdout + r.stderr
