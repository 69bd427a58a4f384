"""The host thread pool of the ensemble step (xcore.jl_gb300/csrc/xc_pool.h),
compiled for the host and stressed on the CPU: across thousands of runs of
varying size, with pools smaller and larger than the job count, every index
runs exactly once and run() returns only after all of them finished."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROBE = r"""
#include <chrono>
#include <cstdio>
#include <memory>
#include <random>
#include "xc_pool.h"

int main() {
  std::mt19937 rng(7);
  for (int threads : {1, 2, 5, 16, 64}) {
    xc::WorkerPool pool(threads, 0);
    for (int rep = 0; rep < 400; ++rep) {
      const int n = (int)(rng() % 97);   // 0 .. 96 jobs
      std::unique_ptr<std::atomic<int>[]> hits(new std::atomic<int>[n > 0 ? n : 1]);
      for (int i = 0; i < n; ++i) hits[i].store(0);
      std::atomic<int> done{0};
      pool.run(n, [&](int i) {
        if (i % 11 == 0) std::this_thread::sleep_for(std::chrono::microseconds(50));
        hits[i].fetch_add(1);
        done.fetch_add(1);
      });
      if (done.load() != n) {
        std::printf("FAIL threads=%d rep=%d: run returned after %d of %d jobs\n", threads, rep, done.load(), n);
        return 1;
      }
      for (int i = 0; i < n; ++i)
        if (hits[i].load() != 1) {
          std::printf("FAIL threads=%d rep=%d: job %d ran %d times\n", threads, rep, i, hits[i].load());
          return 1;
        }
    }
  }
  std::printf("ok\n");
  return 0;
}
"""


def test_worker_pool_runs_every_job_once(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    src = tmp_path / "pool_probe.cu"
    src.write_text(PROBE)
    exe = tmp_path / "pool_probe"
    subprocess.run([nvcc, "-std=c++17", "-I", os.path.join(ROOT, "xcore.jl_gb300", "csrc"), str(src), "-o",
                    str(exe)], check=True, capture_output=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stdout + r.stderr
