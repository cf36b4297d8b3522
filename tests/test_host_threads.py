"""The library's host-side threading and exception barrier, compiled on their
own (no GPU): host_parallel / host_tasks give split-independent results, carry
an exception from a worker thread to the caller after every thread has been
joined, and ABI_TRY / ABI_CATCH turn host exceptions into status codes.  These
run in the mesh, tile and coarse-space builders, where a worker exception
would otherwise end the process."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
CSRC = ROOT / "juliafem.jl_gb300" / "csrc"

SOURCE = r"""
#include "jfem_common.cuh"
#include "jfem_abi_guard.h"

#include <atomic>
#include <cstdio>
#include <stdexcept>

static int guarded(int which) {
  ABI_TRY
  if (which == 0) throw std::bad_alloc();
  if (which == 1) throw std::system_error(std::make_error_code(std::errc::resource_unavailable_try_again));
  if (which == 2) throw std::runtime_error("bad input");
  return 7;
  ABI_CATCH(nullptr)
}

int main() {
  const int64_t n = 100000;
  std::vector<int64_t> v((size_t)n, -1);
  jfem::host_parallel(n, [&](int64_t a, int64_t b) {
    for (int64_t i = a; i < b; ++i) v[(size_t)i] = 3 * i + 1;
  });
  for (int64_t i = 0; i < n; ++i)
    if (v[(size_t)i] != 3 * i + 1) { std::printf("range %lld wrong\n", (long long)i); return 1; }

  std::atomic<int64_t> done{0};
  bool caught = false;
  try {
    jfem::host_parallel(n, [&](int64_t a, int64_t b) {
      if (b == n) throw std::runtime_error("last range");   // the last range exists for any split
      done += b - a;
    });
  } catch (const std::runtime_error&) {
    caught = true;
  }
  if (!caught) { std::printf("worker exception lost\n"); return 1; }

  std::atomic<int> sum{0};
  jfem::host_tasks(7, [&](int64_t k) { sum += (int)k; });
  if (sum != 21) { std::printf("host_tasks sum %d\n", (int)sum); return 1; }

  std::string msg;
  try { throw std::bad_alloc(); } catch (...) {
    if (jfem::host_exception_status(&msg) != JFEM_ERR_OOM || msg.empty()) { std::printf("status\n"); return 1; }
  }
  if (guarded(0) != JFEM_ERR_OOM || guarded(1) != JFEM_ERR_OOM || guarded(2) != JFEM_ERR_INVALID ||
      guarded(3) != 7) { std::printf("guard codes\n"); return 1; }
  std::printf("ok\n");
  return 0;
}
"""


def test_host_threads_and_exception_barrier(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(nvcc).exists():
        pytest.skip("nvcc unavailable")
    src = tmp_path / "host_threads.cu"
    src.write_text(SOURCE)
    exe = tmp_path / "host_threads"
    r = subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-std=c++17", "-O1",
                        "--expt-relaxed-constexpr", "-I", str(CSRC), str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0 and out.stdout.strip() == "ok", out.stdout + out.stderr
