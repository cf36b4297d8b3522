"""Host-side C++ pieces of the library, compiled on their own (no GPU): the
threading helpers and the exception barrier — host_parallel / host_tasks give
split-independent results and carry an exception from a worker thread to the
caller after every thread has been joined, and ABI_TRY / ABI_CATCH turn host
exceptions into status codes (they run in the mesh, tile and coarse-space
builders, where a worker exception would otherwise end the process) — and the
rule by which the batched solver accepts an autotuner cache entry."""
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


TUNE_SOURCE = r"""
#include "jfem_tune.h"
#include <cstdio>
#include <limits>

int main() {
  using jfem::TuneEntry;
  // what the autotuner stores: single-CTA teams, or single-CTA plus clustered
  const TuneEntry good[] = {{512, 1, 1, 0, 0, 1, 88.9}, {128, 4, 1, 0, 0, 1, 0.0}, {1024, 2, 1, 0, 0, 1, 5.0},
                            {512, 1, 4, 256, 2, 1, 88.9}, {256, 2, 8, 512, 8, 2, 1.0}};
  // anything else is not launched
  const TuneEntry bad[] = {{96, 1, 1, 0, 0, 1, 1.0},    {512, 0, 1, 0, 0, 1, 1.0},   {1024, 4, 1, 0, 0, 1, 1.0},
                           {512, 1, 3, 256, 2, 1, 1.0},  {512, 1, 16, 256, 2, 1, 1.0}, {512, 1, 4, 128, 2, 1, 1.0},
                           {512, 1, 4, 256, 3, 1, 1.0},  {512, 1, 4, 256, 0, 1, 1.0},  {512, 1, 4, 256, 2, 4, 1.0},
                           {512, 1, 1, 256, 0, 1, 1.0},  {512, 1, 1, 0, 2, 1, 1.0},    {512, 1, 1, 0, 0, 1, -1.0},
                           {512, 1, 1, 0, 0, 1, std::numeric_limits<double>::quiet_NaN()}};
  for (const TuneEntry& e : good)
    if (!jfem::tune_entry_valid(e)) { std::printf("rejected bs %d\n", e.bs); return 1; }
  int k = 0;
  for (const TuneEntry& e : bad) {
    if (jfem::tune_entry_valid(e)) { std::printf("accepted bad entry %d\n", k); return 1; }
    ++k;
  }
  std::printf("ok\n");
  return 0;
}
"""


def test_autotuner_cache_entries_are_validated(tmp_path):
    """The batched solver launches a cached autotuner entry only when it is one
    of the configurations the autotuner can choose (csrc/jfem_tune.h)."""
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ unavailable")
    src = tmp_path / "tune.cpp"
    src.write_text(TUNE_SOURCE)
    exe = tmp_path / "tune"
    r = subprocess.run([gxx, "-std=c++17", "-O1", "-I", str(CSRC), str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert out.returncode == 0 and out.stdout.strip() == "ok", out.stdout + out.stderr
