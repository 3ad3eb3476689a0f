"""The per-device record of raised kernel attributes (voss_gb300/csrc/attr_cache.h),
driven on the CPU with a fake setter: the dynamic shared-memory attribute is a
per-device setting, so it must be raised once on every device a process
launches on, never skipped for a device because another one has it, never
recorded when the raise failed, and never raised twice for one size when
host threads launch at once."""
import shutil
import subprocess

import pytest

from conftest import ROOT

PROBE = r"""
#include <atomic>
#include <cstdio>
#include <thread>
#include <vector>
#include "attr_cache.h"
using namespace vg;

int main() {
  AttrCache c;
  std::atomic<int> calls[kMaxDevices] = {};
  std::atomic<int> fail_next{0};
  auto setter = [&](int dev) {
    return [&, dev](size_t) {
      calls[dev].fetch_add(1);
      if (fail_next.exchange(0)) return 1;      // a refused raise
      return 0;
    };
  };
  // device 0, then device 1 with the same size: both are raised
  const int r0 = c.ensure(0, 1000, setter(0));
  std::printf("r %d\n", r0);
  const int r1 = c.ensure(1, 1000, setter(1));
  std::printf("r %d\n", r1);
  std::printf("calls %d %d\n", calls[0].load(), calls[1].load());
  // smaller or equal sizes on a raised device: no call
  c.ensure(0, 999, setter(0));
  c.ensure(0, 1000, setter(0));
  std::printf("calls %d\n", calls[0].load());
  // a larger size raises again
  c.ensure(0, 2000, setter(0));
  std::printf("raised %zu calls %d\n", c.raised(0), calls[0].load());
  // a failed raise is reported and not recorded; the next call retries
  fail_next = 1;
  const int rc1 = c.ensure(2, 500, setter(2));
  std::printf("fail %d raised %zu\n", rc1, c.raised(2));
  const int rc2 = c.ensure(2, 500, setter(2));
  std::printf("retry %d raised %zu calls %d\n", rc2, c.raised(2), calls[2].load());
  // 16 threads on 4 fresh devices, the same size: one raise per device
  std::vector<std::thread> ts;
  for (int t = 0; t < 16; ++t)
    ts.emplace_back([&, t] {
      for (int k = 0; k < 1000; ++k) c.ensure(10 + t % 4, 4096, setter(10 + t % 4));
    });
  for (auto& th : ts) th.join();
  std::printf("threads %d %d %d %d\n", calls[10].load(), calls[11].load(), calls[12].load(), calls[13].load());
  // an out-of-table device is raised on every call
  int n = 0;
  c.ensure(-1, 10, [&](size_t) { ++n; return 0; });
  c.ensure(kMaxDevices, 10, [&](size_t) { ++n; return 0; });
  std::printf("outside %d\n", n);
  return 0;
}
"""


@pytest.fixture(scope="module")
def lines(tmp_path_factory):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not available")
    d = tmp_path_factory.mktemp("attr")
    src = d / "probe.cpp"
    src.write_text(PROBE)
    exe = d / "probe"
    subprocess.run([gxx, "-std=c++17", "-O1", "-pthread", "-I", str(ROOT / "voss_gb300" / "csrc"), str(src),
                    "-o", str(exe)], check=True, capture_output=True, text=True)
    return subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.splitlines()


def test_every_device_is_raised_once(lines):
    assert lines[0:3] == ["r 0", "r 0", "calls 1 1"]
    assert lines[3] == "calls 1"
    assert lines[4] == "raised 2000 calls 2"


def test_failed_raise_is_not_recorded(lines):
    assert lines[5] == "fail 1 raised 0"
    assert lines[6] == "retry 0 raised 500 calls 2"


def test_concurrent_threads_raise_once_per_device(lines):
    assert lines[7] == "threads 1 1 1 1"
    assert lines[8] == "outside 2"
