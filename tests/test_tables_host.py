"""Host-built tables of the sieve, checked on the CPU against independent
computations: the presieve tiles (every shifted copy of each tile against the
pattern computed here), the tile-prime fix-up bits, and the compile-time
constant table of the first sieving primes with their Barrett constants.
The header that defines them (voss_gb300/csrc/sieve.cuh) is compiled with the
host compiler."""
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT

W30 = [1, 7, 11, 13, 17, 19, 23, 29]
MAX_SEG = 226944          # the library's largest segment

PROBE = r"""
#include <cstdio>
#include <cstdint>
#include <vector>
#include "sieve.cuh"
using namespace vg;
int main(int argc, char** argv) {
  std::printf("first %u\n", kFirstTablePrime);
  std::printf("bits %llu\n", (unsigned long long)kTilePrimeBits);
  constexpr ConstPrimeTable ct = make_const_prime_table();
  for (uint32_t i = 0; i < kConstPrimes; ++i) std::printf("c %u %llu\n", ct.p[i], ct.m[i]);
  std::vector<uint8_t> base(kMaxTilePeriod);
  for (int t = 0; t < kTiles; ++t) {
    const uint32_t period = tile_period(t), stride = tile_copy_stride(period, %MAXSEG%u);
    std::printf("tile %d %u %u", t, period, stride);
    for (int i = 0; i < 4; ++i) std::printf(" %u", kTilePrimes[t][i]);
    std::printf("\n");
    std::vector<uint8_t> out((size_t)kTileShifts * stride);
    build_tile_copies(kTilePrimes[t], kTilePrimes[t][3] ? 4 : 3, period, stride, base.data(), out.data());
    char name[512];
    std::snprintf(name, sizeof(name), "%s/tile%d.bin", argv[1], t);
    FILE* f = std::fopen(name, "wb");
    std::fwrite(out.data(), 1, out.size(), f);
    std::fclose(f);
  }
  return 0;
}
""".replace("%MAXSEG%", str(MAX_SEG))


@pytest.fixture(scope="module")
def probe(tmp_path_factory):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not available")
    d = tmp_path_factory.mktemp("tables")
    src = d / "probe.cpp"
    src.write_text(PROBE)
    exe = d / "probe"
    subprocess.run([gxx, "-std=c++17", "-O1", "-D__host__=", "-D__device__=", "-I", str(ROOT / "voss_gb300" / "csrc"),
                    str(src), "-o", str(exe)], check=True, capture_output=True, text=True)
    out = subprocess.run([str(exe), str(d)], check=True, capture_output=True, text=True).stdout
    return d, out.splitlines()


def _primes_below(n):
    s = np.ones(n, dtype=bool)
    s[:2] = False
    for i in range(2, int(n ** 0.5) + 1):
        if s[i]:
            s[i * i::i] = False
    return np.nonzero(s)[0]


def test_tile_primes_and_fixup_bits(probe):
    _, lines = probe
    first = int(lines[0].split()[1])
    bits = int(lines[1].split()[1])
    tiles = [list(map(int, l.split()[1:])) for l in lines if l.startswith("tile ")]
    tile_primes = sorted(q for t in tiles for q in t[3:] if q)
    primes = [int(p) for p in _primes_below(200)]
    # the tiles hold exactly the primes 7 .. first-1, the table starts at the next prime
    assert tile_primes == [p for p in primes if 7 <= p < first]
    assert first in primes
    for _, period, _, *ps in tiles:
        assert period == int(np.prod([q for q in ps if q]))
    # fix-up bits: bit 8k + o set exactly for the tile primes 30k + W30[o]
    want = 0
    for q in tile_primes:
        want |= 1 << (8 * (q // 30) + W30.index(q % 30))
    assert bits == want


def test_shifted_tile_copies(probe):
    d, lines = probe
    for l in (l for l in lines if l.startswith("tile ")):
        t, period, stride, *ps = map(int, l.split()[1:])
        ps = [q for q in ps if q]
        assert stride % 16 == 0 and stride >= period + MAX_SEG + 32
        j = np.arange(period, dtype=np.int64)
        pattern = np.zeros(period, dtype=np.uint8)
        for o, w in enumerate(W30):
            x = 30 * j + w
            keep = np.ones(period, dtype=bool)
            for q in ps:
                keep &= (x % q) != 0
            pattern |= (keep.astype(np.uint8) << o)
        copies = np.fromfile(d / f"tile{t}.bin", dtype=np.uint8).reshape(16, stride)
        for c in range(16):
            idx = (np.arange(stride, dtype=np.int64) + c) % period
            assert np.array_equal(copies[c], pattern[idx]), (t, c)


def test_constant_prime_table(probe):
    _, lines = probe
    first = int(lines[0].split()[1])
    rows = [l.split()[1:] for l in lines if l.startswith("c ")]
    ps = [int(p) for p in _primes_below(20000) if p >= first][:len(rows)]
    assert len(rows) == 1024 and [int(p) for p, _ in rows] == ps
    assert all(int(m) == ((1 << 64) - 1) // p for (_, m), p in zip(rows, ps))
