"""The C-ABI library: loads, exports every declared symbol, validates like the
reference (no GPU needed for any of these)."""
import ctypes
import os
import re
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
HEADERS = sorted((ROOT / "include" / "voss").glob("*.h"))


def declared_symbols():
    names = set()
    for h in HEADERS:
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?\w+\s*\*?\s*(voss_\w+)\s*\(", text, flags=re.M):
            names.add(m.group(1))
    return names


@pytest.fixture(scope="module")
def lib():
    from conftest import build_library
    build_library()
    return ctypes.CDLL(str(ROOT / "voss_gb300" / "libvoss.so"))


def test_exports_every_declared_symbol(lib):
    names = declared_symbols()
    assert len(names) >= 50
    out = subprocess.run(["nm", "-D", "--defined-only", str(ROOT / "voss_gb300" / "libvoss.so")],
                         capture_output=True, text=True, check=True).stdout
    exported = {l.split()[-1] for l in out.splitlines() if " T " in l}
    missing = names - exported
    assert not missing, missing
    for n in names:
        getattr(lib, n)


def test_reference_symbol_set_present(lib):
    # the 38 symbols the reference exports (library/include/voss/*.h)
    ref = ("voss_free voss_get_last_error voss_strerror voss_primes_prime_count "
           "voss_primes_ctx_new voss_primes_ctx_free voss_primes_ctx_prime_count "
           "voss_primes_ctx_twins voss_primes_ctx_cousin voss_primes_ctx_sexy "
           "voss_primes_ctx_statistics voss_primes_ctx_chebyshev_bias "
           "voss_primes_ctx_large_gaps_count voss_primes_ctx_large_gaps_get "
           "voss_primes_ctx_export_csv voss_primes_ctx_set_progress voss_primes_ctx_sophie_germain "
           "voss_primes_ctx_sophie_germain_upto voss_primes_in_range voss_primes_in_range_with_limit "
           "voss_primes_nth voss_primes_next voss_primes_prev voss_primes_is_prime "
           "voss_primes_factorize voss_primes_is_mersenne_prime voss_primes_is_fermat_prime "
           "voss_primes_goldbach_count voss_primes_goldbach_partitions voss_primes_goldbach_test_upto "
           "voss_numbers_phi voss_numbers_tau voss_numbers_sigma voss_numbers_mu voss_numbers_gcd "
           "voss_numbers_lcm voss_numbers_fibonacci voss_numbers_factorial").split()
    assert len(ref) == 38
    for n in ref:
        getattr(lib, n)


def test_nth_next_prev_validation_without_gpu(lib):
    out = ctypes.c_uint64(0)
    assert lib.voss_primes_nth(ctypes.c_uint64(0), ctypes.byref(out)) == 1
    assert lib.voss_primes_nth(ctypes.c_uint64(50000001), ctypes.byref(out)) == 2
    assert lib.voss_primes_nth(ctypes.c_uint64(4), ctypes.byref(out)) == 0 and out.value == 7
    assert lib.voss_primes_next(ctypes.c_uint64(1), ctypes.byref(out)) == 0 and out.value == 2
    assert lib.voss_primes_prev(ctypes.c_uint64(2), ctypes.byref(out)) == 1
    assert lib.voss_primes_prev(ctypes.c_uint64(3), ctypes.byref(out)) == 0 and out.value == 2
    assert lib.voss_primes_next(ctypes.c_uint64(10), None) == 6


def test_error_codes_and_validation(lib):
    lib.voss_strerror.restype = ctypes.c_char_p
    lib.voss_get_last_error.restype = ctypes.c_char_p
    assert lib.voss_strerror(0) == b"OK"
    assert lib.voss_strerror(5) == b"CUDA error"
    assert lib.voss_strerror(99) == b"Unknown error"
    out = ctypes.c_uint64(999)
    # prime_count(0): INVALID_N, out untouched (test_prime_count.cpp:46-51)
    assert lib.voss_primes_prime_count(ctypes.c_uint64(0), ctypes.byref(out)) == 1
    assert out.value == 999
    assert lib.voss_primes_prime_count(ctypes.c_uint64(10**14 + 1), ctypes.byref(out)) == 2
    assert lib.voss_primes_prime_count(ctypes.c_uint64(10), None) == 6
    # N < 7 is answered without the sieve (prime_count.cu:143-145)
    assert lib.voss_primes_prime_count(ctypes.c_uint64(5), ctypes.byref(out)) == 0 and out.value == 3
    ctx = ctypes.c_void_p()
    assert lib.voss_primes_ctx_new(ctypes.c_uint64(1), 1, ctypes.byref(ctx)) == 1
    assert lib.voss_primes_ctx_new(ctypes.c_uint64(10**6), 7, ctypes.byref(ctx)) == 6
    assert lib.voss_primes_ctx_new(ctypes.c_uint64(10**6), 0, None) == 6
    assert lib.voss_primes_ctx_new(ctypes.c_uint64(10**6), 0, ctypes.byref(ctx)) == 0
    # MINIMAL: gap queries are INVALID_ARG, without touching the GPU
    assert lib.voss_primes_ctx_twins(ctx, ctypes.byref(out)) == 6
    assert b"MINIMAL" in lib.voss_get_last_error()
    lib.voss_primes_ctx_free(ctx)
    lib.voss_primes_ctx_free(None)
    arr, cnt = ctypes.POINTER(ctypes.c_uint64)(), ctypes.c_uint64(7)
    assert lib.voss_primes_goldbach_test_upto(ctypes.c_uint64(3), ctypes.byref(arr), ctypes.byref(cnt),
                                              ctypes.c_uint64(10)) == 1
    assert lib.voss_primes_goldbach_test_upto(ctypes.c_uint64(100), ctypes.byref(arr), ctypes.byref(cnt),
                                              ctypes.c_uint64(0)) == 0
    assert cnt.value == 0
    assert lib.voss_primes_in_range_with_limit(ctypes.c_uint64(1), ctypes.c_uint64(10), ctypes.c_uint64(0),
                                               ctypes.byref(arr), ctypes.byref(cnt)) == 6
    assert lib.voss_primes_in_range_with_limit(ctypes.c_uint64(1), ctypes.c_uint64(10**14 + 1),
                                               ctypes.c_uint64(5), ctypes.byref(arr), ctypes.byref(cnt)) == 2
    lib.voss_free(None)


def test_outside_entry_points_fail_loudly(lib):
    out = ctypes.c_uint64(0)
    lib.voss_get_last_error.restype = ctypes.c_char_p
    assert lib.voss_primes_is_prime(ctypes.c_uint64(5), ctypes.byref(ctypes.c_int())) == 7
    assert b"outside the sieve" in lib.voss_get_last_error()


def test_python_mirror_validation():
    import voss_gb300 as v
    with pytest.raises(TypeError):
        v.primes.prime_count("x")
    with pytest.raises(v.VossError):
        v.primes.prime_count(1)
    with pytest.raises(ValueError):
        v.Context(10**6, profile="bogus")
    c = v.Context(10**6)
    c.close()
    with pytest.raises(v.VossError):
        c.prime_count()
    with v.Context(10**6, profile="minimal") as c:
        for q in (c.twins, c.statistics, c.chebyshev, c.large_gaps, c.sophie_germain):
            with pytest.raises(v.VossError):
                q()
        assert c.profile == "minimal" and c.N == 10**6
    assert v.primes.in_range(5, 4) == []
    with pytest.raises(TypeError):
        v.primes.in_range("a", 10)
    with pytest.raises(v.VossError):
        v.conjectures.test_goldbach_upto(3)
    with pytest.raises(v.VossError):
        v.conjectures.test_goldbach_upto(10**10)
    with pytest.raises(TypeError):
        v.conjectures.test_goldbach_upto(None)


# The reference checkout, when one is available: VOSS_REFERENCE_ROOT names its
# top folder (the one holding library/).
_REF_ROOT = os.environ.get("VOSS_REFERENCE_ROOT")
REF_BINDINGS = Path(_REF_ROOT) / "library" / "bindings" / "python" if _REF_ROOT else None


@pytest.mark.skipif(REF_BINDINGS is None or not REF_BINDINGS.exists(),
                    reason="VOSS_REFERENCE_ROOT is unset or holds no library/bindings/python")
def test_reference_binding_loads_this_library(lib):
    """The unmodified reference ctypes package binds this libvoss.so and its
    validation-only behaviour matches (the reference's non-GPU tests)."""
    code = r"""
import sys, pytest
sys.path.insert(0, sys.argv[1])
import voss
assert hasattr(voss.primes, "prime_count")
with pytest.raises(TypeError): voss.primes.prime_count("hello")
with pytest.raises(voss.VossError): voss.primes.Context(0)
with pytest.raises(ValueError): voss.primes.Context(10**6, profile="invalid")
with voss.primes.Context(10**6, profile="minimal") as ctx:
    for q in (ctx.twins, ctx.statistics, ctx.chebyshev, ctx.large_gaps, ctx.sophie_germain):
        with pytest.raises(voss.VossError): q()
ctx = voss.primes.Context(10**6); ctx.close()
with pytest.raises(voss.VossError): ctx.prime_count()
assert voss.primes.in_range(5, 4) == []
with pytest.raises(voss.VossError): voss.conjectures.test_goldbach_upto(3)
print("ok")
"""
    env = dict(os.environ, VOSS_LIBRARY_PATH=str(ROOT / "voss_gb300" / "libvoss.so"))
    r = subprocess.run([sys.executable, "-c", code, str(REF_BINDINGS)], env=env, capture_output=True,
                       text=True, timeout=120)
    assert r.returncode == 0, r.stderr[-2000:]
    assert r.stdout.strip().endswith("ok")
