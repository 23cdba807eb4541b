"""Host-side logic that needs no GPU: the C ABI exports, the factor-cache
layout, the residue tricks the kernels rely on, and the replica partitioner."""
import math
import re
from pathlib import Path

import pytest

import hss

ROOT = Path(__file__).resolve().parent.parent


def test_library_exports_every_declared_symbol(built):
    header = (ROOT / "include" / "hss.h").read_text()
    declared = set(re.findall(r"^\s*(?:const\s+)?\w[\w\s\*]*?\b(hss_\w+)\s*\(", header, re.M))
    assert {"hss_open", "hss_search", "hss_close", "hss_search_many", "hss_submit"} <= declared
    lib = hss.load_library()
    missing = [name for name in sorted(declared) if not hasattr(lib, name)]
    assert not missing, missing
    assert lib.hss_version().startswith(b"hss-gb300")
    assert lib.hss_strerror(-5) == b"checkpoint does not match requested range"


def test_open_without_sm103_device_fails_loudly(built):
    """No CPU fallback: without an sm_103 device, opening a handle raises."""
    import ctypes
    lib = hss.load_library()
    count = ctypes.c_int()
    try:
        import torch  # noqa: F401
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if has_gpu:
        pytest.skip("a GPU is present")
    with pytest.raises(hss.HssError):
        hss.Search(100)
    del count


@pytest.mark.parametrize("limit,flattened,cached", [(5000, 5124, 54406), (70000, 49608, 1106318)])
def test_cache_sizes_match_reference_stderr(built, limit, flattened, cached):
    """The reference prints these sizes while preparing (gpu_search_v42.cu:
    567, 606); the cache here stores free + central only, but recomputes them."""
    info = hss.cache_inspect(limit)
    assert info["flattened"] == flattened
    assert info["cached"] == cached


def _split_primes(x):
    out, p = [], 2
    while p * p <= x:
        if x % p == 0:
            e = 0
            while x % p == 0:
                x //= p
                e += 1
            out.append((p, e))
        p += 1
    if x > 1:
        out.append((x, 1))
    return out


def _gauss_mul(a, b):
    return (a[0] * b[0] - a[1] * b[1], a[0] * b[1] + a[1] * b[0])


def _raw_set(x):
    """All Gaussian divisor products fixed(x) * prod pi^r conj(pi)^(4e-r)."""
    fixed, terms = 1, []
    for p, e in _split_primes(x):
        if p % 4 == 1:
            u = next(u for u in range(1, p) if math.isqrt(p - u * u) ** 2 == p - u * u)
            v = math.isqrt(p - u * u)
            pi, cj = (u, v), (u, -v)
            vals = []
            for r in range(4 * e + 1):
                z = (1, 0)
                for _ in range(r):
                    z = _gauss_mul(z, pi)
                for _ in range(4 * e - r):
                    z = _gauss_mul(z, cj)
                vals.append(z)
            terms.append(vals)
        else:
            fixed *= p ** (2 * e)
    out = [(fixed, 0)]
    for vals in terms:
        out = [_gauss_mul(a, b) for a in out for b in vals]
    return out


@pytest.mark.parametrize("x", [1, 2, 5, 25, 65, 325, 1105, 2197, 4225, 5525, 9945])
def test_segment_is_one_per_conjugate_pair(built, x):
    seg = hss.cache_inspect(10000, x)["segment"]
    raw = _raw_set(x)
    w = len(raw)
    assert len(seg) == (w - 1) // 2 + 1
    assert seg[-1] == (x * x, 0)                       # central value
    free = seg[:-1]
    for a, b in free:
        assert a * a + b * b == x ** 4                  # norm x^4
    keys = {(a, b) for a, b in free}
    assert len(keys) == len(free)
    assert not any((a, -b) in keys for a, b in free)   # no conjugate pairs
    assert sorted(free + [(a, -b) for a, b in free] + [(x * x, 0)]) == sorted(raw)


def test_area_gate_rotation_identity():
    """The kernels test 8D | n (D in 3, 9, 15, 45) with one multiply and a
    rotate; check the identity for every residue sum the kernels can form."""
    for d in (3, 9, 15, 45):
        inv = pow(d, -1, 1 << 32)
        q = 8 * d
        thr = 0xFFFFFFFF // q
        for n in list(range(0, 1 << 14)) + list(range((1 << 21) - 4096, 1 << 21)):
            h = (n * inv) & 0xFFFFFFFF
            rot = ((h >> 3) | (h << 29)) & 0xFFFFFFFF
            assert (rot <= thr) == (n % q == 0), (d, n)


def _generic_digits(k, exps):
    """A side's list entry k as one digit per term, decoded the general way
    (block of the first non-central term, then mixed radix over the later
    terms, the last one fastest); the central entry has every digit 2e."""
    sizes = [4 * e + 1 for e in exps]
    suffix = [math.prod(sizes[j + 1:]) for j in range(len(exps))]
    free = sum(2 * e * suffix[i] for i, e in enumerate(exps))
    if k >= free:
        return [2 * e for e in exps]
    i = 0
    while k >= 2 * exps[i] * suffix[i]:
        k -= 2 * exps[i] * suffix[i]
        i += 1
    digits = [2 * e for e in exps[:i]] + [k // suffix[i]]
    rem = k % suffix[i]
    for j in range(i + 1, len(exps)):
        digits.append(rem // suffix[j])
        rem %= suffix[j]
    return digits


def _direct_digits(k, exps):
    """The same for sides of one to three terms, in the form the warp kernel's
    list build computes it (no block search, no suffix table)."""
    if len(exps) == 1:
        return [k]
    if len(exps) == 2:
        s1, block0 = 4 * exps[1] + 1, 2 * exps[0] * (4 * exps[1] + 1)
        r = k // s1 if k < block0 else 2 * exps[0]
        return [r, k - r * s1 if k < block0 else k - block0]
    s1, s2 = 4 * exps[1] + 1, 4 * exps[2] + 1
    block0, block1 = 2 * exps[0] * s1 * s2, 2 * exps[1] * s2
    if k < block0:
        q = k // s2
        return [q // s1, q % s1, k - q * s2]
    if k < block0 + block1:
        return [2 * exps[0], (k - block0) // s2, (k - block0) % s2]
    return [2 * exps[0], 2 * exps[1], k - block0 - block1]


def test_direct_list_decode_matches_general_decode():
    """Every entry of every side of one to three terms (exponents 1..4, the
    central entry included) gets the same digits from the direct decode of
    the warp kernel's list build as from the general decode that the big-pair
    kernel and the exact path use, so both build the same values."""
    import itertools
    for count in (1, 2, 3):
        for exps in itertools.product(range(1, 5), repeat=count):
            entries = (math.prod(4 * e + 1 for e in exps) - 1) // 2 + 1
            for k in range(entries):
                assert _direct_digits(k, list(exps)) == _generic_digits(k, list(exps)), (exps, k)


def test_partition_rows_balances_pairs():
    parts = hss.partition_rows(10 ** 7, 7500000, 7500511, 4)
    assert parts[0][0] == 7500000 and parts[-1][1] == 7500511
    assert all(parts[i][1] + 1 == parts[i + 1][0] for i in range(3))
    sizes = [hss.logical_pairs(10 ** 7, a, b) for a, b in parts]
    assert sum(sizes) == 1279869696
    assert max(sizes) - min(sizes) <= 2 * 2500001
    small = hss.partition_rows(100, 1, 1, 3)
    assert [p for p in small if p[0] <= p[1]] == [(1, 1)]
