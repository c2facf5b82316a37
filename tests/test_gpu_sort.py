"""Radix sort through the C ABI vs the oracle's stable sorts: keys and
values bit-exact (the radix sort is stable, so unstable sort is checked
exactly too, which implies the reference's per-key multiset rule)."""
import os

import numpy as np
import pytest

from conftest import to_dev, to_host

pytestmark = pytest.mark.gpu

G = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
# tiles hold 9216 keys for 32-bit keys alone (384 threads x 24), 6144 otherwise
SIZES = [0, 1, 2, 3, 100, 4097, 6143, 6144, 6145, 9215, 9216, 9217, 12289, 18433, 100003,
         (1 << 20) + 5]


def test_golden_sort(prims):
    g = np.load(os.path.join(G, "sort.npz"))
    k, v = to_dev(g["ku"]), to_dev(np.arange(g["ku"].size, dtype=np.int32))
    prims.sort_pairs(k, v)
    np.testing.assert_array_equal(to_host(k), g["ku_sorted"])
    np.testing.assert_array_equal(to_host(v), g["ku_perm"])
    k, v = to_dev(g["kf"]), to_dev(np.arange(g["kf"].size, dtype=np.int32))
    prims.sort_pairs(k, v)
    np.testing.assert_array_equal(to_host(k), g["kf_sorted"])
    np.testing.assert_array_equal(to_host(v), g["kf_perm"])
    k = to_dev(g["k64"])
    prims.sort(k)
    np.testing.assert_array_equal(to_host(k), g["k64_sorted"])
    k = to_dev(g["k64"])
    prims.sort(k, descending=True)
    np.testing.assert_array_equal(to_host(k), g["k64_desc"])
    for desc, ks, ps in ((False, "kd_sorted", "kd_perm"), (True, "kd_desc", "kd_desc_perm")):
        k, v = to_dev(g["kd"]), to_dev(np.arange(g["kd"].size, dtype=np.int32))
        prims.sort_pairs(k, v, descending=desc)
        np.testing.assert_array_equal(to_host(k), g[ks])
        np.testing.assert_array_equal(to_host(v), g[ps])


def _keys(kt, n, seed, dup=False):
    rng = np.random.default_rng(seed)
    if dup:
        return rng.integers(-n, n + 1, n).astype(kt) if np.dtype(kt).kind != "u" else \
            rng.integers(0, 2 * n + 1, n).astype(kt)
    if np.dtype(kt).kind == "f":
        return rng.normal(0, 1, n).astype(kt)
    info = np.iinfo(kt)
    if info.bits == 64:
        return rng.integers(0, 2 ** 64, n, dtype=np.uint64).view(kt) if kt == np.int64 else \
            rng.integers(0, 2 ** 64, n, dtype=np.uint64)
    return rng.integers(info.min, info.max, n, dtype=np.int64).astype(kt)


@pytest.mark.parametrize("kt", [np.uint32, np.int32, np.float32, np.uint64, np.int64, np.float64])
def test_sort_keys_bit_exact(prims, orc, kt):
    for i, n in enumerate(SIZES):
        for dup in (False, True):
            x = _keys(kt, n, 7 * i + dup, dup)
            for desc in (False, True):
                d = to_dev(x)
                prims.sort(d, descending=desc)
                np.testing.assert_array_equal(to_host(d), orc.sort(x, descending=desc),
                                              err_msg=f"n={n} dup={dup} desc={desc}")


PAIRS = [(np.uint32, np.int32), (np.uint32, np.uint32), (np.int32, np.int32),
         (np.float32, np.int32), (np.uint64, np.int32), (np.uint64, np.int64),
         (np.int64, np.int64), (np.float64, np.int64), (np.float64, np.int32),
         (np.int64, np.int32), (np.uint32, np.int64), (np.int32, np.int64), (np.float32, np.int64)]


@pytest.mark.parametrize("kt,vt", PAIRS)
def test_sort_pairs_stable_bit_exact(prims, orc, kt, vt):
    for i, n in enumerate(SIZES):
        x = _keys(kt, n, 11 * i, dup=(i % 2 == 1))
        v = np.arange(n).astype(vt)
        for desc in (False, True):
            dk, dv = to_dev(x), to_dev(v)
            prims.sort_pairs(dk, dv, descending=desc)
            ek, ev = orc.sort_pairs(x, v, descending=desc)
            np.testing.assert_array_equal(to_host(dk), ek, err_msg=f"n={n} desc={desc}")
            np.testing.assert_array_equal(to_host(dv), ev, err_msg=f"n={n} desc={desc}")


def test_special_values_and_patterns(prims, orc):
    # infinities, extremes, sorted / reverse-sorted / constant inputs
    f = np.array([np.inf, -np.inf, 1.0, -1.0, 3.4e38, -3.4e38, 1e-45, -1e-45, 0.0] * 1000,
                 dtype=np.float32)
    for desc in (False, True):
        d = to_dev(f)
        prims.sort(d, descending=desc)
        np.testing.assert_array_equal(to_host(d), orc.sort(f, descending=desc))
    for x in (np.arange(100000, dtype=np.uint32), np.arange(100000, dtype=np.uint32)[::-1].copy(),
              np.full(100000, 7, dtype=np.uint32)):
        v = np.arange(x.size, dtype=np.int32)
        dk, dv = to_dev(x), to_dev(v)
        prims.sort_pairs(dk, dv)
        ek, ev = orc.sort_pairs(x, v)
        np.testing.assert_array_equal(to_host(dk), ek)
        np.testing.assert_array_equal(to_host(dv), ev)


def test_copy_forms_leave_input(prims, orc):
    import torch
    x = _keys(np.uint32, 300007, 5)
    d = to_dev(x)
    out = torch.empty_like(d)
    prims.sort_copy(d, out)
    np.testing.assert_array_equal(to_host(d), x)
    np.testing.assert_array_equal(to_host(out), np.sort(x))
    kf = _keys(np.float32, 300007, 6)
    v = np.arange(kf.size, dtype=np.int32)
    dk, dv = to_dev(kf), to_dev(v)
    ok, ov = torch.empty_like(dk), torch.empty_like(dv)
    prims.sort_pairs_copy(dk, dv, ok, ov, descending=True)
    ek, ev = orc.sort_pairs(kf, v, descending=True)
    np.testing.assert_array_equal(to_host(ok), ek)
    np.testing.assert_array_equal(to_host(ov), ev)
    np.testing.assert_array_equal(to_host(dk), kf)


# Mid-size sorts (2^21 + 4097 keys, 293 tiles) with special float values and
# skewed key distributions.
NG = (1 << 21) + 4097


@pytest.mark.parametrize("kt", [np.uint32, np.int32, np.float32, np.uint64, np.int64, np.float64])
def test_sort_2m_keys_bit_exact(prims, orc, kt):
    for seed, dup in ((1, False), (2, True)):
        x = _keys(kt, NG, seed, dup)
        if np.dtype(kt).kind == "f":
            # (NaN has no place under operator<; +-0.0 compare equal, so
            # floats are compared as values)
            x[:6] = [0.0, -0.0, np.inf, -np.inf, 1e-40, -1e-40]
        for desc in (False, True):
            d = to_dev(x)
            prims.sort(d, descending=desc)
            np.testing.assert_array_equal(to_host(d), orc.sort(x, descending=desc),
                                          err_msg=f"{kt} dup={dup} desc={desc}")


def test_sort_2m_out_of_place_and_offsets(prims, orc):
    import torch
    x = _keys(np.uint64, NG + 3, 5)
    src = to_dev(x)
    out = torch.empty_like(src)
    prims.sort_copy(src, out)
    np.testing.assert_array_equal(to_host(out), orc.sort(x))
    np.testing.assert_array_equal(to_host(src), x)            # input untouched
    # a view 1 element into the buffer (unaligned for the 16-byte loads)
    y = _keys(np.uint32, NG + 1, 6)
    d = to_dev(np.concatenate([np.zeros(1, np.uint32), y]))
    prims.sort(d[1:])
    np.testing.assert_array_equal(to_host(d)[1:], orc.sort(y))


@pytest.mark.parametrize("case", ["one_group", "many_big", "mixed"])
def test_sort_2m_skewed_keys(prims, orc, case):
    """Skewed keys: most keys share their top bits (one digit value per
    pass carries most of a tile), or a large share does."""
    rng = np.random.default_rng(9)
    n = NG
    if case == "one_group":      # 64-bit keys below 2^40: every key in group 0
        x = rng.integers(0, 1 << 40, n, dtype=np.uint64)
    elif case == "many_big":     # 32-bit keys over 100 top-16 values
        x = (rng.integers(0, 100, n, dtype=np.uint32) << np.uint32(16)) | \
            rng.integers(0, 1 << 16, n, dtype=np.uint32)
    else:                        # 40 % in one group, the rest spread
        x = rng.integers(0, 2 ** 32, n, dtype=np.uint64).astype(np.uint32)
        sel = rng.random(n) < 0.4
        x[sel] = (np.uint32(0x1234) << np.uint32(16)) | (x[sel] & np.uint32(0xFFFF))
    for desc in (False, True):
        d = to_dev(x)
        prims.sort(d, descending=desc)
        np.testing.assert_array_equal(to_host(d), orc.sort(x, descending=desc), err_msg=case)


# 2^26, 2^27 and 2^28 keys (2^28 is the bandwidth-sweep size): uniform
# keys, keys with few distinct top bits, and stable f32/i32 pairs with many
# equal keys, +-0.0 and infinities, ascending and descending, in place and
# out of place.  The reference is a stable torch sort of an
# order-preserving int64 key, so every key and value is compared exactly.
NL = [(1 << 26) + 777, (1 << 27) + 5, 1 << 28]


def _ord64(t):
    import torch
    if t.dtype == torch.uint32:
        return t.view(torch.int32).to(torch.int64) & 0xFFFFFFFF
    if t.dtype == torch.float32:
        b = t.view(torch.int32).to(torch.int64)
        return torch.where(b < 0, b ^ 0x7FFFFFFF, b)
    if t.dtype == torch.uint64:
        return t.view(torch.int64) ^ (-2 ** 63)
    raise TypeError(t.dtype)


def _large_input(kind, n, gen):
    import torch
    dev = "cuda"
    if kind.startswith("u32"):
        k = torch.randint(-2 ** 31, 2 ** 31, (n,), generator=gen, device=dev, dtype=torch.int32)
        if kind.endswith("skew"):            # every key below 2^16
            k = k & 0xFFFF
        return k.view(torch.uint32), None
    if kind.startswith("u64"):
        k = torch.randint(-2 ** 63, 2 ** 63 - 1, (n,), generator=gen, device=dev, dtype=torch.int64)
        if kind.endswith("skew"):            # keys below 2^40
            k = k & ((1 << 40) - 1)
        return k.view(torch.uint64), None
    k = torch.randn(n, generator=gen, device=dev, dtype=torch.float32)
    k[: n // 8] = torch.round(k[: n // 8] * 4) / 4   # many equal keys
    k[1::997] = 0.0
    k[2::997] = -0.0
    k[3::4099] = float("inf")
    k[4::4099] = float("-inf")
    if kind.endswith("skew"):                # keys in [1, 2): 128 top-16 values
        k = 1.0 + torch.rand(n, generator=gen, device=dev, dtype=torch.float32)
        k[: n // 4] = 1.5
    return k, torch.arange(n, device=dev, dtype=torch.int32)


@pytest.mark.parametrize("n", NL)
@pytest.mark.parametrize("kind", ["u32", "u64", "pairs", "u32_skew", "u64_skew", "pairs_skew"])
def test_sort_large_sizes_exact(prims, n, kind):
    import torch
    gen = torch.Generator(device="cuda")
    gen.manual_seed(n + sum(map(ord, kind)))
    k, v = _large_input(kind, n, gen)
    sint = torch.int32 if k.element_size() == 4 else torch.int64   # same-width signed view
    for desc in (False, True):
        perm = torch.sort(_ord64(k), descending=desc, stable=True).indices
        want = k.view(sint)[perm]
        if v is None:
            if desc:
                got = k.clone()
                prims.sort(got, descending=True)               # in place
            else:
                got = torch.empty_like(k)
                prims.sort_copy(k, got)                        # out of place
            assert torch.equal(got.view(sint), want), (kind, desc)
        else:
            ko, vo = k.clone(), v.clone()
            prims.sort_pairs(ko, vo, descending=desc)
            assert torch.equal(ko.view(sint), want), (kind, desc)
            assert torch.equal(vo, v[perm]), (kind, desc)        # stable: values in input order


def _digits_varying(kt, n, seed, spec):
    """Keys whose order-preserving form varies only in the digit positions
    listed in spec (byte index -> True); the other digits are one value."""
    rng = np.random.default_rng(seed)
    ut = np.uint32 if np.dtype(kt).itemsize == 4 else np.uint64
    nb = np.dtype(kt).itemsize
    u = np.zeros(n, dtype=ut)
    for b in range(nb):
        byte = rng.integers(0, 256, n, dtype=np.uint64) if spec.get(b) else np.full(n, 0x5a, np.uint64)
        u |= (byte.astype(ut) << ut(8 * b))
    return u.view(kt) if kt in (np.uint32, np.uint64) else u.view(np.dtype(kt))


# digit passes whose digit is the same for every key run as plain copies,
# decided on the device: several such passes, first and last included, in
# place and out of place, keys and pairs, ascending and descending
@pytest.mark.parametrize("kt,spec", [
    (np.uint64, {0: 1, 1: 1, 2: 1}),          # 5 of 8 passes copy
    (np.uint64, {0: 1, 1: 1, 7: 1}),          # 5 copy
    (np.uint64, {}),                          # all equal: every pass copies
    (np.uint32, {0: 1, 1: 1}),                # 2 of 4 copy, the last included
    (np.uint32, {1: 1, 3: 1}),                # the first pass copies
    (np.int64, {0: 1, 4: 1}),                 # signed: 6 copy
    (np.float64, {0: 1, 5: 1, 6: 1}),         # 5 copy (bit patterns of doubles)
])
def test_sort_constant_digits_exactly(prims, orc, kt, spec):
    n = 300007
    x = _digits_varying(kt, n, 11, spec)
    if np.dtype(kt).kind == "f":
        x = np.where(np.isnan(x), np.zeros_like(x), x)
    for desc in (False, True):
        d = to_dev(x)
        prims.sort(d, descending=desc)  # in place
        np.testing.assert_array_equal(to_host(d), orc.sort(x, descending=desc), err_msg=f"{spec} {desc}")
        v = np.arange(n, dtype=np.int32)
        dk, dv = to_dev(x), to_dev(v)
        prims.sort_pairs(dk, dv, descending=desc)
        ek, ev = orc.sort_pairs(x, v, descending=desc)
        np.testing.assert_array_equal(to_host(dk), ek)
        np.testing.assert_array_equal(to_host(dv), ev)
    if kt in (np.uint32, np.uint64):
        src = to_dev(x)
        out = to_dev(np.zeros_like(x))
        prims.sort_copy(src, out)  # out of place: the input stays
        np.testing.assert_array_equal(to_host(out), orc.sort(x))
        np.testing.assert_array_equal(to_host(src), x)
