"""The standalone stable 16-bit sort (sl_sort_keys16) against the restated radix order (oracle sort16): identical
permutations, on random keys, heavy ties, all-equal keys, INVALID-heavy inputs, ragged sizes and the maximum tile
count of a 2^24-slot frame."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _sort(torch, keys16: np.ndarray) -> np.ndarray:
    from splatlight_gb300 import _native as N
    k = torch.from_numpy(keys16.astype(np.uint16).view(np.int16)).cuda()
    o = torch.empty(max(len(keys16), 1), dtype=torch.int32, device="cuda")
    N.check(N.lib().sl_sort_keys16(k.data_ptr(), len(keys16), o.data_ptr(), None))
    return o[: len(keys16)].cpu().numpy().view(np.uint32)


@pytest.mark.parametrize("n", [1, 2, 255, 4095, 4096, 4097, 100003, 1048609])
def test_random_keys(cuda, orc, n):
    rng = np.random.default_rng(n)
    k = rng.integers(0, 65536, n).astype(np.uint32)
    assert np.array_equal(_sort(cuda, k), orc.sort16(k))


@pytest.mark.parametrize("dist", ["ties", "equal", "invalid", "sorted", "reversed"])
def test_key_distributions(cuda, orc, dist):
    n = 300000
    rng = np.random.default_rng(1)
    k = {"ties": rng.integers(0, 7, n), "equal": np.full(n, 1234), "invalid": np.where(rng.random(n) < 0.7, 0xFFFF,
         rng.integers(0, 0xFFFE, n)), "sorted": np.arange(n) % 65536, "reversed": (n - np.arange(n)) % 65536}[dist]
    k = k.astype(np.uint32)
    assert np.array_equal(_sort(cuda, k), orc.sort16(k))


def test_large(cuda, orc):
    n = 1 << 24
    rng = np.random.default_rng(9)
    k = rng.integers(0, 65536, n).astype(np.uint32)
    got = _sort(cuda, k)
    assert np.array_equal(got, orc.sort16(k))


def _sort32(torch, keys: np.ndarray, bits: int) -> np.ndarray:
    from splatlight_gb300 import _native as N
    k = torch.from_numpy(keys.astype(np.uint32).view(np.int32)).cuda()
    before = k.clone()
    o = torch.empty(max(len(keys), 1), dtype=torch.int32, device="cuda")
    N.check(N.lib().sl_sort_keys32(k.data_ptr(), len(keys), bits, o.data_ptr(), None))
    assert torch.equal(k, before)   # the input keys are left intact
    return o[: len(keys)].cpu().numpy().view(np.uint32)


@pytest.mark.parametrize("n,bits", [(1, 8), (4097, 17), (300001, 24), (1 << 20, 32), (2_000_003, 22)])
def test_sort32_segmented_keys(cuda, n, bits):
    """32-bit keys (view id above 16 depth bits, tile ids of many views): stable order by the low `bits` bits,
    against numpy's stable argsort."""
    rng = np.random.default_rng(bits)
    k = rng.integers(0, 1 << bits, n, dtype=np.uint64).astype(np.uint32)
    k[rng.random(n) < 0.2] = k[0]          # heavy ties
    ref = np.argsort(k, kind="stable").astype(np.uint32)
    assert np.array_equal(_sort32(cuda, k, bits), ref)
