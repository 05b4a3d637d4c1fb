"""sl_sort_keys16_noalloc -- the 16-bit key sort for callers that may not allocate device memory (a host engine
that owns all device memory through its own pool, or a latency-bound frame loop) -- must give exactly the
permutation of the allocating sl_sort_keys16 and of the CPU restatement of radix.wgsl's stable order, on
consecutive calls that share its fixed scratch array (on the default stream and on a caller's stream), and must
refuse inputs larger than that array with a clear error.  This file is collected last on purpose."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_KEYS = 1 << 20


def _run(torch, fn_name, keys, stream=None):
    from splatlight_gb300 import _native as N
    k = torch.from_numpy(keys.astype(np.uint16).view(np.int16)).cuda()
    o = torch.full((len(keys),), -1, dtype=torch.int32, device="cuda")
    handle = None
    if stream is not None:
        torch.cuda.current_stream().synchronize()   # inputs written before the caller's stream reads them
        handle = stream.cuda_stream
    rc = getattr(N.lib(), fn_name)(k.data_ptr(), len(keys), o.data_ptr(), handle)
    N.check(rc)
    if stream is not None:
        stream.synchronize()
    return o.cpu().numpy().view(np.uint32)


def _inputs():
    rng = np.random.default_rng(2024)
    return [rng.integers(0, 65536, MAX_KEYS),                                   # full size, random keys
            np.where(rng.random(300001) < 0.5, 0xFFFF, rng.integers(0, 9, 300001))]  # ragged, heavy ties


def test_noalloc_matches_allocating_sort_on_consecutive_calls(cuda):
    torch = cuda
    for keys in _inputs():                                            # two calls in a row on the shared array
        want = _run(torch, "sl_sort_keys16", keys)
        got = _run(torch, "sl_sort_keys16_noalloc", keys)
        assert np.array_equal(got, want)


def test_noalloc_on_a_caller_stream_matches_the_oracle(cuda, orc):
    torch = cuda
    stream = torch.cuda.Stream()
    for keys in _inputs():
        got = _run(torch, "sl_sort_keys16_noalloc", keys, stream=stream)
        assert np.array_equal(got, orc.sort16(keys))
        assert np.array_equal(got, _run(torch, "sl_sort_keys16", keys))


def test_noalloc_rejects_more_keys_than_its_scratch(cuda):
    torch = cuda
    from splatlight_gb300 import _native as N
    k = torch.zeros(MAX_KEYS + 1, dtype=torch.int16, device="cuda")
    o = torch.empty(MAX_KEYS + 1, dtype=torch.int32, device="cuda")
    rc = N.lib().sl_sort_keys16_noalloc(k.data_ptr(), MAX_KEYS + 1, o.data_ptr(), None)
    assert rc == -1
    assert "at most 1048576" in N.last_error()
