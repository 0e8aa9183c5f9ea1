"""sph_RadixSort_noalloc, the sort for callers that cannot allocate device
memory while they run (its scratch is a fixed array inside the library),
against the existing sph_RadixSort through the C ABI: calls in a row, each
compared bit for bit (an integer sort has no tolerance), the last two at the
array's 4,194,304-pair limit, plus the refusal of larger sizes.

The file name makes pytest collect it last, so a run that stops at the first
failure has run every other test before this one."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_PAIRS = 1 << 22


def _pairs(torch, n, seed):
    rng = np.random.default_rng(seed)
    kv = np.stack([rng.integers(0, 1 << 32, n, dtype=np.uint64).astype(np.uint32),
                   np.arange(n, dtype=np.uint32)], axis=1)
    kv[: n // 4, 0] &= 0x3FF  # runs of equal keys exercise stability
    return torch.from_numpy(kv.view(np.int32).copy()).cuda()


def _sort(torch, fn, kv, bits):
    d0 = kv.clone()
    d1 = torch.empty_like(kv)
    from pibiti_gb300 import _lib
    _lib.check(fn(ctypes.c_void_p(d0.data_ptr()), ctypes.c_void_p(d1.data_ptr()), kv.shape[0], bits))
    torch.cuda.synchronize()
    out = d0 if ((bits + 7) // 8) % 2 == 0 else d1
    return out.cpu().numpy().view(np.uint32)


def test_noalloc_matches_radix_sort_twice(cuda):
    torch = cuda
    from pibiti_gb300 import _lib
    L = _lib.lib()
    # the last two calls fill the whole array (an odd pass count at 24 bits)
    cases = [(1_048_576, 32, 1), (300_001, 24, 2), (MAX_PAIRS, 32, 3), (MAX_PAIRS, 24, 4)]
    for call, (n, bits, seed) in enumerate(cases):
        kv = _pairs(torch, n, seed)
        ref = _sort(torch, L.sph_RadixSort, kv, bits)
        got = _sort(torch, L.sph_RadixSort_noalloc, kv, bits)
        np.testing.assert_array_equal(got, ref, err_msg=f"call {call + 1}")


def test_noalloc_refuses_beyond_limit(cuda):
    torch = cuda
    from pibiti_gb300 import _lib
    L = _lib.lib()
    d = torch.empty((2, 2), dtype=torch.int32, device="cuda")
    rc = L.sph_RadixSort_noalloc(ctypes.c_void_p(d.data_ptr()), ctypes.c_void_p(d.data_ptr()),
                                 MAX_PAIRS + 1, 32)
    assert rc == 2
    assert "4194304" in _lib.last_error()
