"""fl_radix_sort_noalloc, the sort for callers that cannot allocate device memory, against
fl_radix_sort, the allocating entry point, through the C ABI.

The two must agree bit for bit (integer work) on two calls in a row: the second call finds the
first call's contents in the shared built-in scratch and must not be affected by them. Device
buffers come from torch here only because a test needs some owner for them; the entry point
itself allocates nothing. This file is collected last (its name sorts last), and it passes
alone in a fresh process as well.
"""
import numpy as np
import pytest

from forcegpu._lib import (FL_E_ARG, SORT_NOALLOC_MAX_PAIRS, FlError, radix_sort,
                           radix_sort_noalloc)

torch = pytest.importorskip("torch")


def device_sort(keys, vals, lo_bit, in_place=False):
    k = torch.from_numpy(keys.view(np.int64).copy()).cuda()
    v = torch.from_numpy(vals.view(np.int32).copy()).cuda()
    ko, vo = (k, v) if in_place else (torch.empty_like(k), torch.empty_like(v))
    torch.cuda.synchronize()
    radix_sort_noalloc(k.data_ptr(), v.data_ptr(), len(keys), lo_bit, ko.data_ptr(), vo.data_ptr(), 0)
    return ko.cpu().numpy().view(np.uint64), vo.cpu().numpy().view(np.uint32)


@pytest.mark.gpu
def test_noalloc_sort_matches_the_allocating_sort_on_consecutive_calls():
    rng = np.random.default_rng(2024)
    # call 1: the largest size allowed, full 64-bit keys (8 digit passes)
    n1 = SORT_NOALLOC_MAX_PAIRS
    k1 = rng.integers(0, 2 ** 63, n1, dtype=np.uint64) * np.uint64(2) + rng.integers(0, 2, n1, dtype=np.uint64)
    v1 = np.arange(n1, dtype=np.uint32)
    # call 2: fewer pairs, many equal keys (stability), bits [8, 64) only (7 passes, so the
    # result ends in the scratch half and is copied out)
    n2 = 150_001
    k2 = rng.integers(0, 5000, n2, dtype=np.uint64) << np.uint64(40) | rng.integers(0, 256, n2, dtype=np.uint64)
    v2 = rng.permutation(n2).astype(np.uint32)
    for keys, vals, lo in ((k1, v1, 0), (k2, v2, 8)):
        want_k, want_v = radix_sort(keys, vals, lo)
        got_k, got_v = device_sort(keys, vals, lo)
        np.testing.assert_array_equal(got_k, want_k)
        np.testing.assert_array_equal(got_v, want_v)
        # and directly against numpy's stable sort on the same key bits
        order = np.argsort(keys >> np.uint64(lo), kind="stable")
        np.testing.assert_array_equal(got_k, keys[order])
        np.testing.assert_array_equal(got_v, vals[order])
    # a third call, sorting in place
    want_k, want_v = radix_sort(k2, v2, 8)
    got_k, got_v = device_sort(k2, v2, 8, in_place=True)
    np.testing.assert_array_equal(got_k, want_k)
    np.testing.assert_array_equal(got_v, want_v)


@pytest.mark.gpu
def test_noalloc_sort_rejects_sizes_beyond_its_scratch():
    with pytest.raises(FlError) as e:
        radix_sort_noalloc(0, 0, SORT_NOALLOC_MAX_PAIRS + 1, 0, 0, 0, 0)  # rejected before any use
    assert e.value.code == FL_E_ARG
    assert "exceeds the maximum of %d pairs" % SORT_NOALLOC_MAX_PAIRS in str(e.value)


@pytest.mark.gpu
def test_noalloc_sort_rejects_outputs_overlapping_the_other_input():
    """keys_out over the values (or vals_out over the keys) would be overwritten before it is
    read: rejected with FL_E_ARG, nothing launched."""
    n = 1024
    k = torch.zeros(n, dtype=torch.int64, device="cuda")
    v = torch.zeros(2 * n, dtype=torch.int32, device="cuda")  # 8 n bytes: room for n keys too
    ko = torch.empty_like(k)
    torch.cuda.synchronize()
    with pytest.raises(FlError) as e:  # keys_out placed over the values
        radix_sort_noalloc(k.data_ptr(), v.data_ptr(), n, 0, v.data_ptr(), ko.data_ptr(), 0)
    assert e.value.code == FL_E_ARG
    with pytest.raises(FlError) as e:  # vals_out placed over the keys
        radix_sort_noalloc(k.data_ptr(), v.data_ptr(), n, 0, ko.data_ptr(), k.data_ptr(), 0)
    assert e.value.code == FL_E_ARG
