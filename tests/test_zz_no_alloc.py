"""bale_ig_dev_noalloc, the gather entry point that allocates nothing.

It serves callers that cannot allocate device memory when they call (HBM
reserved up front by another allocator, or a loop that cannot take the
device synchronisation cudaMalloc/cudaFree may imply).  Its scratch is a
fixed array inside the library, so it has a per-call size limit.  This file
is collected last so that a failing run that stops at the first failure has
already run every other test.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LIMIT = 1 << 18  # requests per call (fixed scratch)


def _call_noalloc(bale, tgt, index, table, shift, bad) -> int:
    """The C ABI directly: returns the status code."""
    import torch

    return int(bale._lib.bale_ig_dev_noalloc(
        tgt.data_ptr(), index.data_ptr(), index.numel(), table.data_ptr(), table.numel(), shift,
        bad.data_ptr(), torch.cuda.current_stream().cuda_stream))


def test_noalloc_matches_existing_entry_point_on_consecutive_calls(cuda, bale):
    import torch

    cases = []
    # call 1: the full per-call limit over a table of just over six 2^21-entry
    # regions (the partition's 16 MiB table regions), the last one partial
    t1 = (6 << 21) + 5
    cases.append((bale.gen_values(t1, 41), bale.gen_uniform(LIMIT, t1, 42), 0))
    # call 2: fewer requests, packed indices, a smaller table and some bad indices,
    # so stale scratch from call 1 would show up if it leaked
    t2 = 1 << 20
    idx2 = bale.gen_uniform(100_003, t2 + 2_000, 43)
    idx2[::997] = -7
    cases.append((bale.gen_values(t2, 44), bale.pack_index(idx2), 16))
    # call 3: the first input again
    cases.append(cases[0])

    dev = []
    for table_h, index_h, shift in cases:
        table = torch.from_numpy(table_h).to(cuda)
        index = torch.from_numpy(index_h).to(cuda)
        want, got = torch.empty_like(index), torch.full_like(index, 123)
        bad_want = torch.zeros(1, dtype=torch.int64, device=cuda)
        bad_got = torch.zeros(1, dtype=torch.int64, device=cuda)
        bale.ig_dev(want, index, table, shift=shift, bad=bad_want)  # existing entry point
        dev.append((table, index, shift, want, got, bad_want, bad_got))
    torch.cuda.synchronize()

    # the first no-alloc call on the device looks up the scratch address
    table, index, shift, want, got, bad_want, bad_got = dev[0]
    assert _call_noalloc(bale, got, index, table, shift, bad_got) == 0
    torch.cuda.synchronize()
    bad_got.zero_()
    got.fill_(123)
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info()[0]
    rcs = []
    for table, index, shift, want, got, bad_want, bad_got in dev:  # consecutive calls
        rcs.append(_call_noalloc(bale, got, index, table, shift, bad_got))
        torch.cuda.synchronize()
    free_after = torch.cuda.mem_get_info()[0]
    assert rcs == [0, 0, 0], bale._last_error()
    assert free_after == free_before  # the calls allocated nothing
    for (table_h, index_h, shift), (table, index, shift, want, got, bad_want, bad_got) in zip(cases, dev):
        assert torch.equal(got, want)  # integer gather: bit-exact with bale_ig_dev
        assert int(bad_got.item()) == int(bad_want.item())
        # and with table[index] itself (out-of-range requests give 0 and are counted)
        ref, nbad = _table_at(table_h, index_h, shift)
        np.testing.assert_array_equal(got.cpu().numpy(), ref)
        assert int(bad_got.item()) == nbad
    assert int(dev[1][5].item()) > 0  # call 2 really had bad indices


def _table_at(table_h, index_h, shift):
    """table[index >> shift] on the host, 0 where the index is out of range;
    also returns how many were."""
    k = index_h >> shift
    ok = (k >= 0) & (k < table_h.size)
    return np.where(ok, table_h[np.where(ok, k, 0)], 0), int((~ok).sum())


def test_noalloc_without_bad_counter_and_with_an_empty_table(cuda, bale):
    """Two calls whose paths differ from the others: no bad counter (the
    count goes to a discard word inside the fixed array) and an empty table
    (every request is out of range: value 0).  Each is checked against
    bale_ig_dev and against table[index], twice in a row."""
    import torch

    t = (2 << 21) + 3
    table_h = bale.gen_values(t, 61)
    index_h = bale.gen_uniform(77_777, t + 100, 62)  # a few beyond the table
    table = torch.from_numpy(table_h).to(cuda)
    index = torch.from_numpy(index_h).to(cuda)
    empty = torch.zeros(0, dtype=torch.int64, device=cuda)
    few = torch.from_numpy(bale.gen_uniform(5_000, 1_000, 63)).to(cuda)
    for _ in range(2):
        want, got = torch.empty_like(index), torch.full_like(index, 5)
        bale.ig_dev(want, index, table)
        bale.ig_dev_noalloc(got, index, table)  # bad=None
        torch.cuda.synchronize()
        assert torch.equal(got, want)
        np.testing.assert_array_equal(got.cpu().numpy(), _table_at(table_h, index_h, 0)[0])

        want, got = torch.full_like(few, 9), torch.full_like(few, 7)
        bad_want = torch.zeros(1, dtype=torch.int64, device=cuda)
        bad_got = torch.zeros(1, dtype=torch.int64, device=cuda)
        bale.ig_dev(want, few, empty, bad=bad_want)
        bale.ig_dev_noalloc(got, few, empty, bad=bad_got)
        torch.cuda.synchronize()
        assert torch.equal(got, want) and not got.any()
        assert int(bad_got.item()) == int(bad_want.item()) == few.numel()


def test_noalloc_rejects_oversize_and_unaligned(cuda, bale):
    import torch

    table = torch.zeros(16, dtype=torch.int64, device=cuda)
    bad = torch.zeros(1, dtype=torch.int64, device=cuda)
    big = torch.zeros(LIMIT + 1, dtype=torch.int64, device=cuda)
    out = torch.empty_like(big)
    assert _call_noalloc(bale, out, big, table, 0, bad) == 1  # BALE_EINVAL
    assert "limit" in bale._last_error()
    with pytest.raises(bale.BaleError):
        bale.ig_dev_noalloc(out, big, table)
    base = torch.zeros(1001, dtype=torch.int64, device=cuda)
    with pytest.raises(bale.BaleError, match="aligned"):
        bale.ig_dev_noalloc(torch.empty(1000, dtype=torch.int64, device=cuda), base[1:], table)
