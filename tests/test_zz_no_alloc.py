"""sph_sort_pairs_noalloc: the sort for callers that cannot allocate device
memory (hosts whose memory manager owns every device allocation, loops that
must not risk an allocation's synchronisation).  Its scratch is a static
device array of fixed size shared by every call, so this file checks that it
gives the same pairs as the allocating sph_sort_pairs and as numpy's stable
argsort on two calls in a row -- a large one, then a smaller one that must not
see the first call's leftovers -- and that it refuses sizes beyond its limit.
The file sorts last so that a run which stops at the first failure has
already run every other test."""
import numpy as np
import pytest

from sph2s_final_gb300 import _abi

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

LIMIT = 1 << 20


def _dev(a):
    return torch.from_numpy(np.ascontiguousarray(a, np.uint32).view(np.int32).copy()).cuda()


def _run(fn, keys, vals, bits):
    n = keys.size
    k_in, v_in = _dev(keys), None if vals is None else _dev(vals)
    k_out = torch.empty(n, dtype=torch.int32, device="cuda")
    v_out = torch.empty(n, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    _abi.check(fn(k_in.data_ptr(), None if v_in is None else v_in.data_ptr(), k_out.data_ptr(),
                  v_out.data_ptr(), n, bits, None))
    return k_out.cpu().numpy().view(np.uint32), v_out.cpu().numpy().view(np.uint32)


def test_noalloc_sort_matches_allocating_sort_twice_in_a_row():
    lib = _abi.lib()
    rng = np.random.default_rng(21)
    calls = [
        (rng.integers(0, 1 << 21, LIMIT).astype(np.uint32), None, 21),  # the full limit, 3 passes
        (rng.integers(0, 1 << 15, 40000).astype(np.uint32),
         rng.integers(0, 1 << 32, 40000, dtype=np.uint64).astype(np.uint32), 15),  # smaller, 2 passes
    ]
    for keys, vals, bits in calls:
        want_k, want_v = _run(lib.sph_sort_pairs, keys, vals, bits)
        got_k, got_v = _run(lib.sph_sort_pairs_noalloc, keys, vals, bits)
        np.testing.assert_array_equal(got_k, want_k)
        np.testing.assert_array_equal(got_v, want_v)
        perm = np.argsort(keys, kind="stable")  # ties keep input order
        np.testing.assert_array_equal(got_k, keys[perm])
        np.testing.assert_array_equal(got_v, perm.astype(np.uint32) if vals is None else vals[perm])


def test_noalloc_sort_rejects_sizes_beyond_its_static_limit():
    lib = _abi.lib()
    dummy = torch.zeros(1, dtype=torch.int32, device="cuda")
    p = dummy.data_ptr()
    assert lib.sph_sort_pairs_noalloc(p, None, p, p, LIMIT + 1, 8, None) == _abi.SPH_E_CAPACITY
    assert b"1,048,576" in lib.sph_last_error()
