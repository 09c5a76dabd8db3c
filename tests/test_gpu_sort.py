"""The onesweep radix sort through the C ABI (sph_sort_pairs), bit-exact
against a stable numpy argsort: the contract of thrust::sort_by_key at
SPH2S_FINAL_SINGLE_SCALE/Solver.cu:1110-1115 plus stability (ties keep input
order), on the edge cases the step meets (empty, one key, all keys equal,
sorted and reversed input, ragged tails, the largest key widths) and at 4M
keys."""
import numpy as np
import pytest

from sph2s_final_gb300 import _abi

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def gpu_sort(keys: np.ndarray, vals, key_bits: int):
    n = keys.size
    as_i32 = lambda a: torch.from_numpy(np.ascontiguousarray(a, np.uint32).view(np.int32).copy())
    k_in = as_i32(keys).cuda()
    v_in = None if vals is None else as_i32(vals).cuda()
    k_out = torch.empty(max(n, 1), dtype=torch.int32, device="cuda")
    v_out = torch.empty(max(n, 1), dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    rc = _abi.lib().sph_sort_pairs(k_in.data_ptr() if n else None,
                                   None if v_in is None else v_in.data_ptr(),
                                   k_out.data_ptr(), v_out.data_ptr(), n, key_bits, None)
    _abi.check(rc)
    ko = k_out.cpu().numpy()[:n].view(np.uint32)
    vo = v_out.cpu().numpy()[:n].view(np.uint32)
    return ko, vo


def expect(keys, vals):
    order = np.argsort(keys, kind="stable")
    v = np.arange(keys.size, dtype=np.uint32) if vals is None else vals
    return keys[order], v[order]


CASES = [
    ("empty", np.zeros(0, np.uint32), 15),
    ("one", np.array([7], np.uint32), 15),
    ("all_equal", np.full(10000, 1234, np.uint32), 15),
    ("sorted", np.arange(50000, dtype=np.uint32), 16),
    ("reversed", np.arange(50000, dtype=np.uint32)[::-1].copy(), 16),
    ("ragged_tail", np.random.default_rng(1).integers(0, 1 << 21, 4096 * 3 + 17).astype(np.uint32), 21),
    ("few_distinct", np.random.default_rng(2).integers(0, 4, 100000).astype(np.uint32), 2),
    ("bits30", np.random.default_rng(3).integers(0, 1 << 30, 300001).astype(np.uint32), 30),
    ("bits32", np.random.default_rng(4).integers(0, 1 << 32, 300001, dtype=np.uint64).astype(np.uint32), 32),
]


@pytest.mark.parametrize("name,keys,bits", CASES, ids=[c[0] for c in CASES])
def test_sort_pairs_matches_stable_argsort(name, keys, bits):
    ko, vo = gpu_sort(keys, None, bits)
    ek, ev = expect(keys, None)
    np.testing.assert_array_equal(ko, ek)
    np.testing.assert_array_equal(vo, ev)


def test_sort_pairs_carries_values_and_large_n():
    rng = np.random.default_rng(5)
    n = 4 * 1024 * 1024 + 3
    keys = rng.integers(0, 1 << 21, n).astype(np.uint32)
    vals = rng.integers(0, 1 << 32, n, dtype=np.uint64).astype(np.uint32)
    ko, vo = gpu_sort(keys, vals, 21)
    ek, ev = expect(keys, vals)
    np.testing.assert_array_equal(ko, ek)
    np.testing.assert_array_equal(vo, ev)


def test_sort_pairs_rejects_bad_arguments():
    lib = _abi.lib()
    assert lib.sph_sort_pairs(None, None, None, None, 5, 8, None) == _abi.SPH_E_INVALID
    assert lib.sph_sort_pairs(None, None, None, None, 0, 8, None) == _abi.SPH_OK


def gpu_sort_coherent(keys: np.ndarray, hint: np.ndarray, key_bits: int):
    n = keys.size
    as_i32 = lambda a: torch.from_numpy(np.ascontiguousarray(a, np.uint32).view(np.int32).copy())
    k_in, h_in = as_i32(keys).cuda(), as_i32(hint).cuda()
    k_out = torch.empty(max(n, 1), dtype=torch.int32, device="cuda")
    p_out = torch.empty(max(n, 1), dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    rc = _abi.lib().sph_sort_keys_coherent(k_in.data_ptr() if n else None,
                                           h_in.data_ptr() if n else None, k_out.data_ptr(),
                                           p_out.data_ptr(), n, key_bits, None)
    return rc, k_out.cpu().numpy()[:n].view(np.uint32), p_out.cpu().numpy()[:n].view(np.uint32)


def perturbed(hint, movers, bits, rng):
    """The hint with exactly `movers` positions given a different key."""
    keys = hint.copy()
    idx = rng.choice(hint.size, movers, replace=False)
    keys[idx] = (hint[idx] + rng.integers(1, 1 << bits, movers).astype(np.uint32)) & np.uint32((1 << bits) - 1 if bits < 32 else 0xFFFFFFFF)
    return keys


def coherent_cases():
    rng = np.random.default_rng(7)
    out = []
    h = np.sort(rng.integers(0, 1 << 21, 300001).astype(np.uint32))
    # up to 32,768 changed keys are radix-sorted in tiles of 512, more in tiles of 4,096
    for m in (0, 1, 5000, 32768, 32769, 100000, 300001):
        out.append((f"movers{m}", perturbed(h, m, 21, rng), h, 21))
    keys = rng.integers(0, 1 << 21, 50000).astype(np.uint32)
    out.append(("unrelated_hint", keys, np.sort(rng.integers(0, 1 << 21, 50000).astype(np.uint32)), 21))
    out.append(("hint_all_max", keys, np.full(50000, 0xFFFFFFFF, np.uint32), 21))
    out.append(("hint_all_zero", keys, np.zeros(50000, np.uint32), 21))
    out.append(("equal_keys", np.full(40000, 77, np.uint32), np.sort(rng.integers(0, 200, 40000)).astype(np.uint32), 8))
    out.append(("one", np.array([5], np.uint32), np.array([9], np.uint32), 4))
    for n in (31, 33, 2047, 2049):  # ragged flag words and tiles
        k = rng.integers(0, 64, n).astype(np.uint32)
        out.append((f"ragged{n}", k, np.sort(perturbed(np.sort(k), n // 3, 6, rng)), 6))
    hb = np.sort(rng.integers(0, 1 << 32, 70000, dtype=np.uint64).astype(np.uint32))
    out.append(("bits32", perturbed(hb, 9000, 32, rng), hb, 32))  # four passes, in place
    hb = np.sort(rng.integers(0, 1 << 16, 70000).astype(np.uint32))
    out.append(("bits16_many", perturbed(hb, 40000, 16, rng), hb, 16))  # two passes
    return out


COHERENT = coherent_cases()


@pytest.mark.parametrize("name,keys,hint,bits", COHERENT, ids=[c[0] for c in COHERENT])
def test_coherent_sort_matches_stable_argsort_for_every_hint(name, keys, hint, bits):
    rc, ko, po = gpu_sort_coherent(keys, hint, bits)
    _abi.check(rc)
    ek, ev = expect(keys, None)
    np.testing.assert_array_equal(ko, ek)
    np.testing.assert_array_equal(po, ev)


def test_coherent_sort_rejects_a_decreasing_hint():
    keys = np.arange(1000, dtype=np.uint32)
    hint = np.arange(1000, dtype=np.uint32)
    hint[500] = 0
    rc, _, _ = gpu_sort_coherent(keys, hint, 10)
    assert rc == _abi.SPH_E_INVALID
    assert _abi.lib().sph_sort_keys_coherent(None, None, None, None, 5, 8, None) == _abi.SPH_E_INVALID
