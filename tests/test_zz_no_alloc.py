"""snow_sort_keys_static: the binning sort for callers that cannot allocate
device memory (their application owns every device buffer, or cudaMalloc
would stall their frame loop). Its output is checked on the CPU against a
stable sort of the same keys (numpy's stable argsort, and the oracle's
std::stable_sort of the cell keys of a stepped scene), on two calls in a row
(the shared scratch keeps the previous call's contents). This file is
collected last so a failure here does not hide any other test's result.

The device buffers below are torch tensors: the test harness allocates them,
the entry point under test allocates nothing."""
import ctypes as C

import numpy as np
import pytest

from oracle import oracle as O
from snow_gb300 import scenes

gpu = pytest.mark.gpu


def _sort_twice(keys_np, key_bits, in_place=False):
    """Two calls in a row through the C ABI; returns both (sorted, perm)."""
    import torch

    from snow_gb300 import native as N

    L = N.load()
    dev = torch.device("cuda:0")
    out = []
    for _ in range(2):
        keys = torch.from_numpy(keys_np.view(np.int32).copy()).to(dev)
        sorted_keys = keys if in_place else torch.empty_like(keys)
        perm = torch.full_like(keys, -1)
        st = L.snow_sort_keys_static(keys.data_ptr(), sorted_keys.data_ptr(), perm.data_ptr(), len(keys_np),
                                     key_bits, C.c_void_p(torch.cuda.current_stream().cuda_stream))
        assert st == N.SNOW_OK
        torch.cuda.synchronize()
        out.append((sorted_keys.cpu().numpy().view(np.uint32), perm.cpu().numpy().view(np.uint32)))
    return out


@gpu
@pytest.mark.parametrize("key_bits", [16, 18, 24])
@pytest.mark.parametrize("n", [1, 4097, "max"])
def test_static_sort_matches_a_cpu_stable_sort(n, key_bits):
    """16 key bits take two 8-bit passes (the result lands in the output
    arrays), 18 and 24 take three (the result is copied back from the
    scratch); n = SNOW_SORT_STATIC_MAX_KEYS fills the histogram and scan
    regions of the scratch. Few distinct keys make long runs of ties."""
    from snow_gb300 import native as N

    n = N.SORT_STATIC_MAX_KEYS if n == "max" else n
    rng = np.random.default_rng(1000 + key_bits + n)
    distinct = rng.integers(0, 1 << key_bits, size=max(1, n // 7), dtype=np.uint64)
    keys = distinct[rng.integers(0, len(distinct), size=n)].astype(np.uint32)
    want_perm = np.argsort(keys, kind="stable").astype(np.uint32)
    for got_keys, got_perm in _sort_twice(keys, key_bits):
        assert np.array_equal(got_perm, want_perm)
        assert np.array_equal(got_keys, keys[want_perm])


@gpu
def test_static_sort_in_place_matches_the_oracle_binning():
    """The cell keys of a stepped scene (downloaded positions keyed on the
    CPU by the oracle), sorted in place (keys == sorted_keys), against the
    oracle's std::stable_sort of the same keys."""
    from snow_gb300 import api, native as N

    ctx = api.Context(0)
    s = scenes.small_scene(n=50000, grid_edge=64, seed=123, v0=(1.0, -2.0, 0.5))
    sim = api.SimScene(ctx, s, mode=N.MODE_FAST).upload().init().step(s.dt, 3)
    x = sim.download()["x"]
    _, keys, want_perm = O.cell_keys(x, s.grid_pos, s.grid_dim, s.grid_spacing)
    key_bits = int(np.ceil(np.log2((((64 + 3) // 4) ** 3) * 64)))
    for got_keys, got_perm in _sort_twice(keys, key_bits, in_place=True):
        assert np.array_equal(got_perm, want_perm)
        assert np.array_equal(got_keys, keys[want_perm])
    sim.close()
    ctx.close()


@gpu
def test_static_sort_rejects_sizes_beyond_its_scratch_and_aliased_outputs():
    import torch

    from snow_gb300 import native as N

    L = N.load()
    n = N.SORT_STATIC_MAX_KEYS + 1
    buf = torch.zeros(n, dtype=torch.int32, device="cuda:0")
    assert L.snow_sort_keys_static(buf.data_ptr(), buf.data_ptr(), buf.data_ptr(), n, 24, None) == N.SNOW_EINVAL
    a = torch.zeros(1000, dtype=torch.int32, device="cuda:0")
    b = torch.zeros(1000, dtype=torch.int32, device="cuda:0")
    # perm is the output key array, or overlaps the input keys
    assert L.snow_sort_keys_static(a.data_ptr(), b.data_ptr(), b.data_ptr(), 1000, 24, None) == N.SNOW_EINVAL
    assert L.snow_sort_keys_static(a.data_ptr(), b.data_ptr(), a.data_ptr() + 400, 1000, 24, None) == N.SNOW_EINVAL
    # the two key arrays overlap without being the same array
    assert L.snow_sort_keys_static(a.data_ptr(), a.data_ptr() + 4, b.data_ptr(), 500, 24, None) == N.SNOW_EINVAL
    torch.cuda.synchronize()
