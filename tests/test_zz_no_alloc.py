"""snow_sort_keys_static: the binning sort for callers that cannot allocate
device memory (their application owns every device buffer, or cudaMalloc
would stall their frame loop). It must give the same stable order as the
library's own binning entry point, snow_scene_cell_keys, whose sort uses
scratch the scene allocated. This file is collected last so a failure here
does not hide any other test's result.

The device buffers below are torch tensors: the test harness allocates them,
the entry point under test allocates nothing."""
import ctypes as C

import numpy as np
import pytest

from snow_gb300 import scenes

gpu = pytest.mark.gpu


@gpu
def test_static_sort_matches_scene_binning_twice_in_a_row():
    import torch

    from snow_gb300 import api, native as N

    L = N.load()
    ctx = api.Context(0)
    s = scenes.small_scene(n=50000, grid_edge=64, seed=123, v0=(1.0, -2.0, 0.5))
    sim = api.SimScene(ctx, s, mode=N.MODE_FAST).upload().init().step(s.dt, 3)
    keys_ref, perm_ref = sim.cell_keys()  # the scene's own binning (allocating scratch)
    key_bits = int(np.ceil(np.log2((((64 + 3) // 4) ** 3) * 64)))
    dev = torch.device("cuda:0")
    keys = torch.from_numpy(keys_ref.view(np.int32)).to(dev)
    for _ in range(2):  # the shared scratch keeps the last call's contents
        sorted_keys = torch.empty_like(keys)
        perm = torch.empty_like(keys)
        st = L.snow_sort_keys_static(keys.data_ptr(), sorted_keys.data_ptr(), perm.data_ptr(), len(keys_ref),
                                     key_bits, C.c_void_p(torch.cuda.current_stream().cuda_stream))
        assert st == N.SNOW_OK
        torch.cuda.synchronize()
        got_perm = perm.cpu().numpy().view(np.uint32)
        got_keys = sorted_keys.cpu().numpy().view(np.uint32)
        assert np.array_equal(got_perm, perm_ref)
        assert np.array_equal(got_keys, keys_ref[perm_ref])


@gpu
def test_static_sort_rejects_sizes_beyond_its_scratch():
    import torch

    from snow_gb300 import native as N

    L = N.load()
    n = N.SORT_STATIC_MAX_KEYS + 1
    buf = torch.zeros(n, dtype=torch.int32, device="cuda:0")
    st = L.snow_sort_keys_static(buf.data_ptr(), buf.data_ptr(), buf.data_ptr(), n, 24, None)
    assert st == -1  # SNOW_EINVAL, nothing queued
