"""The allocation-free variant of the perturbation entry point.

Some callers cannot allocate device memory (an allocator owns the whole
device, or their loop may not take an allocation's implicit
synchronisation); clbm_ref_perturbed_state_noalloc serves them from a fixed
device array.  It must give the same result as the allocating
clbm_ref_perturbed_state, call after call, and refuse sizes beyond its array.
This file is collected last on purpose."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_noalloc_matches_allocating_entry_point_twice(gpu, clbm_lib):
    """Calls in a row: a mid-size state, the largest state the array allows
    (n = 1048576), then a smaller one that must not pick up the partial sums
    the larger call left in the shared array.  Both entry points run the same
    kernels, so the results agree bit for bit."""
    torch = gpu
    rng = np.random.default_rng(2024)
    nsnap, eps = 10, 0.05
    for n in (9 * 101 * 33, 1 << 20, 9 * 40 * 24):
        f = (1 + 0.01 * rng.standard_normal(n)) / 9
        snaps = torch.from_numpy((1 + 0.01 * rng.standard_normal(nsnap * n)) / 9).cuda()
        pre = rng.random(nsnap)
        a = torch.from_numpy(f).cuda()
        b = torch.from_numpy(f).cuda()
        clbm_lib.ref_perturbed_state(a.data_ptr(), snaps.data_ptr(), eps, nsnap, n, pre)
        clbm_lib.ref_perturbed_state_noalloc(b.data_ptr(), snaps.data_ptr(), eps, nsnap, n, pre)
        torch.cuda.synchronize()
        np.testing.assert_array_equal(b.cpu().numpy(), a.cpu().numpy())
        assert not np.array_equal(b.cpu().numpy(), f)
        del snaps


def test_noalloc_rejects_sizes_beyond_its_array(gpu, clbm_lib):
    L = clbm_lib.lib()
    pre = np.zeros(10)
    x = gpu.zeros(8, dtype=gpu.float64, device="cuda")
    st = L.clbm_ref_perturbed_state_noalloc(x.data_ptr(), x.data_ptr(), 0.1, 10, (1 << 20) + 1,
                                            pre.ctypes.data_as(C.c_void_p), None)
    assert st == clbm_lib.ERR_INVALID
    assert b"1048576" in L.clbm_last_error()
    st = L.clbm_ref_perturbed_state_noalloc(x.data_ptr(), x.data_ptr(), 0.1, 65, 8,
                                            pre.ctypes.data_as(C.c_void_p), None)
    assert st == clbm_lib.ERR_INVALID
