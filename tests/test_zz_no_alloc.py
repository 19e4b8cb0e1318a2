"""pvdb_grid_sample_backward_noalloc — the grid backward for callers that
cannot let the library allocate device memory (processes that pre-reserve all
device memory in their own pool or run under a fixed budget, and callers that
cannot absorb the device-wide synchronisation of cudaMalloc/cudaFree). It uses
one fixed device array instead of allocating scratch, so it is limited to
32768 points per call.

This file is collected last so a run that stops at the first failure has run
every other test already; it also passes alone in a fresh process."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _grid(cls, n, act, reso):
    g = cls.from_mask(reso, act, background=-1.0, n=n) if n != 1 else cls.from_mask(
        reso, act, background=-1.0)
    return g


@pytest.mark.parametrize("channels", [1, 12])
def test_noalloc_backward_matches_the_allocating_entry_point(channels):
    import torch

    from plenvdb_gb300 import ColorVDB, DensityVDB
    from plenvdb_gb300 import _lib as L
    from plenvdb_gb300 import build
    build.build()
    rng = np.random.default_rng(17 + channels)
    reso = [37, 29, 41]
    act = (rng.random(reso) < 0.3).astype(np.uint8)
    cls = DensityVDB if channels == 1 else ColorVDB
    a = _grid(cls, channels, act, reso)  # reference: the allocating entry point
    b = _grid(cls, channels, act, reso)  # the fixed-scratch entry point
    n = 20000
    st = L.stream_of()
    for call in range(2):  # two calls in a row, accumulating into the gradient
        xyz = torch.from_numpy(rng.uniform(-1.0, np.array(reso) + 0.5, (n, 3)).astype(np.float32)).cuda()
        xs, ys, zs = (xyz[:, q].contiguous() for q in range(3))
        g = torch.from_numpy(rng.normal(0, 1, n * channels).astype(np.float32)).cuda()
        L.call("pvdb_grid_sample_backward", a.handle, L.ptr(xs), L.ptr(ys), L.ptr(zs), L.ptr(g),
               n, L.MEM_DEVICE, st)
        L.call("pvdb_grid_sample_backward_noalloc", b.handle, L.ptr(xs), L.ptr(ys), L.ptr(zs),
               L.ptr(g), n, st)
        torch.cuda.synchronize()
        ga = a.get_dense_grid(which=L.WHICH_GRAD)
        gb = b.get_dense_grid(which=L.WHICH_GRAD)
        # the same stable sort and per-slot sums in the same order: bit for bit
        np.testing.assert_array_equal(gb, ga)
        assert np.abs(ga).sum() > 0


def test_noalloc_backward_at_its_size_limit_with_four_sort_passes():
    """n = 32768 points (the limit) on a dense 256^3 grid: 2^24 voxel slots
    need 25-bit keys, so the sort runs all four digit passes and its histogram
    words reach the fixed array's sizing."""
    import torch

    from plenvdb_gb300 import DensityVDB
    from plenvdb_gb300 import _lib as L
    rng = np.random.default_rng(4)
    reso = [256, 256, 256]
    a, b = DensityVDB(reso, 1), DensityVDB(reso, 1)
    assert a.info()[2] == 32 ** 3
    n = 32768
    st = L.stream_of()
    for call in range(2):
        xyz = torch.from_numpy(rng.uniform(-0.5, 255.5, (n, 3)).astype(np.float32)).cuda()
        xs, ys, zs = (xyz[:, q].contiguous() for q in range(3))
        g = torch.from_numpy(rng.normal(0, 1, n).astype(np.float32)).cuda()
        L.call("pvdb_grid_sample_backward", a.handle, L.ptr(xs), L.ptr(ys), L.ptr(zs), L.ptr(g),
               n, L.MEM_DEVICE, st)
        L.call("pvdb_grid_sample_backward_noalloc", b.handle, L.ptr(xs), L.ptr(ys), L.ptr(zs),
               L.ptr(g), n, st)
        torch.cuda.synchronize()
        ga = a.get_dense_grid(which=L.WHICH_GRAD)
        gb = b.get_dense_grid(which=L.WHICH_GRAD)
        np.testing.assert_array_equal(gb, ga)
        assert np.count_nonzero(ga) > 100000


def test_noalloc_backward_rejects_sizes_beyond_its_scratch():
    import torch

    from plenvdb_gb300 import DensityVDB
    from plenvdb_gb300 import _lib as L
    g = DensityVDB([8, 8, 8], 1)
    n = 32769
    x = torch.zeros(n, device="cuda")
    rc = L.load().pvdb_grid_sample_backward_noalloc(g.handle, L.ptr(x), L.ptr(x), L.ptr(x),
                                                    L.ptr(x), n, None)
    assert rc == L.PVDB_ERR_ARG
    assert "32768" in L.last_error()
