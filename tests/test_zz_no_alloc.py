"""The no-allocation trace-statistics entry point (krr_accel_trace_stats_noalloc).

It is meant for callers that must not allocate device memory while they run
(a render loop with a fixed per-frame memory budget, where cudaMalloc could
stall the device, or a host whose pool allocator owns all device memory).
Its scratch sits in a static device array, so it must give the same node and
triangle counts as krr_accel_trace_stats, which allocates its scratch per
call, and keep giving them on back-to-back calls that reuse the array.
This file is collected last so that a run stopping at the first failure has
already run every other test."""
import ctypes as C

import pytest
import torch

from kiraray_gb300 import _lib, scenes
from kiraray_gb300.accel import Accel
from tests import helpers as H

pytestmark = pytest.mark.gpu


def _counts(fn, acc, rays, any_hit):
    out = (C.c_ulonglong * 2)()
    st = fn(acc._h, rays.data_ptr(), rays.shape[0], int(any_hit), out,
            torch.cuda.current_stream().cuda_stream)
    _lib.check(st, fn.__name__)
    return int(out[0]), int(out[1])


def test_noalloc_stats_match_allocating_entry_point(krr_lib, cuda):
    sc = scenes.cornell_box(128, 128)
    tris = sc.world_triangles()
    acc = Accel(tris)
    rays = torch.from_numpy(H.pinhole_rays(sc, jitter_seed=4)[:_lib.NOALLOC_MAX_RAYS]).cuda()
    lib = _lib.load()
    for any_hit in (False, True):
        want = _counts(lib.krr_accel_trace_stats, acc, rays, any_hit)
        first = _counts(lib.krr_accel_trace_stats_noalloc, acc, rays, any_hit)
        second = _counts(lib.krr_accel_trace_stats_noalloc, acc, rays, any_hit)
        # integer counts: the tolerance is exact equality
        assert first == want and second == want, (any_hit, want, first, second)
        assert want[0] > 0 and want[1] > 0


def test_noalloc_stats_on_a_smaller_batch_after_a_larger_one(krr_lib, cuda):
    tris = H.random_soup(4000, 12)
    acc = Accel(tris)
    lib = _lib.load()
    big = torch.from_numpy(H.random_rays(_lib.NOALLOC_MAX_RAYS, 13)).cuda()
    small = big[:1000].contiguous()
    _counts(lib.krr_accel_trace_stats_noalloc, acc, big, False)
    got = _counts(lib.krr_accel_trace_stats_noalloc, acc, small, False)
    assert got == _counts(lib.krr_accel_trace_stats, acc, small, False)


def test_noalloc_rejects_sizes_beyond_the_static_scratch(krr_lib, cuda):
    acc = Accel(H.random_soup(10, 1))
    lib = _lib.load()
    rays = torch.zeros((_lib.NOALLOC_MAX_RAYS + 1, 8), device="cuda")
    out = (C.c_ulonglong * 2)()
    st = lib.krr_accel_trace_stats_noalloc(acc._h, rays.data_ptr(), rays.shape[0], 0, out,
                                           torch.cuda.current_stream().cuda_stream)
    assert st == 1   # KRR_ERR_INVALID_ARGUMENT
    assert b"static scratch" in lib.krr_last_error()
    st = lib.krr_accel_trace_stats_noalloc(acc._h, rays.data_ptr(), 0, 0, out,
                                           torch.cuda.current_stream().cuda_stream)
    assert st == 1


def test_noalloc_leaves_device_memory_unchanged(krr_lib, cuda):
    """Free device memory (cudaMemGetInfo) is the same before and after calls
    of the no-allocation entry point; nothing between the two readings goes
    through torch's caching allocator."""
    tris = H.random_soup(3000, 21)
    acc = Accel(tris)
    lib = _lib.load()
    rays = torch.from_numpy(H.random_rays(20000, 22)).cuda()
    _counts(lib.krr_accel_trace_stats_noalloc, acc, rays, False)   # set-up on this device
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info()[0]
    for any_hit in (False, True, False):
        _counts(lib.krr_accel_trace_stats_noalloc, acc, rays, any_hit)
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free_before


def test_noalloc_reports_a_stack_overflow(krr_lib, cuda):
    """A traversal stack limit that cuts rays off makes the call return
    KRR_ERR_OVERFLOW, as the allocating entry point does."""
    sc = scenes.large_scene(width=64, height=48, grid=96, n_spheres=30, sky_size=(32, 16))
    acc = Accel(sc.world_triangles())
    lib = _lib.load()
    rays = torch.from_numpy(H.pinhole_rays(sc, jitter_seed=1)).cuda()
    acc.set_stack_limit(1)
    out = (C.c_ulonglong * 2)()
    for fn in (lib.krr_accel_trace_stats_noalloc, lib.krr_accel_trace_stats):
        st = fn(acc._h, rays.data_ptr(), rays.shape[0], 0, out,
                torch.cuda.current_stream().cuda_stream)
        assert st == 3, fn.__name__   # KRR_ERR_OVERFLOW
    acc.set_stack_limit(48)
    assert _counts(lib.krr_accel_trace_stats_noalloc, acc, rays, False) == \
        _counts(lib.krr_accel_trace_stats, acc, rays, False)
