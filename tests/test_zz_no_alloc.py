"""sst_occluded_noalloc, the allocation-free variant of the any-hit query, against sst_occluded.

Both entry points run the same traversal kernel on the same rays, so the flags must be equal.
Each case calls the new entry point twice in a row: the scratch array is shared by all calls, and
the second call must not see anything the first one left behind.  This file is collected last so
that it also runs after every other test in one process."""
import ctypes

import numpy as np
import pytest

from seesharp_gb300 import _native, workloads

pytestmark = pytest.mark.gpu


def _rays(n, seed):
    """Rays from inside the Cornell box in random directions, with tmax in [0.05, 3] or infinite:
    a mix of occluded and unoccluded queries, including rays that leave through the open front."""
    rng = np.random.default_rng(seed)
    r = np.zeros((n, 8), np.float32)
    r[:, 0:3] = rng.uniform(-0.9, 0.9, size=(n, 3))
    d = rng.standard_normal((n, 3))
    r[:, 4:7] = d / np.linalg.norm(d, axis=1, keepdims=True)
    r[:, 3] = 0.0
    r[:, 7] = np.where(rng.uniform(size=n) < 0.8, rng.uniform(0.05, 3.0, size=n), np.inf)
    return r


@pytest.fixture(scope="module")
def scene():
    sc = workloads.cornell_box(64, 64)
    sc.Prepare()
    return sc


def _p(a):
    return ctypes.c_void_p(a.ctypes.data)


@pytest.mark.parametrize("n", [1, 5000, _native.SST_NOALLOC_MAX_RAYS])
def test_noalloc_matches_sst_occluded_host_memory(scene, n):
    L, h = scene.native.lib, scene.native.handle
    rays = _rays(n, seed=n)
    ref = np.zeros(n, np.int32)
    _native.check(L.sst_occluded(h, _p(rays), n, _p(ref), _native.SST_MEM_HOST))
    if n > 100:
        assert 0 < ref.sum() < n
    for _ in range(2):
        out = np.full(n, -7, np.int32)
        _native.check(L.sst_occluded_noalloc(h, _p(rays), n, _p(out), _native.SST_MEM_HOST))
        assert np.array_equal(out, ref)


def test_noalloc_matches_sst_occluded_device_memory(scene):
    torch = pytest.importorskip("torch")
    L, h = scene.native.lib, scene.native.handle
    n = 20000
    rays = _rays(n, seed=3)
    ref = np.zeros(n, np.int32)
    _native.check(L.sst_occluded(h, _p(rays), n, _p(ref), _native.SST_MEM_HOST))
    d_rays = torch.from_numpy(rays).cuda()
    for _ in range(2):
        d_out = torch.full((n,), -7, dtype=torch.int32, device="cuda")
        torch.cuda.synchronize()
        _native.check(L.sst_occluded_noalloc(h, ctypes.c_void_p(d_rays.data_ptr()), n, ctypes.c_void_p(d_out.data_ptr()),
                                             _native.SST_MEM_DEVICE))
        assert np.array_equal(d_out.cpu().numpy(), ref)


def test_noalloc_rejects_more_rays_than_its_scratch_holds(scene):
    L, h = scene.native.lib, scene.native.handle
    n = _native.SST_NOALLOC_MAX_RAYS + 1
    rays = _rays(n, seed=9)
    out = np.full(n, -7, np.int32)
    rc = L.sst_occluded_noalloc(h, _p(rays), n, _p(out), _native.SST_MEM_HOST)
    assert rc == -1
    assert "exceed the limit of 65536 rays" in _native.last_error()
    assert np.all(out == -7)
    # the next call in range still works
    ok = scene.native.occluded_noalloc(rays[:100])
    assert np.array_equal(ok, scene.native.occluded(rays[:100]))


def test_noalloc_allocates_no_device_memory(scene):
    """The property the entry point exists for: after its first call on the device (which looks up
    the scratch array's address), repeated calls leave the device's free memory unchanged.  The
    same measurement sees the growth of sst_occluded's context buffers for a larger query, so it
    would see an allocation."""
    torch = pytest.importorskip("torch")
    L, h = scene.native.lib, scene.native.handle
    n = _native.SST_NOALLOC_MAX_RAYS
    rays = _rays(n, seed=21)
    out = np.zeros(n, np.int32)
    _native.check(L.sst_occluded_noalloc(h, _p(rays), n, _p(out), _native.SST_MEM_HOST))
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for k in range(20):
        _native.check(L.sst_occluded_noalloc(h, _p(rays), n, _p(out), _native.SST_MEM_HOST))
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    # a query larger than any before grows the context buffers of sst_occluded by about 68 MB
    big = np.tile(rays, (64, 1))
    flags = np.zeros(big.shape[0], np.int32)
    _native.check(L.sst_occluded(h, _p(big), big.shape[0], _p(flags), _native.SST_MEM_HOST))
    free2, _ = torch.cuda.mem_get_info()
    assert free2 < free1 - 32 * 2**20
