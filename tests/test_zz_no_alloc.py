"""mexct_tvmin3d_dev_noalloc: the TV descent for callers that cannot allocate.

Some callers cannot allocate device memory while they run.  One example is a
serving loop that reserved all of its HBM at start-up, because a cudaMalloc
or cudaFree on the request path can synchronise the device and stall other
streams.  Another is a host application whose GPU memory belongs to another
allocator.  This entry point keeps its scratch in a fixed array inside the
library.  These tests check, through the C ABI, that it returns what the
allocating entry point (mexct_tvmin3d_dev) returns, on two calls in a row
that share that array, and that it rejects volumes beyond its fixed limit.

This file is collected last on purpose: a run that stops at its first failure
has then already run every other test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# Both entry points run the same kernels in the same order with fixed-order FP64
# reductions, so their outputs are compared for exact equality.


def _entry(lib):
    f = lib.mexct_tvmin3d_dev_noalloc
    f.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_float,
                  ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    f.restype = ctypes.c_int
    return f


def _volume(shape, seed):
    import torch
    from mexct import phantoms

    nx, ny, nz = shape
    v = phantoms.ellipsoids(max(nx, ny), count=5, seed=seed, nz=nz)[:nx, :ny, :]
    v = v + np.random.default_rng(seed).normal(0, 1e-3, v.shape).astype(np.float32)
    return torch.from_numpy(np.ascontiguousarray(v.transpose(2, 1, 0))).cuda()  # (z, y, x)


def test_noalloc_matches_allocating_tv_on_two_calls(cuda, lib):
    import torch
    from mexct import _lib, ops

    f = _entry(lib)
    stream = torch.cuda.current_stream()
    # Two calls in a row with different shapes share the one scratch array.
    for shape, c, seed in [((48, 40, 36), 0.05, 1), ((64, 64, 64), 0.02, 2)]:
        vol = _volume(shape, seed)
        ref = ops.tvmin3d_dev(vol, c, 20)
        out = torch.empty_like(vol)
        rc = f(vol.data_ptr(), shape[0], shape[1], shape[2], c, 20, out.data_ptr(),
               stream.cuda_stream)
        assert rc == _lib.OK, _lib.last_error()
        torch.cuda.synchronize()
        assert torch.equal(out, ref)


def test_noalloc_allocates_no_device_memory(cuda, lib):
    """Calls on shapes no call has used yet leave the device's free memory
    exactly where it was (the property this entry point exists for).  One
    call comes first: the first call on a device loads the library's device
    code there (and with it the fixed array), which is not an allocation of
    the call's own."""
    import torch
    from mexct import _lib

    f = _entry(lib)
    shapes = ((36, 44, 28), (52, 30, 40))
    vols = [_volume(s, 9) for s in shapes]
    outs = [torch.empty_like(v) for v in vols]
    stream = torch.cuda.current_stream()
    warm = _volume((24, 20, 16), 8)
    rc = f(warm.data_ptr(), 24, 20, 16, 0.04, 2, warm.data_ptr(), stream.cuda_stream)
    assert rc == _lib.OK, _lib.last_error()
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for v, o, shp in zip(vols, outs, shapes):
        rc = f(v.data_ptr(), shp[0], shp[1], shp[2], 0.04, 20, o.data_ptr(), stream.cuda_stream)
        assert rc == _lib.OK, _lib.last_error()
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0


def test_noalloc_in_place_odd_steps(cuda, lib):
    import torch
    from mexct import _lib, ops

    f = _entry(lib)
    vol = _volume((40, 40, 24), 3)
    ref = ops.tvmin3d_dev(vol, 0.03, 7)
    work = vol.clone()
    rc = f(work.data_ptr(), 40, 40, 24, 0.03, 7, work.data_ptr(),
           torch.cuda.current_stream().cuda_stream)
    assert rc == _lib.OK, _lib.last_error()
    torch.cuda.synchronize()
    assert torch.equal(work, ref)


def test_noalloc_rejects_volumes_beyond_its_limit(cuda, lib):
    import torch
    from mexct import _lib

    f = _entry(lib)
    small = torch.zeros(8, device="cuda")
    rc = f(small.data_ptr(), 129, 128, 128, 0.01, 20, small.data_ptr(),
           torch.cuda.current_stream().cuda_stream)
    assert rc == _lib.ERR_UNSUPPORTED
    assert "limit" in _lib.last_error()


def test_noalloc_rejects_shapes_beyond_the_launch_grid(cuda, lib):
    """1 x 1 x 2^21 voxels fits the voxel and partial-sum limits but needs 65536
    tiles along z, one more than a launch grid holds: a clear rejection, not a
    launch error."""
    import torch
    from mexct import _lib

    f = _entry(lib)
    small = torch.zeros(8, device="cuda")
    rc = f(small.data_ptr(), 1, 1, 1 << 21, 0.01, 20, small.data_ptr(),
           torch.cuda.current_stream().cuda_stream)
    assert rc == _lib.ERR_UNSUPPORTED
    assert "grid" in _lib.last_error()
