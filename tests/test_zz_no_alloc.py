"""ptgpu_build_bvh_noalloc (the LBVH build whose intermediates live in a fixed
array inside the library) against the context build, ptgpu_build(ctx,
PTGPU_ACCEL_BVH, 0) + ptgpu_get_bvh: the btn/btl arrays must match byte for
byte, on two calls in a row that share the array.  The file name sorts last
so that the calls also run after every other GPU test of the session."""
import ctypes

import numpy as np
import pytest

from ptgpu_pc_gb300 import abi, scenes

pytestmark = pytest.mark.gpu

MAX_SHAPES = 1 << 18


def _context_bvh(shapes, light_cnt=0):
    import ptgpu_pc_gb300 as pt
    with pt.Context(8, 8) as ctx:
        ctx.set_shapes(shapes, light_cnt)
        ctx.build(abi.ACCEL_BVH)
        return ctx.get_bvh()


def _device_bytes(arr):
    import torch
    return torch.from_numpy(np.ascontiguousarray(arr).view(np.uint8).reshape(-1).copy()).cuda()


def _noalloc_bvh(shapes):
    """Shapes and node arrays in caller-allocated device memory; the call
    itself goes through the C ABI with the legacy default stream."""
    import torch
    import ptgpu_pc_gb300 as pt
    L = pt.lib()
    n = len(shapes)
    d_shapes = _device_bytes(shapes)
    d_btn = torch.full((max(n - 1, 1) * abi.BVH_NODE.itemsize,), 0xAB, dtype=torch.uint8, device="cuda")
    d_btl = torch.full((n * abi.BVH_NODE.itemsize,), 0xAB, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    st = L.ptgpu_build_bvh_noalloc(ctypes.c_void_p(d_shapes.data_ptr()), n,
                                   ctypes.c_void_p(d_btn.data_ptr()), ctypes.c_void_p(d_btl.data_ptr()),
                                   None)
    assert st == 0, L.ptgpu_last_error().decode()
    btn = d_btn.cpu().numpy()[: (n - 1) * abi.BVH_NODE.itemsize].view(abi.BVH_NODE)
    btl = d_btl.cpu().numpy().view(abi.BVH_NODE)
    return btn, btl


def _check(shapes, light_cnt=0):
    c_btn, c_btl = _context_bvh(shapes, light_cnt)
    n_btn, n_btl = _noalloc_bvh(shapes)
    assert n_btl.tobytes() == c_btl.tobytes()
    assert n_btn.tobytes() == c_btn.tobytes()


def test_noalloc_two_calls_in_a_row(built_lib):
    # a large triangle soup, then a smaller sphere scene over the stale
    # contents of the shared array
    _check(scenes.triangle_soup(150_000, seed=21))
    shapes, light_cnt, _ = scenes.cornell_spheres()
    _check(shapes, light_cnt)


def test_noalloc_icosphere_then_maximum_size(built_lib):
    shapes, light_cnt, _ = scenes.icosphere_scene(level=5)
    _check(shapes, light_cnt)
    _check(scenes.triangle_soup(MAX_SHAPES, seed=22))


def test_noalloc_rejects_sizes_beyond_the_array(built_lib):
    import torch
    import ptgpu_pc_gb300 as pt
    L = pt.lib()
    buf = torch.zeros(256, dtype=torch.uint8, device="cuda")
    p = ctypes.c_void_p(buf.data_ptr())
    # rejected on the host before any buffer is touched
    assert L.ptgpu_build_bvh_noalloc(p, MAX_SHAPES + 1, p, p, None) == -6
    assert b"262144" in L.ptgpu_last_error()
    assert L.ptgpu_build_bvh_noalloc(p, 0, p, p, None) == -1
    assert L.ptgpu_build_bvh_noalloc(None, 4, p, p, None) == -1
