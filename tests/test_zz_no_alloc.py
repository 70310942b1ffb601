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


def _noalloc_bvh(shapes, on_stream=False):
    """Shapes and node arrays in caller-allocated device memory, each node
    array followed by one node's worth of guard bytes; the call goes through
    the C ABI on the legacy default stream, or on a stream of the caller's.
    Returns the node arrays and whether both guards are untouched."""
    import torch
    import ptgpu_pc_gb300 as pt
    L = pt.lib()
    n = len(shapes)
    sz = abi.BVH_NODE.itemsize
    btn_nodes = max(n - 1, 1)
    d_shapes = _device_bytes(shapes)
    d_btn = torch.full(((btn_nodes + 1) * sz,), 0xAB, dtype=torch.uint8, device="cuda")
    d_btl = torch.full(((n + 1) * sz,), 0xAB, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    stream = torch.cuda.Stream() if on_stream else None
    handle = ctypes.c_void_p(stream.cuda_stream) if stream is not None else None
    st = L.ptgpu_build_bvh_noalloc(ctypes.c_void_p(d_shapes.data_ptr()), n,
                                   ctypes.c_void_p(d_btn.data_ptr()), ctypes.c_void_p(d_btl.data_ptr()),
                                   handle)
    assert st == 0, L.ptgpu_last_error().decode()
    h_btn, h_btl = d_btn.cpu().numpy(), d_btl.cpu().numpy()
    guards_ok = bool((h_btn[btn_nodes * sz:] == 0xAB).all() and (h_btl[n * sz:] == 0xAB).all())
    btn = h_btn[: (n - 1) * sz].view(abi.BVH_NODE)
    btl = h_btl[: n * sz].view(abi.BVH_NODE)
    return btn, btl, guards_ok


def _check(shapes, light_cnt=0, on_stream=False):
    c_btn, c_btl = _context_bvh(shapes, light_cnt)
    n_btn, n_btl, guards_ok = _noalloc_bvh(shapes, on_stream)
    assert n_btl.tobytes() == c_btl.tobytes()
    assert n_btn.tobytes() == c_btn.tobytes()
    assert guards_ok, "bytes written past the node arrays"


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


@pytest.mark.parametrize("n", [1, 2, 3])
def test_noalloc_smallest_scenes(n, built_lib):
    """One to three shapes, after a larger build left the shared array
    stale: the same nodes as the context build, nothing written past them
    (one shape: btl[0] only, d_btn holds one node)."""
    _check(scenes.triangle_soup(5000, seed=40))
    _check(scenes.triangle_soup(n, seed=40 + n))


def test_noalloc_on_a_caller_stream(built_lib):
    """The build enqueued on a stream of the caller's (not the legacy default
    stream), twice in a row."""
    _check(scenes.triangle_soup(70_000, seed=44), on_stream=True)
    _check(scenes.icosphere_scene(level=4)[0], 2, on_stream=True)


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
