"""The C ABI without a GPU: libptgpu.so loads, exports every function that
include/ptgpu.h declares, the Python binding lists exactly those, and the
struct layouts of the binding match the header's static asserts."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "ptgpu.h")


def _declared():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\s*\**\s*(ptgpu_[a-z_0-9]+)\s*\(", text, re.M)))


def test_header_declares_the_expected_entry_points():
    names = _declared()
    for must in ("ptgpu_create", "ptgpu_build", "ptgpu_draw_frame", "ptgpu_get_bvh",
                 "ptgpu_get_kdtree", "ptgpu_trace_closest", "ptgpu_build_bvh_noalloc",
                 "ptgpu_batch_build", "ptgpu_batch_render"):
        assert must in names


def test_library_loads_and_exports_every_declared_symbol(built_lib):
    L = ctypes.CDLL(built_lib._name)
    missing = [n for n in _declared() if not hasattr(L, n)]
    assert not missing, missing


def test_binding_lists_the_header(built_lib):
    import ptgpu_pc_gb300 as pt
    assert sorted(pt.EXPORTS) == _declared()


def test_abi_version_without_a_device(built_lib):
    # a pure function: callable on a machine without a GPU
    assert built_lib.ptgpu_abi_version() == 1


@pytest.mark.parametrize("name,size", [("SHAPE", 104), ("CAMERA", 76), ("BVH_NODE", 60),
                                       ("KD_NODE", 36), ("KD_NODE_WIDE", 48), ("CONFIG", 40),
                                       ("SCENE", 120),
                                       ("BATCH_INFO", 40), ("REQUEST", 112), ("REQUEST_STATS", 24),
                                       ("SERVER_INFO", 96)])
def test_binding_struct_sizes(name, size):
    from ptgpu_pc_gb300 import abi
    assert getattr(abi, name).itemsize == size
    text = open(HEADER).read()
    c = {"SHAPE": "ptgpu_shape", "CAMERA": "ptgpu_camera", "BVH_NODE": "ptgpu_bvh_node",
         "KD_NODE": "ptgpu_kd_node", "KD_NODE_WIDE": "ptgpu_kd_node_wide", "SCENE": "ptgpu_scene", "BATCH_INFO": "ptgpu_batch_info",
         "REQUEST": "ptgpu_request", "REQUEST_STATS": "ptgpu_request_stats",
         "SERVER_INFO": "ptgpu_server_info"}.get(name)
    if c:
        assert re.search(r"sizeof\(%s\)\s*==\s*%d" % (c, size), text)
