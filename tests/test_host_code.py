"""The library's host code (closed-form LBVH topology, KD-tree build, scene
loader, camera, seeds) on the CPU, against the oracle and the golden
fixtures.  Compiled without CUDA from the library's own sources."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

from ptgpu_pc_gb300 import abi, scenes

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


@pytest.fixture(scope="module")
def shim(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("shim") / "libshim.so")
    src = [os.path.join(HERE, "host", "host_shim.cpp"),
           os.path.join(ROOT, "ptgpu_pc_gb300", "csrc", "kdtree.cpp"),
           os.path.join(ROOT, "ptgpu_pc_gb300", "csrc", "loader.cpp")]
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off",
                           "-o", out] + src)
    L = ctypes.CDLL(out)
    vp = ctypes.c_void_p
    L.shim_topology.argtypes = [ctypes.c_int] + [vp] * 6
    L.shim_check_blocks.argtypes = [ctypes.c_int]
    L.shim_kd_build.argtypes = [vp, ctypes.c_int, vp, vp, vp]
    L.shim_kd_export.argtypes = [vp, ctypes.c_int64, vp]
    L.shim_kd_export_wide.argtypes = [vp, vp]
    L.shim_read_scene.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_int, vp, vp, vp,
                                  ctypes.c_char_p, ctypes.c_int]
    L.shim_scene_get.argtypes = [vp, vp]
    L.shim_update_camera.argtypes = [vp]
    L.shim_read_obj.argtypes = [ctypes.c_char_p, ctypes.c_int, vp, vp, ctypes.c_char_p, ctypes.c_int]
    L.shim_ra_new.restype = vp
    L.shim_ra_delete.argtypes = [vp]
    L.shim_ra_grow.argtypes = [vp, ctypes.c_int64]
    L.shim_ra_alloc.argtypes = [vp, ctypes.c_int64, vp]
    L.shim_ra_release.argtypes = [vp, ctypes.c_int64, ctypes.c_int64]
    L.shim_ra_used.argtypes = [vp]
    L.shim_ra_used.restype = ctypes.c_int64
    L.shim_ra_free.argtypes = [vp, vp, ctypes.c_int]
    L.shim_ra_free_tail.argtypes = [vp]
    L.shim_ra_free_tail.restype = ctypes.c_int64
    L.shim_obj_get.argtypes = [vp, vp]
    L.shim_read_scene_compact.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_int, vp, vp, vp]
    L.shim_compact_get.argtypes = [vp]
    L.shim_make_seeds.argtypes = [ctypes.c_uint64, vp, ctypes.c_uint32]
    L.shim_step_selection.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int64, vp]
    return L


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


@pytest.mark.parametrize("n", list(range(2, 200)) + [1000, 1023, 1024, 1025, 4097, 81934, 100003])
def test_closed_form_topology(n, shim, orc):
    mn, mx, g, par, leaf = (np.zeros(n - 1, np.int32) for _ in range(5))
    lp = np.zeros(n, np.int32)
    shim.shim_topology(n, _p(mn), _p(mx), _p(g), _p(par), _p(leaf), _p(lp))
    btn, btl = orc.radix_tree(n)
    assert np.array_equal(mn, btn["min"]) and np.array_equal(mx, btn["max"])
    assert np.array_equal(g, btn["nLeft"]) and np.array_equal(g + 1, btn["nRight"])
    assert np.array_equal(par, btn["nParent"]) and np.array_equal(leaf, btn["leaf"])
    assert np.array_equal(lp, btl["nParent"])


def test_block_fields_short_form(shim):
    """The emission kernels' short form of a block's record fields equals the
    general closed form, which equals the node carrying the block's index."""
    for n in list(range(2, 1100)) + [4095, 4096, 4097, 81934, 100003, 262144, 262145, 4194304]:
        assert shim.shim_check_blocks(n) == 0, n


@pytest.mark.parametrize("case", ["cornell", "ico2", "ico4", "soup", "ico6", "soup100k"])
def test_kd_build_matches_oracle(case, shim, orc):
    """The host KD build against the oracle's pointer tree: the int16 heap
    byte for byte (truncated the reference's way where it overflows, as at the
    config-2 size, 81,934 shapes) and the 32-bit breadth-first export node by
    node."""
    shapes = {"cornell": lambda: scenes.cornell_spheres()[0],
              "ico2": lambda: scenes.icosphere_scene(level=2)[0],
              "ico4": lambda: scenes.icosphere_scene(level=4)[0],
              "soup": lambda: scenes.triangle_soup(3000, seed=9),
              "ico6": lambda: scenes.icosphere_scene(level=6)[0],
              "soup100k": lambda: scenes.triangle_soup(100_000, seed=29)}[case]()
    md, sz, heap = ctypes.c_int(), ctypes.c_int(), ctypes.c_int64()
    shim.shim_kd_build(_p(shapes), len(shapes), ctypes.byref(md), ctypes.byref(sz), ctypes.byref(heap))
    kd = orc.KD(shapes)
    assert md.value == kd.max_depth and sz.value == kd.szbuf
    okng, okn, ost = kd.heap()
    if heap.value <= (1 << 20):
        kng = np.zeros(heap.value, abi.KD_NODE)
        kn = np.zeros(max(sz.value, 1), np.int32)
        st = shim.shim_kd_export(_p(kng), heap.value, _p(kn))
        assert st == ost
        assert kng.tobytes() == okng.tobytes()
        assert np.array_equal(kn[: sz.value], okn)
    from test_gpu_kdtree import _oracle_bfs
    want = _oracle_bfs(kd)
    nodes = np.zeros(shim.shim_kd_node_count(), abi.KD_NODE_WIDE)
    kn = np.zeros(max(sz.value, 1), np.int32)
    shim.shim_kd_export_wide(_p(nodes), _p(kn))
    assert nodes.tobytes() == want.tobytes()
    assert np.array_equal(kn[: sz.value], kd.kn)


def test_seeds_match_oracle(shim, orc):
    a = np.zeros(1000, np.uint32)
    shim.shim_make_seeds(1, _p(a), 1000)
    assert np.array_equal(a, orc.make_seeds(1, 1000))
    assert (a >= 2).all()


def test_camera_matches_golden(shim):
    z = np.load(os.path.join(HERE, "golden", "obj_model_scene.npz"))
    cam = np.array(z["camera"].view(abi.CAMERA))
    shim.shim_update_camera(_p(cam))
    assert cam.tobytes() == z["camera_updated"].tobytes()


def test_loader_txt_scene(shim, tmp_path):
    """A .txt scene of this test's own: spheres, triangles and an OBJ model,
    with the area and light-count rules of ReadTxt (displayfunc.cpp:144-505)."""
    obj = tmp_path / "quad.obj"
    # ends with a blank line: the reference's OBJ reader drops the final line
    obj.write_text("v 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 0\nf 1 2 3\nf 1/1/1 3/3/3 4/4/4\n\n")
    scene = tmp_path / "s.txt"
    scene.write_text("gamma 2.2  sky1 0 0 0  sky2 0 0 0\ncamera 1 2 3  4 5 6\nmaterials 1\n"
                     "matte 0.5 0.5 0.5  0.1\nobjects 4\n"
                     "sphere 2  0 0 0  1 1 1  0 0 0  0\n"
                     "triangle  0 0 0  2 0 0  0 2 0  0 0 0  0.5 0.5 0.5  1\n"
                     "model %s  10 0 0  2 3 1  0 0 0  0.2 0.3 0.4  2\n"
                     "sphere 1  5 5 5  0 0 0  0.9 0.9 0.9  2\n" % obj)
    n, lc, wl = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    err = ctypes.create_string_buffer(256)
    st = shim.shim_read_scene(str(scene).encode(), 64, 48, ctypes.byref(n), ctypes.byref(lc),
                              ctypes.byref(wl), err, 256)
    assert st == 0, err.value
    assert n.value == 5 and lc.value == 1 and wl.value == 0
    sh = np.zeros(n.value, abi.SHAPE)
    cam = np.zeros(1, abi.CAMERA)
    shim.shim_scene_get(_p(sh), _p(cam))
    assert list(sh["type"]) == [0, 1, 1, 1, 0]
    assert list(sh["refl"]) == [abi.DIFF, abi.SPEC, abi.REFR, abi.REFR, abi.REFR]
    assert sh["area"][0] == np.float32(4.0) * np.float32(3.14159265358979323846) * 2 * 2
    assert sh["area"][1] == np.float32(2.0)
    # model vertices scaled then translated
    assert np.array_equal(sh["p2"][2], np.array([12, 0, 0], np.float32))
    assert cam[0]["width"] == 64 and cam[0]["height"] == 48
    assert np.array_equal(cam[0]["orig"], np.array([1, 2, 3], np.float32))


def test_obj_last_line_rule(shim, tmp_path):
    """A model whose last face is followed by a single newline loses that face,
    as the reference loader does (tinyobj treats the buffer's last byte as a
    terminator); the reference scenes rely on it (table.obj, teapot.obj)."""
    obj = tmp_path / "tri2.obj"
    obj.write_text("v 0 0 0\nv 1 0 0\nv 1 1 0\nf 1 2 3\nf 3 2 1\n")
    scene = tmp_path / "m.txt"
    scene.write_text("camera 0 0 0  0 0 -1\nmaterials 0\nobjects 1\n"
                     "model %s  0 0 0  1 1 1  0 0 0  0.5 0.5 0.5  0\n" % obj)
    n, lc, wl = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    err = ctypes.create_string_buffer(256)
    assert shim.shim_read_scene(str(scene).encode(), 8, 8, ctypes.byref(n), ctypes.byref(lc),
                                ctypes.byref(wl), err, 256) == 0
    assert n.value == 1


def test_loader_scn_scene_adds_wall_light(shim, tmp_path):
    scene = tmp_path / "s.scn"
    scene.write_text("camera 0 0 75 0 0 0\nsize 2\nsphere 3  0 0 0  0 0 0  .5 .5 .5  0\n"
                     "sphere 1  1 1 1  4 4 4  0 0 0  1\n")
    n, lc, wl = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    err = ctypes.create_string_buffer(256)
    st = shim.shim_read_scene(str(scene).encode(), 8, 8, ctypes.byref(n), ctypes.byref(lc),
                              ctypes.byref(wl), err, 256)
    assert st == 0 and wl.value == 1 and n.value == 2 + 9 and lc.value == 0


def test_loader_errors(shim, tmp_path):
    n, lc, wl = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    err = ctypes.create_string_buffer(256)
    assert shim.shim_read_scene(b"/nonexistent.txt", 8, 8, ctypes.byref(n), ctypes.byref(lc),
                                ctypes.byref(wl), err, 256) == abi.E_IO
    bad = tmp_path / "bad.txt"
    bad.write_text("camera 1 2\n")
    assert shim.shim_read_scene(str(bad).encode(), 8, 8, ctypes.byref(n), ctypes.byref(lc),
                                ctypes.byref(wl), err, 256) == abi.E_IO
    ply = tmp_path / "x.ply"
    ply.write_text("ply\n")
    assert shim.shim_read_scene(str(ply).encode(), 8, 8, ctypes.byref(n), ctypes.byref(lc),
                                ctypes.byref(wl), err, 256) == abi.E_INVAL


def test_loader_matches_reference_loader(shim):
    """The reference scene file loaded by the reference's own loader (golden
    fixture) and by this library give the same shapes; needs the reference's
    model files, so it runs only where the reference tree is present."""
    ref = os.environ.get("PTGPU_REFERENCE_DIR", "")
    if not ref:
        pytest.skip("PTGPU_REFERENCE_DIR is not set (the reference tree is not named)")
    if not os.path.isfile(os.path.join(ref, "scenes", "obj-model.txt")):
        pytest.skip("reference scene files not found under PTGPU_REFERENCE_DIR")
    z = np.load(os.path.join(HERE, "golden", "obj_model_scene.npz"))
    gold = z["shapes"].view(abi.SHAPE)
    cwd = os.getcwd()
    try:
        os.chdir(ref)
        n, lc, wl = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        err = ctypes.create_string_buffer(256)
        st = shim.shim_read_scene(b"scenes/obj-model.txt", 40, 30, ctypes.byref(n),
                                  ctypes.byref(lc), ctypes.byref(wl), err, 256)
    finally:
        os.chdir(cwd)
    assert st == 0 and n.value == len(gold) and lc.value == int(z["light_cnt"])
    sh = np.zeros(n.value, abi.SHAPE)
    cam = np.zeros(1, abi.CAMERA)
    shim.shim_scene_get(_p(sh), _p(cam))
    for f in ("type", "p1", "p2", "p3", "e", "c", "refl", "area"):
        a = sh[f]
        b = gold[f]
        if f in ("p1", "p2", "p3"):
            tri = sh["type"] == abi.TRIANGLE
            a, b = a[tri], b[tri]
        assert a.tobytes() == b.tobytes(), f
    assert cam.tobytes()[:40] == z["camera"].tobytes()[:40]


def _read_obj(shim, path, threads):
    nv, nt = ctypes.c_int64(), ctypes.c_int64()
    err = ctypes.create_string_buffer(256)
    ok = shim.shim_read_obj(str(path).encode(), threads, ctypes.byref(nv), ctypes.byref(nt), err, 256)
    if not ok:
        return None, err.value.decode()
    v = np.zeros(3 * nv.value, np.float32)
    t = np.zeros(3 * nt.value, np.int32)
    shim.shim_obj_get(_p(v), _p(t))
    return (v.reshape(-1, 3), t.reshape(-1, 3)), ""


def test_obj_reader_threads_agree(shim, tmp_path):
    """The OBJ reader cut into runs of lines on several threads gives the
    one-thread result: same vertices (as written, float32), same fanned
    triangles in file order, with relative indices, v/vt/vn tokens, comments,
    CRLF and lone-CR line ends, and the final-line rule."""
    path, verts, tris = scenes.write_obj_model(tmp_path / "big.obj", 200_000, seed=3)
    one, e1 = _read_obj(shim, path, 1)
    many, e2 = _read_obj(shim, path, 16)
    assert one is not None and many is not None, (e1, e2)
    assert one[0].tobytes() == many[0].tobytes() and one[1].tobytes() == many[1].tobytes()
    assert np.array_equal(one[0], verts) and np.array_equal(one[1], tris)
    for threads in (2, 3, 7):
        got, _ = _read_obj(shim, path, threads)
        assert got[1].tobytes() == one[1].tobytes()


def test_obj_reader_errors_in_file_order(shim, tmp_path):
    """Errors are those of a sequential read: the first malformed line
    decides, and a face may only use vertices defined above it."""
    body = "".join("v %d 0 0\n" % i for i in range(50_000))
    bad_face_then_vertex = tmp_path / "a.obj"
    bad_face_then_vertex.write_text(body + "f 1 2 60000\n" + body + "v 1 2\n" + "f 1 2 3\n\n")
    for threads in (1, 8):
        got, err = _read_obj(shim, bad_face_then_vertex, threads)
        assert got is None and err.startswith("malformed face"), err
    bad_vertex = tmp_path / "b.obj"
    bad_vertex.write_text(body + "v 1 x 2\n" + body + "f 1 2 3\n\n")
    for threads in (1, 8):
        got, err = _read_obj(shim, bad_vertex, threads)
        assert got is None and err.startswith("malformed vertex"), err
    forward = tmp_path / "c.obj"
    forward.write_text("f 1 2 3\n" + body + "\n")
    for threads in (1, 8):
        got, err = _read_obj(shim, forward, threads)
        assert got is None and err.startswith("malformed face"), err


def test_compact_scene_expands_to_read_scene(shim, tmp_path):
    """The compact scene form (shape runs + models kept as vertex and index
    arrays) expands, segment by segment, to read_scene's shapes byte for byte."""
    scene = scenes.write_model_scene(tmp_path, 30_000, seed=4)
    n, lc, wl = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    err = ctypes.create_string_buffer(256)
    assert shim.shim_read_scene(str(scene).encode(), 32, 24, ctypes.byref(n), ctypes.byref(lc),
                                ctypes.byref(wl), err, 256) == 0, err.value
    ref = np.zeros(n.value, abi.SHAPE)
    cam = np.zeros(1, abi.CAMERA)
    shim.shim_scene_get(_p(ref), _p(cam))
    n2, lc2, segs = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    assert shim.shim_read_scene_compact(str(scene).encode(), 32, 24, ctypes.byref(n2), ctypes.byref(lc2),
                                        ctypes.byref(segs)) == 0
    assert n2.value == n.value and lc2.value == lc.value and segs.value >= 4
    got = np.zeros(n2.value, abi.SHAPE)
    shim.shim_compact_get(_p(got))
    assert got.tobytes() == ref.tobytes()


def _free_runs(busy):
    """(start, length) of the free runs of a boolean occupancy array."""
    runs, i, n = [], 0, len(busy)
    while i < n:
        if busy[i]:
            i += 1
            continue
        j = i
        while j < n and not busy[j]:
            j += 1
        runs.append((i, j - i))
        i = j
    return runs


def test_server_slot_allocator_first_fit(shim):
    """The server's slot allocator (range_alloc.h) against a first-fit model
    over an occupancy array: random grows, allocations and releases give the
    same starts, refusals, used count and (merged) free ranges."""
    rng = np.random.default_rng(17)
    a = shim.shim_ra_new()
    try:
        busy = np.zeros(0, bool)
        live = []
        start = ctypes.c_int64()
        out = np.zeros(2 * 4096, np.int64)
        for step in range(3000):
            op = rng.random()
            if op < 0.05 or len(busy) == 0:
                cap = len(busy) + int(rng.integers(1, 300))
                shim.shim_ra_grow(a, cap)
                busy = np.concatenate([busy, np.zeros(cap - len(busy), bool)])
            elif op < 0.6:
                n = int(rng.integers(1, 64))
                runs = [r for r in _free_runs(busy) if r[1] >= n]
                ok = shim.shim_ra_alloc(a, n, ctypes.byref(start))
                assert ok == (1 if runs else 0)
                if runs:
                    assert start.value == runs[0][0]
                    busy[start.value:start.value + n] = True
                    live.append((start.value, n))
            elif live:
                s, n = live.pop(int(rng.integers(len(live))))
                shim.shim_ra_release(a, s, n)
                busy[s:s + n] = False
            assert shim.shim_ra_used(a) == int(busy.sum())
            k = shim.shim_ra_free(a, out.ctypes.data, 4096)
            runs = _free_runs(busy)
            assert [tuple(x) for x in out[:2 * k].reshape(-1, 2)] == runs
            # the free run that reaches the capacity (what growth extends)
            tail = runs[-1][1] if runs and runs[-1][0] + runs[-1][1] == len(busy) else 0
            assert shim.shim_ra_free_tail(a) == tail
        # releasing everything leaves one range over the whole capacity
        for s, n in live:
            shim.shim_ra_release(a, s, n)
        k = shim.shim_ra_free(a, out.ctypes.data, 4096)
        assert k == 1 and tuple(out[:2]) == (0, len(busy)) and shim.shim_ra_used(a) == 0
    finally:
        shim.shim_ra_delete(a)


def _step(shim, px, fill_cap, fill_px):
    a = np.asarray(px, np.int64)
    out = np.zeros(max(len(a), 1), np.int32)
    k = shim.shim_step_selection(_p(a), len(a), int(fill_cap), fill_px, _p(out))
    return out[:k].tolist()


def test_step_selection_fill_cap(shim):
    """The server's step policy (step_policy.h): without a cap every admitted
    request; with one, oldest first while the pixels fit, the oldest always
    (even alone over the cap), and younger ones that fit after an older one
    did not."""
    cap = 700_000
    big, mid, small = 1024 * 1024, 512 * 512, 128 * 128
    assert _step(shim, [big, small, mid], False, cap) == [0, 1, 2]
    assert _step(shim, [big, small, mid], True, cap) == [0]
    assert _step(shim, [small, big, mid], True, cap) == [0, 2]
    assert _step(shim, [mid, mid, mid], True, cap) == [0, 1]
    assert _step(shim, [small] * 5, True, cap) == [0, 1, 2, 3, 4]
    assert _step(shim, [], True, cap) == []
    assert _step(shim, [cap], True, cap) == [0]
    assert _step(shim, [cap - 1, 1, 1], True, cap) == [0, 1]
    rng = np.random.default_rng(3)
    for _ in range(200):
        px = rng.choice([small, 256 * 256, mid, big], size=rng.integers(1, 12)).tolist()
        sel = _step(shim, px, True, cap)
        assert sel[0] == 0 and sel == sorted(sel)
        assert sum(px[i] for i in sel[1:]) + px[0] <= max(cap, px[0]) or len(sel) == 1
        # first fit: every request left out would not have fitted when it was reached
        total = 0
        for i, p in enumerate(px):
            if i in sel:
                total += p
            else:
                assert total + p > cap
