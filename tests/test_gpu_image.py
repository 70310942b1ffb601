"""Image output of a frame, encoded on the device (ptgpu_encode_image /
ptgpu_write_image): the PPM is byte for byte what the reference's 'p' key
writes from the same display buffer (smallptGPU.cpp:1238-1257: "P3" header,
then "%d %d %d " per pixel, rows from y = height-1 down to 0), and the PFM
holds the running mean, bottom row first."""
import numpy as np
import pytest

from ptgpu_pc_gb300 import abi, scenes

pytestmark = pytest.mark.gpu


def _reference_ppm(pixels, w, h):
    """The reference's fprintf loop over the RGBA8 display buffer."""
    p = pixels.view(np.uint8).reshape(h, w, 4)
    out = ["P3\n%d %d\n%d\n" % (w, h, 255)]
    for y in range(h - 1, -1, -1):
        out.append("".join("%d %d %d " % (int(q[0]), int(q[1]), int(q[2])) for q in p[y]))
    return "".join(out).encode()


def _frame(w, h, passes=2):
    import ptgpu_pc_gb300 as pt
    shapes, lc, cam = scenes.icosphere_scene(level=3)
    ctx = pt.Context(w, h, accel=abi.ACCEL_BVH)
    ctx.set_shapes(shapes, lc)
    ctx.build(abi.ACCEL_BVH)
    ctx.set_camera(cam)
    ctx.set_seeds(pt.make_seeds(9, 2 * w * h))
    ctx.draw_frame(passes)
    return ctx


@pytest.mark.parametrize("size", [(40, 30), (1, 1), (1000, 3), (257, 1024)])
def test_ppm_equals_the_reference_dump(size, built_lib, tmp_path):
    w, h = size
    with _frame(w, h) as ctx:
        pixels = ctx.get_pixels()
        got = ctx.encode_image(abi.IMAGE_PPM)
        ctx.write_image(tmp_path / "image.ppm", abi.IMAGE_PPM)
    assert got == _reference_ppm(pixels, w, h)
    assert (tmp_path / "image.ppm").read_bytes() == got


def test_pfm_holds_the_running_mean(built_lib, tmp_path):
    w, h = 64, 48
    with _frame(w, h, passes=3) as ctx:
        colors = ctx.get_colors().view(np.float32).reshape(h, w, 3)   # row-flipped: top row first
        got = ctx.encode_image(abi.IMAGE_PFM)
        ctx.write_image(tmp_path / "image.pfm", abi.IMAGE_PFM)
    header = b"PF\n%d %d\n-1.0\n" % (w, h)
    assert got[:len(header)] == header
    body = np.frombuffer(got[len(header):], dtype="<f4").reshape(h, w, 3)
    assert np.array_equal(body.view(np.uint32), colors[::-1].view(np.uint32))   # bottom row first
    assert (tmp_path / "image.pfm").read_bytes() == got


def test_image_before_a_frame_is_a_state_error(built_lib, tmp_path):
    import ptgpu_pc_gb300 as pt
    with pt.Context(8, 8) as ctx:
        with pytest.raises(pt.PtgpuError) as e:
            ctx.encode_image(abi.IMAGE_PPM)
        assert e.value.status == abi.E_STATE
    with _frame(8, 8) as ctx:
        with pytest.raises(pt.PtgpuError) as e:
            ctx.encode_image(7)
        assert e.value.status == abi.E_INVAL
        with pytest.raises(pt.PtgpuError) as e:
            ctx.write_image(tmp_path / "no_such_dir" / "x.ppm")
        assert e.value.status == abi.E_IO
