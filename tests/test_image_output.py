"""Image output (RenderBuffer::GetPixelsRGB8 / SaveToFilePNG / SaveToFileHDR,
src/Tracer/RenderBuffer.cpp:37-84): the PNG writer round-trips through an
independent decoder, the HDR writer's RGBE pixels decode to the input within
the format's 8-bit mantissa, and (GPU) the device RGB8 conversion equals
clamp(v * 255, 0, 255) truncated."""
import numpy as np
import pytest

import mitrace_gb300 as mt
from mitrace_gb300 import gltf


def read_hdr(path):
    data = open(path, "rb").read()
    head_end = data.index(b"\n\n") + 2
    line_end = data.index(b"\n", head_end)
    dims = data[head_end:line_end].split()
    h, w = int(dims[1]), int(dims[3])
    pos = line_end + 1
    img = np.zeros((h, w, 4), np.uint8)
    for y in range(h):
        if 8 <= w < 32768 and data[pos] == 2 and data[pos + 1] == 2:
            pos += 4
            for c in range(4):
                x = 0
                while x < w:
                    n = data[pos]
                    pos += 1
                    if n > 128:  # run
                        img[y, x:x + n - 128, c] = data[pos]
                        pos += 1
                        x += n - 128
                    else:
                        img[y, x:x + n, c] = np.frombuffer(data, np.uint8, n, pos)
                        pos += n
                        x += n
        else:
            img[y] = np.frombuffer(data, np.uint8, 4 * w, pos).reshape(w, 4)
            pos += 4 * w
    e = img[..., 3].astype(np.int32)
    scale = np.where(e > 0, np.ldexp(1.0, e - 136), 0.0)
    return img[..., :3] * scale[..., None]


@pytest.mark.parametrize("shape", [(7, 5), (64, 300), (3, 1)])
def test_png_round_trip(tmp_path, shape):
    rng = np.random.default_rng(shape[0])
    img = rng.integers(0, 256, shape + (3,), dtype=np.uint8)
    p = tmp_path / "x.png"
    mt.write_png(p, img)
    np.testing.assert_array_equal(gltf.decode_png(p.read_bytes()), img)


def test_png_larger_than_one_stored_block(tmp_path):
    img = np.arange(200 * 150 * 3, dtype=np.uint32).astype(np.uint8).reshape(150, 200, 3)  # > 65535 raw bytes
    p = tmp_path / "big.png"
    mt.write_png(p, img)
    np.testing.assert_array_equal(gltf.decode_png(p.read_bytes()), img)


@pytest.mark.parametrize("width", [5, 40, 300])
def test_hdr_round_trip(tmp_path, width):
    rng = np.random.default_rng(width)
    img = (rng.random((6, width, 3)) * np.logspace(-3, 3, width)[None, :, None]).astype(np.float32)
    img[0, 0] = 0.0
    p = tmp_path / "x.hdr"
    mt.write_hdr(p, img)
    back = read_hdr(p)
    m = img.max(axis=-1, keepdims=True)
    assert np.all(np.abs(back - img) <= m / 128 + 1e-30)
    assert np.all(back[0, 0] == 0)


@pytest.mark.gpu
def test_device_rgb8_conversion():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(3)
    img = rng.uniform(-0.5, 1.5, (37, 53, 3)).astype(np.float32)
    img[0, 0] = [1.0, 0.0, 254.9 / 255]
    d = torch.from_numpy(img).cuda()
    out = torch.zeros(img.shape, dtype=torch.uint8, device="cuda")
    mt.image_rgb8_device(d.data_ptr(), 53, 37, out.data_ptr(), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    expect = np.clip(img * np.float32(255), 0, 255).astype(np.uint8)
    np.testing.assert_array_equal(out.cpu().numpy(), expect)
