"""Frame ingest in the reference's layout (DataCam.cpp:10-100): PNG decoding
(every row filter type, 16-bit grey and 8-bit RGB), intrinsic.txt, the
zero-padded frame names with their plain fallback, nearest-neighbour resize."""
import numpy as np
import pytest

from superscanner_gb300._native import SSError
from superscanner_gb300.ingest import FrameReader, frame_name, read_intrinsic, read_png, resize_nearest, write_png


@pytest.mark.parametrize("filt", [0, 1, 2, 3, 4])
def test_png_round_trip(tmp_path, filt):
    rng = np.random.default_rng(filt)
    depth = rng.integers(0, 65536, size=(37, 53), dtype=np.uint16)
    depth[5:9, 10:30] = 1234  # flat runs exercise the predictors
    write_png(tmp_path / "d.png", depth, filt)
    assert np.array_equal(read_png(tmp_path / "d.png"), depth)
    rgb = rng.integers(0, 256, size=(21, 19, 3), dtype=np.uint8)
    write_png(tmp_path / "c.png", rgb, filt)
    assert np.array_equal(read_png(tmp_path / "c.png"), rgb)


def test_intrinsic_file(tmp_path):
    (tmp_path / "intrinsic.txt").write_text("640\n480\n525 0 319.5\n0 525 239.5\n0 0 1\n")
    assert read_intrinsic(tmp_path / "intrinsic.txt") == (640, 480, 525.0, 525.0, 319.5, 239.5)


def test_frame_reader_names_and_resize(tmp_path):
    (tmp_path / "depth").mkdir()
    a = (np.arange(240 * 320, dtype=np.uint32) % 5000).astype(np.uint16).reshape(240, 320)
    write_png(tmp_path / "depth" / (frame_name(3) + ".png"), a, 4)
    write_png(tmp_path / "depth" / "7.png", a[::-1].copy(), 1)  # plain-number fallback
    r = FrameReader(tmp_path, rows=480, cols=640)
    d3 = r.depth(3, pinned=False)
    assert d3.shape == (480, 640) and np.array_equal(d3, np.repeat(np.repeat(a, 2, 0), 2, 1))
    assert np.array_equal(r.depth(7, pinned=False)[::2, ::2], a[::-1])
    assert frame_name(3) == "000003"
    assert r.color(3) is None
    with pytest.raises(FileNotFoundError):
        r.depth(4, pinned=False)
    # downscale picks floor(i * src / dst)
    big = np.arange(10 * 10).reshape(10, 10)
    assert np.array_equal(resize_nearest(big, 4, 4), big[[0, 2, 5, 7]][:, [0, 2, 5, 7]])


@pytest.mark.gpu
def test_ingested_frames_drive_the_pipeline(tmp_path):
    """Depth frames written as PNGs, read back into pinned memory and fed to
    the pipeline (asynchronous upload) track like the same frames on the GPU."""
    import torch
    import synth
    from superscanner_gb300 import GPUVoxelGrid
    from superscanner_gb300.pipeline import Pipeline
    INTR = (525.0, 525.0, 319.5, 239.5)
    sc = synth.Scene(2, 1234)
    P = sc.trajectory(6, 42)
    depth, _ = sc.render(P, 480, 640, INTR, noise=True, noise_seed=7, color=False)
    (tmp_path / "depth").mkdir()
    for k in range(6):
        write_png(tmp_path / "depth" / (frame_name(k) + ".png"), depth[k], k % 5)
    reader = FrameReader(tmp_path)
    poses = {}
    for source in ("png", "device"):
        g = GPUVoxelGrid(int(1e9), 0.016, 0.004, 480, 640, storage="f16", with_color=False, hash_buckets=1 << 18,
                         max_weight=255)
        g.setIntrinsic(*INTR)
        pipe = Pipeline(g, use_graph=False, persistent_track=True)
        pipe.set_pose(P[0])
        out = []
        for k in range(6):
            frame = reader.depth(k) if source == "png" else \
                torch.from_numpy(np.ascontiguousarray(depth[k].view(np.int16))).cuda()
            pipe.frame(frame, track=k > 0)
            out.append(pipe.pose())
        g.sync()
        poses[source] = out
        pipe.close()
        g.close()
    for a, b in zip(poses["png"], poses["device"]):
        assert np.array_equal(a, b)


def _smooth_rgb(rows, cols, seed=0):
    yy, xx = np.mgrid[0:rows, 0:cols].astype(np.float64)
    rng = np.random.default_rng(seed)
    img = np.stack([128 + 90 * np.sin(xx / 17.0 + 0.3), 128 + 80 * np.cos(yy / 13.0),
                    60 + 0.9 * xx + 0.5 * yy], -1) + rng.normal(0, 1.5, (rows, cols, 3))
    return np.clip(np.rint(img), 0, 255).astype(np.uint8)


def test_jpeg_test_encoder_is_sane():
    """The test-side JPEG encoder: SOI / EOI, its segments in order, and a
    reconstruction close to the input (4:4:4 at quality 95)."""
    import jpeg_encode
    img = _smooth_rgb(45, 70)
    data, rec = jpeg_encode.encode(img, 95, subsample=False)
    assert data[:2] == b"\xff\xd8" and data[-2:] == b"\xff\xd9"
    for m in (b"\xff\xdb", b"\xff\xc0", b"\xff\xc4", b"\xff\xda"):
        assert m in data
    mse = np.mean((rec.astype(np.float64) - img) ** 2)
    assert 10 * np.log10(255.0 ** 2 / mse) > 35.0


def test_resize_bilinear_known_answers():
    """cv::resize INTER_LINEAR geometry: 2 -> 4 pixels gives 0, 25, 75, 100
    (source coordinates -0.25 clamped, 0.25, 0.75, 1.25 clamped); equal sizes
    are returned unchanged; a constant image stays constant."""
    from superscanner_gb300.ingest import resize_bilinear
    img = np.zeros((2, 2, 3), np.uint8)
    img[:, 1] = 100
    out = resize_bilinear(img, 2, 4)
    assert out[0, :, 0].tolist() == [0, 25, 75, 100]
    assert resize_bilinear(img, 2, 2) is img
    flat = np.full((7, 9, 3), 77, np.uint8)
    assert (resize_bilinear(flat, 13, 5) == 77).all()


@pytest.mark.gpu
@pytest.mark.parametrize("subsample", [False, True])
def test_jpeg_decodes_on_gpu(subsample):
    """nvJPEG through ss_jpeg_decode_rgb reproduces the test encoder's
    reconstruction (4:4:4: within the IDCT's rounding; 4:2:0: the decoder may
    interpolate chroma where the reconstruction replicates it)."""
    import jpeg_encode
    from superscanner_gb300.ingest import JpegDecoder
    img = _smooth_rgb(61, 83, seed=1)
    data, rec = jpeg_encode.encode(img, 90, subsample=subsample)
    dec = JpegDecoder()
    assert dec.info(data) == (61, 83)
    out = dec.decode(data).cpu().numpy()
    d = np.abs(out.astype(np.int32) - rec)
    if subsample:
        assert d.mean() < 1.5 and d.max() <= 16
    else:  # one level in Y and in Cr can become 1 + 1.402 in R
        assert d.mean() < 0.3 and d.max() <= 3
    with pytest.raises(SSError):
        dec.decode(b"\xff\xd8" + bytes(range(200)))
    dec.close()


@pytest.mark.gpu
def test_jpeg_colour_frames_resized_on_gpu(tmp_path):
    """A colour JPEG of another size is decoded and resized on the GPU like
    the host resize of the decoded image (to one level); the frame reader
    takes color/<NNNNNN>.jpg before .png, on the host or the device."""
    import jpeg_encode
    from superscanner_gb300.ingest import JpegDecoder, resize_bilinear
    img = _smooth_rgb(50, 70, seed=2)
    data, _ = jpeg_encode.encode(img, 92)
    dec = JpegDecoder()
    native = dec.decode(data).cpu().numpy()
    for rows, cols in ((120, 160), (24, 31)):
        gpu = dec.decode(data, rows, cols).cpu().numpy()
        assert np.abs(gpu.astype(np.int32) - resize_bilinear(native, rows, cols)).max() <= 1
    (tmp_path / "color").mkdir()
    (tmp_path / "color" / "000000.jpg").write_bytes(data)
    write_png(tmp_path / "color" / "000000.png", np.zeros((50, 70, 3), np.uint8))
    r = FrameReader(tmp_path, rows=120, cols=160)
    host = r.color(0)
    assert host.shape == (120, 160, 3) and host.dtype == np.uint8
    assert np.abs(host.astype(np.int32) - resize_bilinear(native, 120, 160)).max() <= 1
    assert np.array_equal(r.color(0, device=True).cpu().numpy(), host)
