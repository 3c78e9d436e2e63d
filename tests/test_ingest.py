"""Frame ingest in the reference's layout (DataCam.cpp:10-100): PNG decoding
(every row filter type, 16-bit grey and 8-bit RGB), intrinsic.txt, the
zero-padded frame names with their plain fallback, nearest-neighbour resize."""
import numpy as np
import pytest

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
    from superscanner_gb300 import GPUVoxelGrid, synth
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
