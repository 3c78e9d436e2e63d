"""Frame ingest in the reference's on-disk layout (src/cameras/DataCam.cpp:10-100,
src/utils/coreutil.cpp:381-457): ``<root>/depth/<NNNNNN>.png`` (16-bit grey,
millimetres; a plain number as fallback), ``<root>/color/<NNNNNN>.jpg`` or
``.png`` (8-bit RGB; JPEG decoded on the GPU by ``ss_jpeg_decode_rgb``),
``intrinsic.txt`` (width, height, then the 3x3 intrinsic matrix, one row per
line). Depth frames whose size differs from the target are resized with
nearest-neighbour sampling, as the reference does with OpenCV INTER_NEAREST;
colour frames bilinearly, as its cv::resize default (INTER_LINEAR). Depth
frames are returned in pinned host memory, ready for the pipeline's
asynchronous upload (``Pipeline.frame``)."""
from __future__ import annotations

import ctypes as C
import struct
import zlib
from pathlib import Path

import numpy as np
import torch

from ._native import check, lib

_PNG_SIG = b"\x89PNG\r\n\x1a\n"


def read_png(path) -> np.ndarray:
    """Decodes a non-interlaced PNG of colour type 0 (grey) or 2 (RGB), bit
    depth 8 or 16: [H, W] or [H, W, 3], uint8 or uint16."""
    data = Path(path).read_bytes()
    if data[:8] != _PNG_SIG:
        raise ValueError(f"{path}: not a PNG file")
    pos, idat, hdr = 8, [], None
    while pos < len(data):
        n, kind = struct.unpack(">I4s", data[pos:pos + 8])
        body = data[pos + 8:pos + 8 + n]
        if kind == b"IHDR":
            hdr = struct.unpack(">IIBBBBB", body)
        elif kind == b"IDAT":
            idat.append(body)
        elif kind == b"IEND":
            break
        pos += 12 + n
    if hdr is None:
        raise ValueError(f"{path}: no IHDR")
    w, h, depth, ctype, _, _, interlace = hdr
    if ctype not in (0, 2) or depth not in (8, 16) or interlace != 0:
        raise ValueError(f"{path}: unsupported PNG (colour type {ctype}, depth {depth}, interlace {interlace})")
    channels = 1 if ctype == 0 else 3
    bpp = channels * depth // 8
    raw = np.frombuffer(zlib.decompress(b"".join(idat)), np.uint8)
    row_bytes = w * bpp
    if raw.size != h * (row_bytes + 1):
        raise ValueError(f"{path}: image data of unexpected size")
    out = np.empty(h * row_bytes, np.uint8)
    check(lib.ss_png_unfilter(C.c_void_p(raw.ctypes.data), h, row_bytes, bpp, C.c_void_p(out.ctypes.data)),
          "png_unfilter")
    img = out.view(">u2").astype(np.uint16) if depth == 16 else out
    return img.reshape((h, w) if channels == 1 else (h, w, 3))


def write_png(path, img: np.ndarray, filter_type: int = 0) -> None:
    """Encodes a [H, W] (grey) or [H, W, 3] (RGB) uint8 / uint16 image with
    one PNG row filter type (0..4) on every row."""
    img = np.asarray(img)
    if img.dtype not in (np.uint8, np.uint16) or img.ndim not in (2, 3):
        raise ValueError("uint8 / uint16 [H, W] or [H, W, 3] expected")
    h, w = img.shape[:2]
    channels = 1 if img.ndim == 2 else img.shape[2]
    depth = 16 if img.dtype == np.uint16 else 8
    bpp = channels * depth // 8
    rows = (img.astype(">u2") if depth == 16 else img).reshape(h, -1).view(np.uint8).reshape(h, -1).astype(np.int32)
    left = np.zeros_like(rows)
    left[:, bpp:] = rows[:, :-bpp]
    up = np.zeros_like(rows)
    up[1:] = rows[:-1]
    upleft = np.zeros_like(rows)
    upleft[1:, bpp:] = rows[:-1, :-bpp]
    if filter_type == 0:
        pred = np.zeros_like(rows)
    elif filter_type == 1:
        pred = left
    elif filter_type == 2:
        pred = up
    elif filter_type == 3:
        pred = (left + up) >> 1
    elif filter_type == 4:
        p = left + up - upleft
        pa, pb, pc = np.abs(p - left), np.abs(p - up), np.abs(p - upleft)
        pred = np.where((pa <= pb) & (pa <= pc), left, np.where(pb <= pc, up, upleft))
    else:
        raise ValueError("filter type 0..4")
    filt = ((rows - pred) & 0xFF).astype(np.uint8)
    body = np.concatenate([np.full((h, 1), filter_type, np.uint8), filt], axis=1).tobytes()

    def chunk(kind, payload):
        return struct.pack(">I", len(payload)) + kind + payload + struct.pack(">I", zlib.crc32(kind + payload))

    ihdr = struct.pack(">IIBBBBB", w, h, depth, 0 if channels == 1 else 2, 0, 0, 0)
    Path(path).write_bytes(_PNG_SIG + chunk(b"IHDR", ihdr) + chunk(b"IDAT", zlib.compress(body, 6)) +
                           chunk(b"IEND", b""))


def read_intrinsic(path):
    """(width, height, fx, fy, cx, cy) of an intrinsic.txt (setFromIntrinsicFile,
    coreutil.cpp:381-430)."""
    lines = [ln.split() for ln in Path(path).read_text().splitlines() if ln.strip()]
    width, height = int(lines[0][0]), int(lines[1][0])
    K = np.array([[float(v) for v in ln[:3]] for ln in lines[2:5]])
    return width, height, K[0, 0], K[1, 1], K[0, 2], K[1, 2]


def resize_nearest(img: np.ndarray, rows: int, cols: int) -> np.ndarray:
    """Nearest-neighbour resize (source index floor(dst index x src / dst), as
    OpenCV INTER_NEAREST)."""
    h, w = img.shape[:2]
    if (h, w) == (rows, cols):
        return img
    ii = np.minimum((np.arange(rows) * h) // rows, h - 1)
    jj = np.minimum((np.arange(cols) * w) // cols, w - 1)
    return img[ii][:, jj]


def resize_bilinear(img: np.ndarray, rows: int, cols: int) -> np.ndarray:
    """[H, W, C] uint8 resized bilinearly with cv::resize's INTER_LINEAR
    geometry (source coordinate (d + 0.5) src / dst - 0.5, clamped to the
    first and last pixel), rounded to nearest; the host twin of
    ss_resize_rgb."""
    h, w = img.shape[:2]
    if (h, w) == (rows, cols):
        return img

    def axis(n_dst, n_src):
        f = (np.arange(n_dst) + 0.5) * (n_src / n_dst) - 0.5
        i0 = np.floor(f).astype(np.int64)
        a = f - i0
        a[i0 < 0] = 0.0
        i0 = np.maximum(i0, 0)
        a[i0 >= n_src - 1] = 0.0
        i0 = np.minimum(i0, n_src - 1)
        return i0, np.minimum(i0 + 1, n_src - 1), a

    y0, y1, ay = axis(rows, h)
    x0, x1, ax = axis(cols, w)
    f = img.astype(np.float64)
    top = f[y0][:, x0] + ax[None, :, None] * (f[y0][:, x1] - f[y0][:, x0])
    bot = f[y1][:, x0] + ax[None, :, None] * (f[y1][:, x1] - f[y1][:, x0])
    out = top + ay[:, None, None] * (bot - top)
    return np.clip(np.rint(out), 0, 255).astype(np.uint8)


class JpegDecoder:
    """JPEG -> RGB on the GPU (ss_jpeg_*, nvJPEG); one per host thread."""

    def __init__(self):
        self._h = C.c_void_p()
        check(lib.ss_jpeg_create(C.byref(self._h)), "jpeg_create")

    def close(self):
        if self._h:
            lib.ss_jpeg_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def info(self, data: bytes) -> tuple[int, int]:
        r, c = C.c_int32(), C.c_int32()
        check(lib.ss_jpeg_info(self._h, data, len(data), C.byref(r), C.byref(c)), "jpeg_info")
        return r.value, c.value

    def decode(self, data: bytes, rows: int | None = None, cols: int | None = None, stream=None) -> torch.Tensor:
        """CUDA uint8 tensor [rows, cols, 3] (the image's own size by default)."""
        if rows is None or cols is None:
            rows, cols = self.info(data)
        out = torch.empty((rows, cols, 3), dtype=torch.uint8, device="cuda")
        sp = C.c_void_p(stream.cuda_stream) if stream is not None else C.c_void_p()
        check(lib.ss_jpeg_decode_rgb(self._h, data, len(data), C.c_void_p(out.data_ptr()), rows, cols, sp),
              "jpeg_decode_rgb")
        return out


def frame_name(k: int) -> str:
    """getPicNumberString (coreutil.cpp:449-457): zero-padded to 6 digits."""
    return str(k).rjust(6, "0")


class FrameReader:
    """Depth (and PNG colour) frames of a recording in the reference's layout,
    resized to rows x cols, returned in pinned host memory."""

    def __init__(self, root, rows: int = 480, cols: int = 640):
        self.root = Path(root)
        self.rows, self.cols = rows, cols
        self._jpeg = None

    def _find(self, sub: str, k: int, ext: str):
        for name in (frame_name(k), str(k)):
            p = self.root / sub / f"{name}.{ext}"
            if p.exists():
                return p
        return None

    def depth(self, k: int, pinned: bool = True):
        p = self._find("depth", k, "png")
        if p is None:
            raise FileNotFoundError(f"no depth image {k} under {self.root / 'depth'}")
        img = read_png(p)
        if img.dtype != np.uint16 or img.ndim != 2:
            raise ValueError(f"{p}: 16-bit grey expected")
        img = np.ascontiguousarray(resize_nearest(img, self.rows, self.cols))
        if not pinned:
            return img
        t = torch.empty((self.rows, self.cols), dtype=torch.int16).pin_memory()
        t.numpy()[:] = img.view(np.int16)
        return t

    def color(self, k: int, device: bool = False):
        """RGB frame k resized to rows x cols (None when there is none): the
        reference's order color/<NNNNNN>.jpg, color/<NNNNNN>.png, color/<k>.jpg
        (DataCam.cpp:30-46). A JPEG is decoded and resized on the GPU; a CUDA
        tensor if device, else a host array."""
        zp, plain = self.root / "color" / frame_name(k), self.root / "color" / str(k)
        for p in (zp.with_suffix(".jpg"), zp.with_suffix(".png"), plain.with_suffix(".jpg")):
            if not p.exists():
                continue
            if p.suffix == ".jpg":
                if self._jpeg is None:
                    self._jpeg = JpegDecoder()
                t = self._jpeg.decode(p.read_bytes(), self.rows, self.cols)
                return t if device else t.cpu().numpy()
            img = read_png(p)
            if img.dtype != np.uint8:
                raise ValueError(f"{p}: 8-bit colour expected")
            if img.ndim == 2:
                img = np.repeat(img[..., None], 3, axis=2)
            img = np.ascontiguousarray(resize_bilinear(img[..., :3], self.rows, self.cols))
            return torch.from_numpy(img).cuda() if device else img
        return None
