"""Reference-semantics sequences pinned by the reference's own code.

Each case is a sequence of integrate / deIntegrate / raycast / cleanMemory
calls (GPUVoxelGrid.cpp:41-196, 561-715) plus kokkosICP pairs
(kokkosICP.cpp:25-210) on seeded synthetic frames. tests/golden/make_ref_golden.py
runs them on the reference's code (oracle/_ref) and stores digests in
tests/golden/ref_<case>.npz; the tests run the same sequences on the oracle
(CPU) and on the CUDA path and compare digests.

Digests are 64-bit weighted sums (mod 2^64) of the bit patterns of every
value, -0.0 folded into +0.0, so that equal digests mean equal values:
  blocks   one digest per block (sdf bits, weight, r/g/b bits of its 512
           voxels), blocks sorted by key, plus the block coordinates;
  raycast  one digest per image row of the points (and of the colours).
Frames are re-rendered from the stored poses; a CRC of every rendered frame is
stored and checked first, so a renderer that drifts fails loudly.
"""
from __future__ import annotations

import zlib

import numpy as np

INTR = (525.0, 525.0, 319.5, 239.5)

# Config 1 (the reference's CPU-runnable case): 2x2x2 m room, 6 spheres + 4
# boxes, 100-frame trajectory, 640x480, 5 mm voxels, truncation 4 voxels,
# 2^18 blocks of capacity, FP32 TSDF with colour.
# Config 2 frames through the reference semantics: 4x4x3 m room, 40
# primitives, depth noise and 5 % dropout, 4 mm voxels, 2^20 blocks; depth only.
CASES = {
    "config1": dict(kind=1, n=100, step=1, vl=0.005, trunc=0.02, capacity_blocks=1 << 18, noise=False, color=True,
                    raycast_at=tuple(range(9, 100, 10)), deint=(95, 96, 97, 98, 99),
                    icp_pairs=((10, 12), (30, 34), (50, 56), (70, 78), (88, 98))),
    "config2": dict(kind=2, n=20, step=3, vl=0.004, trunc=0.016, capacity_blocks=1 << 20, noise=True, color=False,
                    raycast_at=(4, 9, 14, 19), deint=(17, 18, 19),
                    icp_pairs=((0, 2), (3, 7), (5, 11), (8, 16), (9, 19))),
}
ICP_PERTURB_SEED = 2024


def poses(case: str) -> np.ndarray:
    import synth
    c = CASES[case]
    sc = synth.Scene(c["kind"], 1234)
    return sc.trajectory(c["n"] * c["step"], 42)[::c["step"]]


def render(case: str, P: np.ndarray):
    import synth
    c = CASES[case]
    sc = synth.Scene(c["kind"], 1234)
    depth, rgb = sc.render(P, 480, 640, INTR, noise=c["noise"], noise_seed=7)
    return depth, (rgb if c["color"] else None)


def frame_crcs(depth, rgb) -> np.ndarray:
    out = np.zeros(len(depth), np.uint32)
    for k in range(len(depth)):
        crc = zlib.crc32(np.ascontiguousarray(depth[k]).tobytes())
        if rgb is not None:
            crc = zlib.crc32(np.ascontiguousarray(rgb[k]).tobytes(), crc)
        out[k] = crc
    return out


def icp_starts(case: str, P: np.ndarray):
    """(tx, ty) per pair: ty the later frame's pose, tx the earlier's moved by a
    seeded rigid perturbation of at most 0.5 deg / 5 mm (so Txy starts off)."""
    rng = np.random.default_rng(ICP_PERTURB_SEED)
    out = []
    for a, b in CASES[case]["icp_pairs"]:
        ax = rng.normal(size=3)
        ax /= np.linalg.norm(ax)
        ang = np.radians(rng.uniform(0.1, 0.5))
        K = np.array([[0, -ax[2], ax[1]], [ax[2], 0, -ax[0]], [-ax[1], ax[0], 0]])
        D = np.eye(4)
        D[:3, :3] = np.eye(3) + np.sin(ang) * K + (1 - np.cos(ang)) * K @ K
        D[:3, 3] = rng.uniform(-0.005, 0.005, 3)
        out.append((P[a] @ D, P[b].copy()))
    return out


_W = np.random.default_rng(0x5EED).integers(1, 1 << 63, size=(5, 512), dtype=np.uint64) | np.uint64(1)
_RW = np.random.default_rng(0x0DD).integers(1, 1 << 63, size=(2, 640 * 3), dtype=np.uint64) | np.uint64(1)


def _bits(a) -> np.ndarray:
    a = np.ascontiguousarray(a, np.float32) + np.float32(0.0)  # -0.0 -> +0.0
    return a.view(np.uint32).astype(np.uint64)


def block_digest(sdf, w, rgb=None) -> np.ndarray:
    """One u64 per block from sdf [n, 512], integer weights [n, 512], rgb [n, 3, 512]."""
    with np.errstate(over="ignore"):
        h = (_bits(sdf) * _W[0]).sum(axis=1, dtype=np.uint64)
        h += (np.asarray(w).astype(np.int64).astype(np.uint64) * _W[1]).sum(axis=1, dtype=np.uint64)
        if rgb is not None:
            for c in range(3):
                h += (_bits(rgb[:, c]) * _W[2 + c]).sum(axis=1, dtype=np.uint64)
    return h


def row_digest(img, which: int = 0) -> np.ndarray:
    """One u64 per row of an [rows, cols, 3] float image."""
    rows = img.shape[0]
    b = _bits(img).reshape(rows, -1)
    with np.errstate(over="ignore"):
        return (b * _RW[which, :b.shape[1]]).sum(axis=1, dtype=np.uint64)


def run(case: str, grid, depth, rgb, P, with_colour_rows: bool = True) -> dict:
    """Runs the case's sequence on a grid adapter (integrate, deintegrate,
    raycast, clean, export: the oracle's and the references's interfaces;
    the GPU tests wrap GPUVoxelGrid in the same shape) and returns its digests."""
    c = CASES[case]
    E = P.astype(np.float32)
    ray_rows, col_rows, ray_poses = [], [], []
    for k in range(c["n"]):
        grid.integrate(depth[k], rgb[k] if rgb is not None else None, E[k], c["color"])
        if k in c["raycast_at"]:
            pcd, col = grid.raycast(E[k])
            ray_rows.append(row_digest(pcd, 0))
            col_rows.append(row_digest(col, 1))
            ray_poses.append(k)
    for k in c["deint"]:
        grid.deintegrate(depth[k], rgb[k] if rgb is not None else None, E[k], c["color"])
    pcd, col = grid.raycast(E[c["n"] - 1])
    ray_rows.append(row_digest(pcd, 0))
    col_rows.append(row_digest(col, 1))
    ray_poses.append(-1)
    before_clean = grid.count()
    grid.clean()
    d = grid.export()
    return dict(coords=d["coords"].astype(np.int16), keys=d["keys"],
                digest=block_digest(d["sdf"], d["w"], d["rgb"] if c["color"] else None),
                observed=int((np.asarray(d["w"]) != 0).sum()), blocks_before_clean=int(before_clean),
                ray_rows=np.stack(ray_rows), col_rows=np.stack(col_rows), ray_frames=np.array(ray_poses),
                last_pcd=pcd)
