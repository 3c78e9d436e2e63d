"""Generates the golden fixtures of tests/golden/ from the CPU oracle.

The reference cannot be built or run here (its path needs Kokkos, Eigen and
Open3D and is hard-wired to Kokkos::Cuda), so the fixtures freeze the
oracle's outputs on small seeded inputs; the inputs are stored too, so the
fixtures do not depend on the synthetic-scene generator staying bit-stable
across machines. Run from the repository root:

    python tests/golden/make_golden.py

Cases (config-1 room, 2x2x2 m, 6 spheres + 4 boxes, 80x60 images;
reference fusion at 10 mm voxels, truncation 30 mm):
  ref_fusion.npz  integrate frames 0 and 1 with colour, deintegrate frame 1,
                  integrate frame 2; sparse dump of the map (keys, coords,
                  sdf and w of the voxels with w != 0), the reference
                  raycast (points and colour) of the result, the pcd normals
                  of frame 0, kokkosICP (both types) of frame 0 against 1.
  method.npz      FP64 method: three fusions at 4 mm (nearest pixel), the
                  trilinear raycast maps at frame 2 (<= 128 steps), and one
                  point-to-plane tracking solve of frame 2 from a start
                  pose 1 cm / 0.5 deg off.
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import oracle  # noqa: E402
from superscanner_gb300 import synth  # noqa: E402

OUT = Path(__file__).resolve().parent
ROWS, COLS = 60, 80
INTR = (65.625, 65.625, 39.5, 29.5)


def sparse_dump(d: dict) -> dict:
    nz = np.nonzero(d["w"])
    return {"keys": d["keys"], "coords": d["coords"], "vox_block": nz[0].astype(np.int32),
            "vox_index": nz[1].astype(np.int16), "sdf": d["sdf"][nz], "w": d["w"][nz]}


def main() -> None:
    sc = synth.Scene(1, 1234)
    P = sc.trajectory(40, 42)[[0, 12, 24]]
    depth, rgb = sc.render(P, ROWS, COLS, INTR, noise=True, noise_seed=7)

    g = oracle.OracleGrid(0.01, 0.03, ROWS, COLS, intr=INTR)  # 10 mm voxels keep the dump small
    for k in (0, 1):
        g.integrate(depth[k], rgb[k], P[k].astype(np.float32))
    g.deintegrate(depth[1], rgb[1], P[1].astype(np.float32))
    g.integrate(depth[2], rgb[2], P[2].astype(np.float32))
    dump = sparse_dump(g.export())
    pcd, col = g.raycast(P[2].astype(np.float32))
    nrm = oracle.normals(oracle.depth_to_pcd(depth[0], INTR))
    icp = {}
    for kind in (0, 1):
        T, rmse, _ = oracle.kokkos_icp(depth[0], depth[1], P[0], P[0], kind, INTR)
        icp[f"icp{kind}_T"], icp[f"icp{kind}_rmse"] = T, np.float32(rmse)
    np.savez_compressed(OUT / "ref_fusion.npz", depth=depth, rgb=rgb, poses=P, intr=np.array(INTR),
                        ray_pcd=pcd, ray_col=col, normals0=nrm, **{f"map_{k}": v for k, v in dump.items()}, **icp)

    m = oracle.MethodGrid64(0.004, 0.016, ROWS, COLS, INTR, 255)
    for k in range(3):
        m.fuse(depth[k], P[k])
    vmap, nmap, steps = m.raycast(P[2], 128, 0.2, 10.0)
    c, sn = np.cos(np.radians(0.5)), np.sin(np.radians(0.5))
    D = np.array([[c, -sn, 0, 0.006], [sn, c, 0, -0.005], [0, 0, 1, 0.006], [0, 0, 0, 1.0]])
    start = P[2] @ D
    T, inl = oracle.track64(depth[2], vmap, nmap, P[2], start, INTR, iters=(6, 4, 3))
    np.savez_compressed(OUT / "method.npz", depth=depth, poses=P, intr=np.array(INTR), vmap=vmap, nmap=nmap,
                        steps=steps, track_start=start, track_T=T, track_inliers=np.int64(inl))
    for f in ("ref_fusion.npz", "method.npz"):
        print(f, (OUT / f).stat().st_size, "bytes")


if __name__ == "__main__":
    main()
