"""Writes the fixtures of tests/golden/ that come from the reference's OWN code.

The reference's hot-path sources (GPUVoxelGrid.cpp, kokkosICP.cpp,
imageutil.cpp, kokkosUtil.cpp, kokkosFunctions.cpp) are compiled unchanged by
``make -C oracle ref`` against oracle/ref_stub (stand-ins for Kokkos, Eigen,
Open3D and OpenCV) into oracle/_ref/libss_ref.so; this script drives that
library through oracle/ref.py. It needs the reference checkout, so it runs
where the checkout is; the fixtures it writes travel with the repository.
Run from the repository root:

    python tests/golden/make_ref_golden.py

Fixtures:
  ref_fusion.npz   config-1 room at 80x60 (10 mm voxels, truncation 30 mm):
                   integrate frames 0 and 1 with colour, deintegrate frame 1,
                   integrate frame 2; sparse dump of the map (keys, coords, sdf
                   and w of the voxels with w != 0); raycast points and colour
                   at frame 2; pcd normals of frame 0; kokkosICP of frame 0
                   against 1 (both types). Inputs stored.
  ref_config1.npz  the config1 sequence of tests/refcases.py (640x480, 100
                   frames, 5 mm, 2^18 blocks, colour): frame CRCs, poses,
                   per-block digests and coordinates after the sequence,
                   per-row raycast digests at 11 poses, kokkosICP of 5 pairs
                   (both types) with perturbed starts.
  ref_config2.npz  the config2 sequence (config-2 frames: 4 mm, noise and
                   dropout, 2^20 blocks, depth only), same contents.

It also prints how far a build of the same sources that contracts a*b+c into
fused multiply-adds (oracle/_ref/libss_ref_fma.so, -ffp-contract=fast) moves
the results, for the record of the reference's own FMA sensitivity.
"""
from __future__ import annotations

import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))

import synth  # noqa: E402
from oracle import ref  # noqa: E402
import refcases  # noqa: E402

OUT = Path(__file__).resolve().parent
ROWS, COLS = 60, 80
INTR_SMALL = (65.625, 65.625, 39.5, 29.5)


def sparse_dump(d: dict) -> dict:
    nz = np.nonzero(d["w"])
    return {"keys": d["keys"], "coords": d["coords"], "vox_block": nz[0].astype(np.int32),
            "vox_index": nz[1].astype(np.int16), "sdf": d["sdf"][nz], "w": d["w"][nz].astype(np.float32)}


def small_fixture() -> None:
    sc = synth.Scene(1, 1234)
    P = sc.trajectory(40, 42)[[0, 12, 24]]
    depth, rgb = sc.render(P, ROWS, COLS, INTR_SMALL, noise=True, noise_seed=7)
    g = ref.RefGrid(0.01, 0.03, ROWS, COLS, intr=INTR_SMALL)
    for k in (0, 1):
        g.integrate(depth[k], rgb[k], P[k].astype(np.float32))
    g.deintegrate(depth[1], rgb[1], P[1].astype(np.float32))
    g.integrate(depth[2], rgb[2], P[2].astype(np.float32))
    dump = sparse_dump(g.export())
    pcd, col = g.raycast(P[2].astype(np.float32))
    nrm = ref.normals(ref.depth_to_pcd(depth[0], INTR_SMALL))
    icp = {}
    for kind in (0, 1):
        T, rmse = ref.kokkos_icp(depth[0], depth[1], P[0], P[0], kind, INTR_SMALL)
        icp[f"icp{kind}_T"], icp[f"icp{kind}_rmse"] = T, np.float32(rmse)
    np.savez_compressed(OUT / "ref_fusion.npz", depth=depth, rgb=rgb, poses=P, intr=np.array(INTR_SMALL),
                        ray_pcd=pcd, ray_col=col, normals0=nrm, **{f"map_{k}": v for k, v in dump.items()}, **icp)


def case_fixture(case: str, fma: bool = False) -> dict:
    c = refcases.CASES[case]
    P = refcases.poses(case)
    depth, rgb = refcases.render(case, P)
    g = ref.RefGrid(c["vl"], c["trunc"], 480, 640, intr=refcases.INTR,
                    capacity_voxels=c["capacity_blocks"] * 512, fma=fma)
    r = refcases.run(case, g, depth, rgb, P)
    starts = refcases.icp_starts(case, P)
    T = np.zeros((len(starts), 2, 4, 4))
    rmse = np.zeros((len(starts), 2), np.float32)
    for p, ((a, b), (tx, ty)) in enumerate(zip(c["icp_pairs"], starts)):
        for kind in (0, 1):
            T[p, kind], rmse[p, kind] = ref.kokkos_icp(depth[a], depth[b], tx, ty, kind, refcases.INTR, fma=fma)
    r.update(icp_T=T, icp_rmse=rmse, crc=refcases.frame_crcs(depth, rgb), poses=P)
    return r


def main() -> None:
    assert ref.build(), "oracle/_ref could not be built: the reference checkout is needed"
    t = time.time()
    small_fixture()
    print(f"ref_fusion.npz ({time.time() - t:.1f} s)")
    for case in refcases.CASES:
        t = time.time()
        r = case_fixture(case)
        np.savez_compressed(OUT / f"ref_{case}.npz", **{k: v for k, v in r.items() if k != "last_pcd"})
        print(f"ref_{case}.npz: {len(r['coords'])} blocks, {r['observed']} observed voxels "
              f"({time.time() - t:.1f} s, {(OUT / f'ref_{case}.npz').stat().st_size} bytes)")
        if ref.available(fma=True):
            f = case_fixture(case, fma=True)
            same_blocks = np.array_equal(r["keys"], f["keys"])
            blocks_differ = int((r["digest"] != f["digest"]).sum()) if same_blocks else -1
            rows_differ = int((r["ray_rows"] != f["ray_rows"]).sum())
            d = np.linalg.norm(r["last_pcd"] - f["last_pcd"], axis=-1)
            both = (r["last_pcd"][..., 2] != 0) & (f["last_pcd"][..., 2] != 0)
            print(f"  contracted build: block set {'identical' if same_blocks else 'DIFFERENT'}, "
                  f"{blocks_differ} of {len(r['digest'])} block payloads differ, "
                  f"{rows_differ} of {r['ray_rows'].size} raycast rows differ, last raycast: "
                  f"p99.9 {1e3 * np.quantile(d[both], 0.999):.4f} mm, max {1e3 * d[both].max():.3f} mm, "
                  f"ICP max |dT| {np.abs(r['icp_T'] - f['icp_T']).max():.2e}")


if __name__ == "__main__":
    main()
