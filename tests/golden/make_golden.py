"""Generates the method fixture of tests/golden/ from the FP64 method oracle.

The per-frame method (trilinear raycast, Gauss-Newton tracker) has no
counterpart in the reference, so its fixture freezes the FP64 oracle's
outputs; the reference-semantics fixtures (ref_*.npz) come from the
reference's own code (make_ref_golden.py). Inputs are stored, so the fixture
does not depend on the synthetic-scene generator staying bit-stable across
machines. Run from the repository root:

    python tests/golden/make_golden.py

  method.npz      config-1 room, 80x60 images: three FP64 fusions at 4 mm
                  (nearest pixel), the trilinear raycast maps at frame 2
                  (<= 128 steps), and one point-to-plane tracking solve of
                  frame 2 from a start pose 1 cm / 0.5 deg off.
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import oracle  # noqa: E402
import synth  # noqa: E402

OUT = Path(__file__).resolve().parent
ROWS, COLS = 60, 80
INTR = (65.625, 65.625, 39.5, 29.5)


def main() -> None:
    sc = synth.Scene(1, 1234)
    P = sc.trajectory(40, 42)[[0, 12, 24]]
    depth, rgb = sc.render(P, ROWS, COLS, INTR, noise=True, noise_seed=7)

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
    for f in ("method.npz",):
        print(f, (OUT / f).stat().st_size, "bytes")


if __name__ == "__main__":
    main()
