"""Differentiable raycast: GPU forward loss against the FP64 oracle, and the
hand-written adjoint (pose se(3) and voxel TSDF gradients) against the FP64
adjoint on a fused scene, against FP64 central finite differences
(h = 1e-4 on the pose twist, 1e-3 of the truncation on voxels) on a smooth
analytic wall, and against FP64 pose differences on the fused FP16 room with
the pixel set frozen."""
import numpy as np
import pytest
import torch

import oracle
import synth
from superscanner_gb300 import GPUVoxelGrid
from superscanner_gb300.raydiff import raycast_loss, raycast_loss_grad, se3_exp
from scenes import wavy_wall, VL as WVL, TRUNC as WTRUNC

pytestmark = pytest.mark.gpu

INTR = (525.0, 525.0, 319.5, 239.5)
VL, TRUNC = 0.004, 0.016


def setup(storage="f32"):
    sc = synth.Scene(2, 1234)
    P = sc.trajectory(8, 42)
    depth, _ = sc.render(P, 480, 640, INTR, noise=True, noise_seed=7, color=False)
    dev = [torch.from_numpy(np.ascontiguousarray(d.view(np.int16))).cuda() for d in depth]
    g = GPUVoxelGrid(int(1e9), TRUNC, VL, 480, 640, storage=storage, with_color=False, hash_buckets=1 << 18,
                     max_weight=255)
    g.setIntrinsic(*INTR)
    for k in range(8):
        g.integrate_fast(dev[k], P[k].astype(np.float32))
    g.sync()
    d = g.export_blocks(with_color=False)
    o = oracle.MethodGrid64(VL, TRUNC, 480, 640, INTR, 255)
    o.import_blocks(d["coords"], d["sdf"], d["w"])
    return g, o, d, P, depth, dev


def test_forward_loss_matches_fp64():
    g, o, d, P, depth, dev = setup()
    T = se3_exp([0.004, -0.003, 0.002, 0.006, -0.004, 0.003]) @ P[7]
    L, nv = raycast_loss(g, T, dev[7])
    L64, nv64 = o.raycast_loss(T, depth[7])
    print("loss gpu", L, nv, "fp64", L64, nv64)
    assert nv > 100000 and abs(nv - nv64) <= 1e-3 * nv64
    assert abs(L - L64) <= 1e-3 * L64


def test_pose_adjoint_matches_fp64_adjoint():
    """On a fused scene the GPU adjoint (FP32) equals the FP64 restatement of
    the same formulas; finite differences are not usable here because pixels
    at silhouettes and dropout enter and leave the loss."""
    g, o, d, P, depth, dev = setup()
    T = se3_exp([0.004, -0.003, 0.002, 0.006, -0.004, 0.003]) @ P[7]
    L, grad, nv = raycast_loss_grad(g, T, dev[7])
    L64, grad64 = o.raycast_loss_grad(T, depth[7])
    print("pose grad gpu", grad, "\n         fp64", grad64)
    assert abs(L - L64) <= 1e-3 * L64
    assert np.abs(grad - grad64).max() <= 0.02 * np.abs(grad64).max()


def wall_grid(storage):
    coords, sdf, w, obs, intr = wavy_wall()
    rows, cols = obs.shape
    g = GPUVoxelGrid(int(1e9), WTRUNC, WVL, rows, cols, storage=storage, with_color=False, hash_buckets=1 << 17,
                     max_weight=255)
    g.setIntrinsic(*intr)
    g.import_blocks(coords, sdf, w)
    g.sync()
    d = g.export_blocks(with_color=False)  # the stored (for F16: quantized) field
    o = oracle.MethodGrid64(WVL, WTRUNC, rows, cols, intr, 255)
    o.import_blocks(d["coords"], d["sdf"], d["w"])
    return g, o, coords, obs


def test_pose_loss_and_gradient_are_bit_reproducible():
    """The CTAs' loss and pose-gradient values are added exactly in fixed
    point: repeated evaluations return the same bits."""
    g, o, d, P, depth, dev = setup()
    T = se3_exp([0.004, -0.003, 0.002, 0.006, -0.004, 0.003]) @ P[7]
    runs = [raycast_loss_grad(g, T, dev[7]) for _ in range(3)]
    for L, grad, nv in runs[1:]:
        assert L == runs[0][0] and np.array_equal(grad, runs[0][1]) and nv == runs[0][2]


@pytest.mark.parametrize("storage,tol", [("f32", 0.01), ("f16", 0.01)])
def test_adjoint_matches_fp64_finite_differences(storage, tol):
    """GPU pose and voxel gradients against FP64 central differences (h = 1e-4
    on the pose twist, 1e-3 of the truncation on a voxel's TSDF value) on a
    smooth analytic wall where every pixel stays in the loss."""
    g, o, coords, obs = wall_grid(storage)
    dev = torch.from_numpy(obs.view(np.int16)).cuda()
    T = se3_exp([0.004, -0.003, 0.002, 0.006, -0.004, 0.003])
    gv = torch.zeros((g.params.hash_buckets, 512), dtype=torch.float32, device="cuda")
    L, grad, nv = raycast_loss_grad(g, T, dev, grad_voxels=gv)
    assert nv == obs.size
    h = 1e-4
    fd = np.zeros(6)
    for i in range(6):
        e = np.zeros(6)
        e[i] = h
        fd[i] = (o.raycast_loss(se3_exp(e) @ T, obs)[0] - o.raycast_loss(se3_exp(-e) @ T, obs)[0]) / (2 * h)
    print(storage, "pose grad gpu", grad, "\n              fd ", fd)
    assert np.abs(grad - fd).max() <= tol * np.abs(fd).max()
    # every voxel: GPU scatter against the FP64 adjoint (blocks matched by coordinates)
    gvn = gv.cpu().numpy()
    _, _, gv64 = o.raycast_loss_grad(T, obs, voxels=True)
    ex64 = o.export()
    row64 = {tuple(c): q for q, c in enumerate(ex64["coords"].tolist())}
    exp = g.export_blocks(with_color=False)
    buckets = g.export_buckets()
    gpu_rows = np.stack([gvn[int(b)] for b in buckets])
    fp64_rows = np.stack([gv64[row64[tuple(c)]] for c in exp["coords"].tolist()])
    scale = np.abs(fp64_rows).max()
    print(storage, "voxel grads: max |gpu - fp64|", np.abs(gpu_rows - fp64_rows).max(), "of", scale)
    assert np.abs(gpu_rows - fp64_rows).max() <= tol * scale
    # and the largest ones against FP64 central differences (step 1e-3 of the truncation)
    q_of = {int(b): q for q, b in enumerate(buckets)}
    hv = 1e-3 * WTRUNC
    rel = []
    for f in np.argsort(-np.abs(gvn).ravel())[:8]:
        b, v = divmod(int(f), 512)
        c = exp["coords"][q_of[b]]
        assert o.add_voxel(c, v, hv)
        lp = o.raycast_loss(T, obs)[0]
        o.add_voxel(c, v, -2 * hv)
        lm = o.raycast_loss(T, obs)[0]
        o.add_voxel(c, v, hv)
        fdv = (lp - lm) / (2 * hv)
        print("voxel", b, v, "gpu", gvn[b, v], "fd", fdv)
        rel.append(abs(gvn[b, v] - fdv) / max(abs(fdv), 1e-12))
    assert np.median(rel) < tol and max(rel) < 4 * tol


def test_pose_adjoint_matches_fp64_differences_with_frozen_pixels():
    """Config 5's check on the fused FP16 room: FP64 central differences
    (h = 1e-4 on the pose twist) of the loss over a frozen pixel set against
    the GPU adjoint over the same pixels (ss_raycast_loss_grad_masked). The
    per-pixel loss is smooth only while its hit stays in one trilinear cell
    (the field's gradient, and so the normal term, changes across cell faces),
    so the set keeps the pixels that are valid at the pose and at all twelve
    perturbed poses, whose hit stays in the same cell in all of them, and whose
    second difference is small (no jump to another crossing)."""
    from superscanner_gb300.raydiff import raycast_loss_grad_masked
    g, o, d, P, depth, dev = setup("f16")
    T = se3_exp([0.004, -0.003, 0.002, 0.006, -0.004, 0.003]) @ P[7]
    h = 1e-4
    vl = float(np.float32(VL))
    jj, ii = np.meshgrid(np.arange(640), np.arange(480))

    def cells(Tm, t):
        dcx, dcy = (jj - INTR[2]) / INTR[0], (ii - (480 - INTR[3])) / INTR[1]
        dd = np.stack([Tm[r, 0] * dcx + Tm[r, 1] * dcy + Tm[r, 2] for r in range(3)], -1)
        with np.errstate(invalid="ignore"):
            return np.floor((Tm[:3, 3] + t[..., None] * dd) / vl - 0.5)

    base, t0 = o.raycast_loss_pixels(T, depth[7])
    frozen = np.isfinite(base)
    c0 = cells(T, t0)
    plus, minus = [], []
    for i in range(6):
        for sgn, out in ((1.0, plus), (-1.0, minus)):
            e = np.zeros(6)
            e[i] = sgn * h
            Te = se3_exp(e) @ T
            L, t = o.raycast_loss_pixels(Te, depth[7])
            frozen &= np.isfinite(L) & (cells(Te, t) == c0).all(-1)
            out.append(L)
    Lp, Lm = np.stack(plus), np.stack(minus)
    with np.errstate(invalid="ignore"):
        frozen &= (np.abs(Lp + Lm - 2 * base) <= 2e-6).all(0)
    assert frozen.sum() > 0.5 * np.isfinite(base).sum()
    fd = np.where(frozen, Lp - Lm, 0.0).sum(axis=(1, 2)) / (2 * h)
    L, grad, nv = raycast_loss_grad_masked(g, T, dev[7], torch.from_numpy(frozen.astype(np.uint8)).cuda())
    print("frozen pixels", int(frozen.sum()), "gpu valid among them", nv)
    print("pose grad gpu", grad, "\n      fp64 fd", fd)
    assert nv >= 0.995 * frozen.sum()
    assert np.abs(grad - fd).max() <= 0.02 * np.abs(fd).max()


def test_pose_refinement_through_the_adjoint():
    """Gradient-based refinement (BFGS on the adjoint's pose gradient) of
    starts perturbed by up to 3 deg / 4 cm reaches the ground truth pose."""
    from superscanner_gb300.raydiff import refine_pose
    sc = synth.Scene(2, 1234)
    P = sc.trajectory(40, 42)
    depth, _ = sc.render(P, 480, 640, INTR, noise=True, noise_seed=7, color=False)
    dev = [torch.from_numpy(np.ascontiguousarray(d.view(np.int16))).cuda() for d in depth]
    g = GPUVoxelGrid(int(1e9), TRUNC, VL, 480, 640, storage="f16", with_color=False, hash_buckets=1 << 18,
                     max_weight=255)
    g.setIntrinsic(*INTR)
    for k in range(40):
        g.integrate_fast(dev[k], P[k].astype(np.float32))
    rng = np.random.default_rng(3)
    for k in (12, 25, 37):
        ax = rng.normal(size=3)
        ax /= np.linalg.norm(ax)
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        T0 = P[k] @ se3_exp(np.concatenate([ax * np.deg2rad(rng.uniform(1.5, 3.0)), d * rng.uniform(0.02, 0.04)]))
        T, info = refine_pose(g, T0, dev[k])
        D = np.linalg.inv(P[k]) @ T
        t_mm = np.linalg.norm(D[:3, 3]) * 1e3
        r_deg = np.rad2deg(np.arccos(np.clip((np.trace(D[:3, :3]) - 1) / 2, -1, 1)))
        print(f"frame {k}: {info}, final {t_mm:.3f} mm {r_deg:.4f} deg")
        assert info["loss"] < info["loss0"]
        assert t_mm < 1.0 and r_deg < 0.05
    g.sync()
