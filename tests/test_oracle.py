"""CPU tests of the oracle: the restatement checked against the reference's
own known-answer test (exe/Test.cpp:117-181), against independent numpy
restatements, and against analytic scenes with known answers."""
import numpy as np
import pytest

import oracle
import synth

INTR = (525.0, 525.0, 319.5, 239.5)


def prime_hash(c):
    """getPrimeHash (GPUVoxelGrid.h:124-128): int32 wrap, sign-extended to u64."""
    c = np.asarray(c, np.int64)
    h = (73856093 * c[..., 0] + 19349669 * c[..., 1] + 83492791 * c[..., 2]) & 0xFFFFFFFF
    h = np.where(h >= 2**31, h - 2**32, h)
    return h.astype(np.int64).view(np.uint64)


def test_matrix_vector_like_reference_test():
    """exe/Test.cpp:117-181: 1000 random 4x4 x 4 products in [-5, 5] vs a
    higher-precision product, tolerance 5e-5."""
    rng = np.random.default_rng(0)
    for _ in range(1000):
        M = rng.uniform(-5, 5, (4, 4)).astype(np.float32)
        v = rng.uniform(-5, 5, 4).astype(np.float32)
        got = oracle.mat4_vec4(M, v)
        ref = M.astype(np.float64) @ v.astype(np.float64)
        assert np.abs(got - ref).max() <= 5e-5
        # and the restated order: rows dotted left to right in float32
        seq = np.zeros(4, np.float32)
        for r in range(4):
            acc = np.float32(M[r, 0] * v[0])
            for c in range(1, 4):
                acc = np.float32(acc + np.float32(M[r, c] * v[c]))
            seq[r] = acc
        assert np.array_equal(got, seq)


def _collect_numpy(depth, E, vl, trunc, intr=INTR, rmin=0.2):
    """Independent float32 numpy restatement of depthToPcd + vbCollectionTag's
    block range (GPUVoxelGrid.h:131-190,229-247,303-307; .cpp:475-489)."""
    f32 = np.float32
    fx, fy, cx, cy = map(f32, intr)
    rows, cols = depth.shape
    ci, cj = f32(rows) - cy, cx
    i, j = np.meshgrid(np.arange(rows, dtype=f32), np.arange(cols, dtype=f32), indexing="ij")
    d = depth.astype(f32) / f32(1000)
    p = np.stack([(j - cj) / fx * d, (i - ci) / fy * d, d], -1)
    m = p[..., 2] > f32(rmin)
    p = p[m]
    E = E.astype(f32)
    pt = np.stack([((p[:, 0] * E[r, 0] + p[:, 1] * E[r, 1]) + p[:, 2] * E[r, 2]) + E[r, 3] for r in range(3)], -1)
    vbl = f32(8) * f32(vl)
    t = f32(trunc)

    def rule(a):
        q = a / vbl
        return np.where(a >= 0, np.trunc(q), np.trunc(q - f32(1))).astype(np.int64)

    lo, hi = rule(pt - t), rule(pt + t)
    out = set()
    for a, b in zip(lo, hi):
        for x in range(a[0], b[0] + 1):
            for y in range(a[1], b[1] + 1):
                for z in range(a[2], b[2] + 1):
                    out.add((x, y, z))
    return out


def _pose(rx=0.0, ry=0.0, rz=0.0, t=(0, 0, 0)):
    cx, sx, cy, sy, cz, sz = np.cos(rx), np.sin(rx), np.cos(ry), np.sin(ry), np.cos(rz), np.sin(rz)
    Rx = np.array([[1, 0, 0], [0, cx, -sx], [0, sx, cx]])
    Ry = np.array([[cy, 0, sy], [0, 1, 0], [-sy, 0, cy]])
    Rz = np.array([[cz, -sz, 0], [sz, cz, 0], [0, 0, 1]])
    T = np.eye(4)
    T[:3, :3] = Rz @ Ry @ Rx
    T[:3, 3] = t
    return T


def test_block_allocation_matches_numpy_restatement():
    sc = synth.Scene(1, 1234)
    P = sc.trajectory(3, 42)
    depth, _ = sc.render(P[:1], rows=60, cols=80, intr=(65.625, 65.625, 39.5, 29.5))
    # shift the world so that blocks straddle negative coordinates
    E = P[0].copy()
    E[:3, 3] -= np.array([1.0, 1.0, 0.9])
    g = oracle.OracleGrid(0.005, 0.02, 60, 80, intr=(65.625, 65.625, 39.5, 29.5))
    g.integrate(depth[0], None, E.astype(np.float32), with_color=False)
    dump = g.export()
    got = {tuple(c) for c in dump["coords"].tolist()}
    want = _collect_numpy(depth[0], E, 0.005, 0.02, intr=(65.625, 65.625, 39.5, 29.5))
    assert got == want
    assert any(min(c) < 0 for c in got)
    assert np.array_equal(dump["keys"], np.sort(prime_hash(dump["coords"])))
    assert np.all(np.diff(dump["keys"].astype(np.float64)) > 0)


def test_negative_index_rule_is_not_floor():
    """A point exactly on a negative block boundary: (int)(a/len - 1) = -2 where floor gives -1."""
    vl, trunc = 0.005, 0.001
    vbl = np.float32(8 * vl)
    # one valid pixel at the image centre column/row whose world x lands on -vbl exactly
    rows, cols = 9, 9
    depth = np.zeros((rows, cols), np.uint16)
    # pixel (i, j) with j - cj = 0 and i - ci = 0 -> camera point (0, 0, d)
    intr = (100.0, 100.0, 4.0, 5.0)  # ci = rows - cy = 4, cj = 4
    depth[4, 4] = 1000
    E = np.eye(4, dtype=np.float32)
    E[0, 3] = -vbl  # world x = -vbl exactly
    g = oracle.OracleGrid(vl, trunc, rows, cols, intr=intr)
    g.integrate(depth, None, E, with_color=False)
    xs = sorted({c[0] for c in g.export()["coords"].tolist()})
    # pt.x -/+ trunc = -vbl -/+ 0.001 -> blocks from (int)((-0.041/0.04) - 1) = -2 to (int)((-0.039/0.04) - 1) = -1
    assert xs == [-2, -1]


def test_plane_tsdf_known_answer():
    """Fronto-parallel plane at Z with identity pose: a voxel of centre z within
    trunc of the plane gets sdf = Z - z after one integration (w = 1)."""
    rows, cols = 48, 64
    intr = (60.0, 60.0, 31.5, 23.5)
    Z = 1.0
    depth = np.full((rows, cols), int(Z * 1000), np.uint16)
    vl, trunc = 0.01, 0.04
    g = oracle.OracleGrid(vl, trunc, rows, cols, intr=intr)
    g.integrate(depth, None, np.eye(4, dtype=np.float32), with_color=False)
    d = g.export()
    assert len(d["keys"]) > 0
    vbl = 8 * vl
    k = np.arange(512)
    vz = (d["coords"][:, 2:3] * np.float32(vbl)).astype(np.float64) + ((k // 64) + 0.5) * vl
    hit = d["w"] > 0
    assert hit.any()
    assert np.all(d["w"][hit] == 1.0)
    np.testing.assert_allclose(d["sdf"][hit], (Z - vz)[hit], atol=1e-6)
    assert np.all(np.abs(d["sdf"][hit]) < trunc)


def test_deintegrate_undoes_integrate():
    sc = synth.Scene(1, 1234)
    P = sc.trajectory(40, 42)
    depth, rgb = sc.render(P[[0, 30]], rows=96, cols=128, intr=(105.0, 105.0, 63.5, 47.5))
    intr = (105.0, 105.0, 63.5, 47.5)
    a = oracle.OracleGrid(0.005, 0.02, 96, 128, intr=intr)
    b = oracle.OracleGrid(0.005, 0.02, 96, 128, intr=intr)
    a.integrate(depth[0], rgb[0], P[0].astype(np.float32))
    b.integrate(depth[0], rgb[0], P[0].astype(np.float32))
    b.integrate(depth[1], rgb[1], P[30].astype(np.float32))
    b.deintegrate(depth[1], rgb[1], P[30].astype(np.float32))
    da, db = a.export(), b.export()
    # b keeps the blocks allocated by frame 1 (allocation is not undone), a's blocks are a subset
    idx = np.searchsorted(db["keys"], da["keys"])
    assert np.array_equal(db["keys"][idx], da["keys"])
    np.testing.assert_array_equal(db["w"][idx], da["w"])
    np.testing.assert_allclose(db["sdf"][idx], da["sdf"], atol=2e-6)
    extra = np.setdiff1d(np.arange(len(db["keys"])), idx)
    assert np.all(db["w"][extra] == 0)
    empty_b = int((db["w"] == 0).all(axis=1).sum())
    assert b.clean() == empty_b
    assert b.count() == int((da["w"] != 0).any(axis=1).sum())


def test_raycast_plane_known_answer():
    rows, cols = 48, 64
    intr = (60.0, 60.0, 31.5, 23.5)
    depth = np.full((rows, cols), 1500, np.uint16)
    g = oracle.OracleGrid(0.01, 0.04, rows, cols, intr=intr)
    for _ in range(3):
        g.integrate(depth, None, np.eye(4, dtype=np.float32), with_color=False)
    pcd, _ = g.raycast(np.eye(4, dtype=np.float32))
    hit = pcd[..., 2] != 0
    assert hit.mean() > 0.95
    # nearest-voxel crossing of a plane at 1.5 m lands within one voxel
    assert np.abs(pcd[hit][:, 2] - 1.5).max() < 0.01


def test_normals_of_a_tilted_plane():
    rows, cols = 30, 40
    intr = (50.0, 50.0, 19.5, 14.5)
    fx, fy, cx, cy = intr
    ci, cj = rows - cy, cx
    i, j = np.meshgrid(np.arange(rows), np.arange(cols), indexing="ij")
    n = np.array([0.2, -0.1, -1.0])
    n /= np.linalg.norm(n)
    # plane n . p = -1.2: z = -1.2 / (n . ray)
    ray = np.stack([(j - cj) / fx, (i - ci) / fy, np.ones_like(i, float)], -1)
    z = -1.2 / (ray @ n)
    depth = np.round(z * 1000).astype(np.uint16)
    pcd = oracle.depth_to_pcd(depth, intr)
    nrm = oracle.normals(pcd)
    inner = nrm[2:-2, 2:-2].reshape(-1, 3)
    cos = np.abs(inner @ n)
    assert np.median(cos) > 0.999
    assert np.array_equal(nrm[0, 0], [0, 0, 1])


def test_svd3_matches_numpy():
    rng = np.random.default_rng(3)
    for _ in range(200):
        H = rng.normal(size=(3, 3))
        U, S, V = oracle.svd3(H)
        np.testing.assert_allclose(U @ np.diag(S) @ V.T, H, atol=1e-12)
        u, s, vt = np.linalg.svd(H)
        np.testing.assert_allclose(V @ U.T, vt.T @ u.T, atol=1e-10)


def _misalignment(T, Ttrue, depth, intr):
    pts = oracle.depth_to_pcd(depth, intr).reshape(-1, 3).astype(np.float64)
    pts = pts[pts[:, 2] > 0]
    d = pts @ (T[:3, :3] - Ttrue[:3, :3]).T + (T[:3, 3] - Ttrue[:3, 3])
    return float(np.sqrt((d ** 2).sum(1).mean()))


def test_kokkos_icp_identity_and_known_motion():
    """kokkosICP (kokkosICP.cpp:25-210) on two rendered frames: identity on
    equal inputs; a known camera motion is mostly recovered (the reference's
    projective 10x10-window association converges over its 10 iterations, it
    does not reach the exact motion) and the RMSE falls monotonically."""
    sc = synth.Scene(1, 1234)
    P = sc.trajectory(40, 42)
    rows, cols = 120, 160
    intr = (131.25, 131.25, 79.5, 59.5)
    depth, _ = sc.render(P[[10, 12]], rows=rows, cols=cols, intr=intr)
    T, rmse, _ = oracle.kokkos_icp(depth[0], depth[0], P[10], P[10], 0, intr)
    np.testing.assert_allclose(T, np.eye(4), atol=1e-5)
    true = np.linalg.inv(P[12]) @ P[10]
    before = _misalignment(np.eye(4), true, depth[0], intr)
    for kind in (0, 1):
        T, rmse, stats = oracle.kokkos_icp(depth[0], depth[1], P[10], P[10], kind, intr)
        assert _misalignment(T, true, depth[0], intr) < 0.6 * before
        assert np.all(np.diff(stats[:5, 1]) < 0)
        assert rmse == pytest.approx(stats[:, 1].min())


def test_aliased_keys_share_one_entry():
    """Two blocks whose prime hashes collide alias one entry (GPUVoxelGrid.cpp:493-502);
    canonical coordinates: the larger packed coordinate word of the call."""
    # a collision vector within the packable range: 73856093 dx + 19349669 dy + 83492791 dz = 0 mod 2^32
    d = np.array(_collision_vector())
    assert prime_hash(d) == 0
    rows, cols = 8, 8
    intr = (100.0, 100.0, 4.0, 4.0)  # ci = 4, cj = 4
    vl, trunc = 0.01, 0.002
    vbl = 8 * vl
    depth = np.zeros((rows, cols), np.uint16)
    depth[4, 4] = 1000  # camera point (0, 0, 1)
    g = oracle.OracleGrid(vl, trunc, rows, cols, intr=intr)
    base = np.array([3, 2, 1])
    for blk in (base, base + d):
        E = np.eye(4, dtype=np.float32)
        # put the point at the centre of block blk
        E[:3, 3] = ((blk + 0.5) * vbl - np.array([0, 0, 1.0])).astype(np.float32)
        g.integrate(depth, None, E, with_color=False)
    dump = g.export()
    assert len(dump["keys"]) == 1
    assert tuple(dump["coords"][0]) == tuple(base + d)


def _collision_vector():
    a, b, c = 73856093, 19349669, 83492791
    inv_a = pow(a, -1, 2**32)
    for dz in range(0, 400):
        for dy in range(-400, 400):
            dx = (-(b * dy + c * dz) * inv_a) % 2**32
            if dx >= 2**31:
                dx -= 2**32
            if abs(dx) < 4000 and (dx, dy, dz) != (0, 0, 0):
                return int(dx), int(dy), int(dz)
    raise AssertionError("no collision vector found")


def test_fp64_raycast_adjoint_matches_finite_differences():
    """The FP64 restatement of the raycast adjoint (implicit differentiation of
    the trilinear zero crossing) against central differences of the FP64 loss
    on a smooth analytic wall: h = 1e-4 on the pose twist, 1e-3 of the
    truncation on a voxel's TSDF value (a step of 1 mm would move hit points
    across cell faces, where a voxel's weight stops, and bias the differences)."""
    from scenes import wavy_wall, VL, TRUNC
    from superscanner_gb300.raydiff import se3_exp
    coords, sdf, w, obs, intr = wavy_wall()
    o = oracle.MethodGrid64(VL, TRUNC, obs.shape[0], obs.shape[1], intr, 255)
    o.import_blocks(coords, sdf, w)
    T = se3_exp([0.004, -0.003, 0.002, 0.006, -0.004, 0.003])
    for lam, tol in ((0.0, 1e-4), (1.0, 5e-3)):
        L, grad = o.raycast_loss_grad(T, obs, lambda_n=lam)
        L2, nv = o.raycast_loss(T, obs, lambda_n=lam)
        assert nv == obs.size and abs(L - L2) <= 1e-12 * L2
        fd = np.zeros(6)
        for i in range(6):
            e = np.zeros(6)
            e[i] = 1e-4
            fd[i] = (o.raycast_loss(se3_exp(e) @ T, obs, lambda_n=lam)[0]
                     - o.raycast_loss(se3_exp(-e) @ T, obs, lambda_n=lam)[0]) / 2e-4
        assert np.abs(grad - fd).max() <= tol * np.abs(fd).max(), (lam, grad, fd)
    _, _, gv = o.raycast_loss_grad(T, obs, voxels=True)
    ex = o.export()
    picks = np.concatenate([np.argsort(-np.abs(gv).ravel())[:6],
                            np.random.default_rng(0).choice(np.flatnonzero(gv.ravel()), 6, replace=False)])
    hv = 1e-3 * TRUNC
    for f in picks:
        q, v = divmod(int(f), 512)
        c = ex["coords"][q]
        o.add_voxel(c, v, hv)
        lp = o.raycast_loss(T, obs)[0]
        o.add_voxel(c, v, -2 * hv)
        lm = o.raycast_loss(T, obs)[0]
        o.add_voxel(c, v, hv)
        fdv = (lp - lm) / (2 * hv)
        assert abs(gv[q, v] - fdv) <= 2e-3 * abs(fdv), (q, v, gv[q, v], fdv)
