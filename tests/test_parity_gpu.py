"""GPU parity of the reference-semantics path against the oracle: block
allocation and hash-table contents bit-exact, TSDF within 1e-3 of the
truncation distance (in practice bit-exact), raycast points bit-exact on
>= 99.9 % of pixels, kokkosICP poses within 1e-4 rad / 0.1 mm."""
import numpy as np
import pytest
import torch

import oracle
import synth
from superscanner_gb300 import GPUVoxelGrid, depth_to_pcd, kokkos_icp, normals_from_pcd
from superscanner_gb300._native import SS_ERR_ARG, SS_ERR_STATE, SS_ERR_TABLE_FULL, SSError

pytestmark = pytest.mark.gpu

INTR = (525.0, 525.0, 319.5, 239.5)
TSDF_TOL = 1e-3  # fraction of the truncation distance


def scaled_intr(rows, cols):
    s = cols / 640.0
    return (525.0 * s, 525.0 * s, (cols - 1) / 2.0, (rows - 1) / 2.0)


def frames(kind=1, n=4, rows=480, cols=640, step=3, noise=False, seed=1234, color=True):
    sc = synth.Scene(kind, seed)
    P = sc.trajectory(n * step, 42)[::step]
    intr = INTR if (rows, cols) == (480, 640) else scaled_intr(rows, cols)
    depth, rgb = sc.render(P, rows, cols, intr, noise=noise, color=color)
    return P, depth, rgb, intr


def dev(a):
    if a.dtype == np.uint16:
        a = a.view(np.int16)
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def make_pair(rows, cols, intr, vl=0.005, trunc=0.02, buckets=1 << 16, storage="f32", color=True, max_weight=0.0):
    g = GPUVoxelGrid(int(1e8), trunc, vl, rows, cols, storage=storage, with_color=color, hash_buckets=buckets,
                     max_weight=max_weight)
    g.setIntrinsic(*intr)
    o = oracle.OracleGrid(vl, trunc, rows, cols, intr=intr, max_weight=max_weight)
    return g, o


def compare(g, o, trunc, color=True):
    gd, od = g.export_blocks(with_color=color), o.export()
    assert len(gd["keys"]) == len(od["keys"]) == o.count() == g.block_count()
    assert np.array_equal(gd["keys"], od["keys"]), "hash-table keys differ"
    assert np.array_equal(gd["coords"], od["coords"]), "block coordinates differ"
    assert np.array_equal(gd["w"], od["w"]), "weights differ"
    diff = np.abs(gd["sdf"].astype(np.float64) - od["sdf"])
    assert diff.max() <= TSDF_TOL * trunc
    if color:
        assert np.abs(gd["rgb"] - od["rgb"]).max() <= 1e-3
    return float((gd["sdf"] == od["sdf"]).mean())


@pytest.mark.parametrize("color", [True, False])
def test_integrate_matches_oracle(color):
    P, depth, rgb, intr = frames(n=4)
    g, o = make_pair(480, 640, intr, color=color)
    for k in range(len(P)):
        E = P[k].astype(np.float32)
        g.integrate(dev(rgb[k]), dev(depth[k]), E, withColor=color)
        o.integrate(depth[k], rgb[k], E, with_color=color)
    g.sync()
    exact = compare(g, o, 0.02, color)
    assert exact == 1.0


def test_deintegrate_matches_oracle():
    P, depth, rgb, intr = frames(n=4, noise=True)
    g, o = make_pair(480, 640, intr)
    for k in range(4):
        E = P[k].astype(np.float32)
        g.integrate(dev(rgb[k]), dev(depth[k]), E)
        o.integrate(depth[k], rgb[k], E)
    for k in (1, 2):
        E = P[k].astype(np.float32)
        g.deIntegrate(dev(rgb[k]), dev(depth[k]), E)
        o.deintegrate(depth[k], rgb[k], E)
    g.sync()
    assert compare(g, o, 0.02) == 1.0
    g.cleanMemory()
    n_clean = o.clean()
    g.sync()
    assert n_clean >= 0
    assert compare(g, o, 0.02) == 1.0


def test_raycast_matches_oracle():
    P, depth, rgb, intr = frames(n=4, noise=True)
    g, o = make_pair(480, 640, intr)
    for k in range(4):
        E = P[k].astype(np.float32)
        g.integrate(dev(rgb[k]), dev(depth[k]), E)
        o.integrate(depth[k], rgb[k], E)
    for pose in (P[3], P[1]):
        E = pose.astype(np.float32)
        pcd, col = g.raycast(E)
        gp, gc = pcd.cpu().numpy(), col.cpu().numpy()
        g.sync()
        op, oc = o.raycast(E)
        same = np.all(gp == op, axis=-1)
        assert same.mean() >= 0.999, same.mean()
        hit_g, hit_o = gp[..., 2] != 0, op[..., 2] != 0
        assert (hit_g == hit_o).mean() >= 0.999
        assert hit_o.mean() > 0.9
        both = hit_g & hit_o
        assert np.abs(gc[both] - oc[both]).max() <= 1e-6


def test_pcd_and_normals_match_oracle():
    _, depth, _, intr = frames(n=1, noise=True)
    d = dev(depth[0])
    pcd = depth_to_pcd(d, *intr)
    nrm = normals_from_pcd(pcd)
    torch.cuda.synchronize()
    opcd = oracle.depth_to_pcd(depth[0], intr)
    assert np.array_equal(pcd.cpu().numpy(), opcd)
    assert np.array_equal(nrm.cpu().numpy(), oracle.normals(opcd))


@pytest.mark.parametrize("kind", [0, 1])
def test_kokkos_icp_matches_oracle(kind):
    sc = synth.Scene(1, 1234)
    P = sc.trajectory(40, 42)
    depth, _ = sc.render(P[[10, 12]], 480, 640, INTR, noise=True, color=False)
    T, rmse = kokkos_icp(dev(depth[0]), dev(depth[1]), P[10], P[10], kind, INTR)
    To, rmse_o, _ = oracle.kokkos_icp(depth[0], depth[1], P[10], P[10], kind, INTR)
    dR = T[:3, :3] @ To[:3, :3].T
    ang = np.arccos(np.clip((np.trace(dR) - 1) / 2, -1, 1))
    assert ang < 1e-4
    assert np.abs(T[:3, 3] - To[:3, 3]).max() < 1e-4
    assert rmse == pytest.approx(rmse_o, rel=1e-3)


def test_kokkos_icp_is_bit_reproducible():
    """The CTAs' totals are added exactly in fixed point, so the result does
    not depend on the order in which the CTAs finish: repeated calls, and the
    allocation-free entry point, return the same bits."""
    import ctypes as C
    from superscanner_gb300._native import f64x16, lib
    sc = synth.Scene(1, 1234)
    P = sc.trajectory(40, 42)
    depth, _ = sc.render(P[[10, 13]], 480, 640, INTR, noise=True, color=False)
    a, b = dev(depth[0]), dev(depth[1])
    stream = torch.cuda.current_stream().cuda_stream

    def call(fn):
        out = (C.c_double * 16)()
        rmse = C.c_float()
        st = fn(C.c_void_p(a.data_ptr()), C.c_void_p(b.data_ptr()), 480, 640, *INTR, f64x16(P[10]), f64x16(P[13]), 1,
                out, C.byref(rmse), C.c_void_p(stream))
        assert st == 0, st
        return np.array(out[:]), rmse.value

    runs = [call(lib.ss_kokkos_icp) for _ in range(3)] + [call(lib.ss_kokkos_icp_noalloc)]
    for T, r in runs[1:]:
        assert np.array_equal(T, runs[0][0]) and r == runs[0][1]


def test_ragged_image_and_empty_frame():
    rows, cols = 97, 131
    P, depth, rgb, intr = frames(n=3, rows=rows, cols=cols)
    g, o = make_pair(rows, cols, intr)
    for k in range(3):
        E = P[k].astype(np.float32)
        g.integrate(dev(rgb[k]), dev(depth[k]), E)
        o.integrate(depth[k], rgb[k], E)
    g.sync()
    assert compare(g, o, 0.02) == 1.0
    pcd, _ = g.raycast(P[2].astype(np.float32))
    op, _ = o.raycast(P[2].astype(np.float32))
    assert (np.all(pcd.cpu().numpy() == op, axis=-1)).mean() >= 0.999
    # an all-invalid frame allocates nothing and the raycast of an empty grid misses everywhere
    e, _ = make_pair(rows, cols, intr)
    zero = np.zeros((rows, cols), np.uint16)
    e.integrate(dev(np.zeros((rows, cols, 3), np.uint8)), dev(zero), P[0].astype(np.float32))
    e.sync()
    assert e.block_count() == 0
    pcd, col = e.raycast(P[0].astype(np.float32))
    assert float(pcd.abs().max()) == 0.0 and float(col.abs().max()) == 0.0


def test_table_full_is_reported_and_grid_stays_usable():
    P, depth, rgb, intr = frames(n=1)
    g, _ = make_pair(480, 640, intr, buckets=64)
    g.integrate(dev(rgb[0]), dev(depth[0]), P[0].astype(np.float32))
    with pytest.raises(SSError) as ei:
        g.sync()
    assert ei.value.code == SS_ERR_TABLE_FULL
    assert g.block_count() == 64
    g.reset()
    small = np.zeros_like(depth[0])
    small[200:204, 300:304] = depth[0][200:204, 300:304]
    g.integrate(dev(rgb[0]), dev(small), P[0].astype(np.float32))
    g.sync()
    assert 0 < g.block_count() <= 64


def test_call_order_and_pose_validation():
    P, depth, rgb, intr = frames(n=1)
    g = GPUVoxelGrid(int(1e8), 0.02, 0.005, 480, 640, hash_buckets=1 << 12)
    with pytest.raises(SSError) as ei:
        g.integrate(dev(rgb[0]), dev(depth[0]), P[0].astype(np.float32))
    assert ei.value.code == SS_ERR_STATE
    g.setIntrinsic(*intr)
    bad = P[0].astype(np.float32)
    bad[0, 3] = np.nan
    with pytest.raises(SSError) as ei:
        g.integrate(dev(rgb[0]), dev(depth[0]), bad)
    assert ei.value.code == SS_ERR_ARG
    with pytest.raises(ValueError):
        g.integrate(dev(rgb[0]), dev(depth[0][:100]), P[0].astype(np.float32))


def test_weight_cap_matches_oracle():
    P, depth, rgb, intr = frames(n=4, noise=True)
    g, o = make_pair(480, 640, intr, max_weight=2.0)
    for k in range(4):
        E = P[k].astype(np.float32)
        g.integrate(dev(rgb[k]), dev(depth[k]), E)
        o.integrate(depth[k], rgb[k], E)
    g.sync()
    assert compare(g, o, 0.02) == 1.0
    assert g.export_blocks()["w"].max() == 2.0


def test_export_import_roundtrip():
    P, depth, rgb, intr = frames(n=2)
    g, o = make_pair(480, 640, intr)
    for k in range(2):
        g.integrate(dev(rgb[k]), dev(depth[k]), P[k].astype(np.float32))
    d = g.export_blocks()
    h, _ = make_pair(480, 640, intr)
    h.import_blocks(d["coords"], d["sdf"], d["w"], d["rgb"])
    e = h.export_blocks()
    for k in ("keys", "coords", "sdf", "w", "rgb"):
        assert np.array_equal(d[k], e[k]), k
    o.import_blocks(d["coords"], d["sdf"], d["w"], d["rgb"])
    pose = P[1].astype(np.float32)
    assert (np.all(h.raycast(pose)[0].cpu().numpy() == o.raycast(pose)[0], axis=-1)).mean() >= 0.999


def test_aliased_blocks_match_oracle():
    from test_oracle import _collision_vector
    d = np.array(_collision_vector())
    rows, cols, intr = 8, 8, (100.0, 100.0, 4.0, 4.0)
    vl, trunc = 0.01, 0.002
    depth = np.zeros((rows, cols), np.uint16)
    depth[4, 4] = 1000
    g, o = make_pair(rows, cols, intr, vl=vl, trunc=trunc, buckets=1 << 10, color=False)
    base = np.array([3, 2, 1])
    for blk in (base + d, base):
        E = np.eye(4, dtype=np.float32)
        E[:3, 3] = ((blk + 0.5) * 8 * vl - np.array([0, 0, 1.0])).astype(np.float32)
        g.integrate(None, dev(depth), E, withColor=False)
        o.integrate(depth, None, E, with_color=False)
    g.sync()
    compare(g, o, trunc, color=False)
    assert g.block_count() == 1


def test_f16_storage_tracks_f32():
    P, depth, rgb, intr = frames(n=6, noise=True)
    a, _ = make_pair(480, 640, intr, storage="f32", color=False)
    b, _ = make_pair(480, 640, intr, storage="f16", color=False)
    for k in range(6):
        E = P[k].astype(np.float32)
        a.integrate(None, dev(depth[k]), E, withColor=False)
        b.integrate(None, dev(depth[k]), E, withColor=False)
    a.sync()
    b.sync()
    da, db = a.export_blocks(with_color=False), b.export_blocks(with_color=False)
    assert np.array_equal(da["keys"], db["keys"])
    assert np.array_equal(da["w"], db["w"])
    assert np.abs(da["sdf"] - db["sdf"]).max() <= 1e-3 * 0.02


def test_scattered_and_far_depths_match_oracle():
    """Block collection off its common path: random depths from 0.4 m to 40 m
    per pixel (blocks beyond the tile set's +-20 m key range take the direct
    global path; tiles meet more distinct blocks than their set holds), on a
    ragged image. Block set, coordinates, weights and TSDF as the oracle."""
    rows, cols = 61, 93
    intr = scaled_intr(rows, cols)
    rng = np.random.default_rng(3)
    depth = rng.integers(400, 40000, size=(2, rows, cols)).astype(np.uint16)
    depth[1, :, : cols // 2] = 0  # a frame with a blank half
    P = [np.eye(4), np.eye(4)]
    P[1][:3, 3] = [0.3, -0.2, 0.1]
    g, o = make_pair(rows, cols, intr, buckets=1 << 18, color=False)
    for k in range(2):
        E = P[k].astype(np.float32)
        g.integrate(None, dev(depth[k]), E, withColor=False)
        o.integrate(depth[k], np.zeros((rows, cols, 3), np.uint8), E, with_color=False)
    g.sync()
    assert g.block_count() > 20000
    assert compare(g, o, 0.02, color=False) == 1.0


@pytest.mark.parametrize("rows", [1, 2, 3, 4, 7, 8])
def test_collection_tile_rows_match_oracle(rows):
    """Block collection with every tile height the launch configuration
    allows (set size 128 slots per row, one warp per row, power of two or
    not): block set, coordinates and TSDF as the oracle."""
    P, depth, rgb, intr = frames(n=3)
    g, o = make_pair(480, 640, intr, color=False)
    g.set_launch_config(collect_rows=rows)
    for k in range(len(P)):
        E = P[k].astype(np.float32)
        g.integrate(None, dev(depth[k]), E, withColor=False)
        o.integrate(depth[k], rgb[k], E, with_color=False)
    g.sync()
    assert compare(g, o, 0.02, color=False) == 1.0


def test_fixed48_sums_are_exact():
    """The fixed-point cross-CTA sums (kokkosICP, differentiable raycast):
    the total of each value truncated to a multiple of 2^-48, over values
    spread across 60 binary orders of magnitude and both signs, is exact, its
    double is the nearest one, and the float pair is (RN(total), RN(rest))."""
    import ctypes as C
    from fractions import Fraction
    from superscanner_gb300._native import SS_ERR_ARG, lib
    rng = np.random.default_rng(11)
    v = (rng.standard_normal(200000) * np.exp2(rng.integers(-40, 20, 200000))).astype(np.float32)
    v[:5] = [0.0, -0.0, 3.0e-30, 1.0e13, -1.0e13]
    dv = torch.from_numpy(v).cuda()
    out = (C.c_double * 3)()
    assert lib.ss_test_fixed48_sum(C.c_void_p(dv.data_ptr()), len(v), out, None) == 0
    unit = Fraction(1, 2 ** 48)
    exact = sum((Fraction(float(x)) / unit).__trunc__() for x in v) * unit
    assert out[0] == float(exact)  # the nearest double
    h, l = out[1], out[2]
    assert h == float(np.float32(float(exact))) or abs(Fraction(h) - exact) <= abs(Fraction(float(np.float32(float(exact)))) - exact)
    assert abs(Fraction(h) + Fraction(l) - exact) <= abs(exact) * Fraction(1, 2 ** 46) + unit
    big = torch.tensor([1.0, 2.0 ** 47], dtype=torch.float32, device="cuda")
    assert lib.ss_test_fixed48_sum(C.c_void_p(big.data_ptr()), 2, out, None) == SS_ERR_ARG
