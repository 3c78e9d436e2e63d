// ss_raycast.cu — reference-semantics raycast (raycastingTag,
// src/VoxelGrid/GPUVoxelGrid.cpp:561-715) and its C-ABI entry point.
//
// One thread per pixel, 32x8 pixel tiles (a warp marches 32 neighbouring rays
// of one row, which stay coherent through the block-skip loop). The unit ray
// table normPcd (createNormPcdTag, :717-722) is recomputed in registers
// instead of being read from a 3.7 MB image.
#include <climits>

#include "ss_grid_impl.cuh"

namespace ss {

constexpr int kRaycastIterCap = 1 << 20;  // far above the d_max / min-stride bound

struct VoxelRead {
    float sdf, w;
};

template <int kStorage>
__device__ __forceinline__ VoxelRead read_voxel(const GridView &g, int bucket, int v) {
    const size_t vi = (size_t)bucket * kBlockVoxels + v;
    if (kStorage == SS_STORAGE_F32) {
        const float2 sw = __ldg(g.vox32 + vi);
        return {sw.x, sw.y};
    } else {
        const uint32_t word = __ldg(g.vox16 + vi);
        return {__half2float(__ushort_as_half((unsigned short)(word & 0xffffu))) * g.trunc, (float)(word >> 16)};
    }
}

__device__ __forceinline__ void block_of(const GridView &g, F3 p, int &bx, int &by, int &bz) {
    bx = idx_rule(p.x, g.vbl);
    by = idx_rule(p.y, g.vbl);
    bz = idx_rule(p.z, g.vbl);
}

// getVinVBIndeces (GPUVoxelGrid.h:192-221): p - vbl * vbInd, then the index rule.
__device__ __forceinline__ int voxel_in_block(const GridView &g, F3 p, int bx, int by, int bz) {
    const F3 q = f3sub(p, F3{__fmul_rn(g.vbl, (float)bx), __fmul_rn(g.vbl, (float)by), __fmul_rn(g.vbl, (float)bz)});
    const int vx = idx_rule(q.x, g.vl), vy = idx_rule(q.y, g.vl), vz = idx_rule(q.z, g.vl);
    return vx + kEdge * vy + kEdge * kEdge * vz;
}

// getVoxelMidPoint (GPUVoxelGrid.h:274-278): vb*vbl (float) + (v + 0.5)*vl
// (double), rounded to float; the double sum is exact, so one fmaf matches.
__device__ __forceinline__ F3 voxel_mid(const GridView &g, int v, int bx, int by, int bz) {
    const int vx = v & 7, vy = (v >> 3) & 7, vz = v >> 6;
    return {__fmaf_rn((float)vx + 0.5f, g.vl, __fmul_rn((float)bx, g.vbl)),
            __fmaf_rn((float)vy + 0.5f, g.vl, __fmul_rn((float)by, g.vbl)),
            __fmaf_rn((float)vz + 0.5f, g.vl, __fmul_rn((float)bz, g.vbl))};
}

__device__ __forceinline__ int find_block(const GridView &g, int bx, int by, int bz) {
    return table_find(g, prime_hash(bx, by, bz));
}

template <int kStorage>
__global__ void __launch_bounds__(256) raycast_ref_kernel(GridView g, Mat34 Er, float *__restrict__ out_pcd,
                                                          float *__restrict__ out_col) {
    const int j = blockIdx.x * 32 + threadIdx.x;
    const int i = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= g.resi || j >= g.resj) return;
    const float vl = g.vl, vbl = g.vbl, dtr = g.trunc, dmax = g.d_max;

    const F3 np = f3normalized(get_point(g.in, i, j, 1.0f));
    F3 rv = xform(Er, np);
    const F3 dir = f3sub(rv, F3{Er.m[3], Er.m[7], Er.m[11]});
    float l = 0.1f;
    rv = f3sub(rv, f3smul(__fsub_rn(1.f, l), dir));

    bool done = false, Fn = false, Lp = false;
    int guard = 0;
    F3 hit{0.f, 0.f, 0.f};
    float cr = 0.f, cg = 0.f, cb = 0.f;

    while (!done && !Fn && l < dmax) {
        int bx, by, bz;
        block_of(g, rv, bx, by, bz);
        int bucket = find_block(g, bx, by, bz);
        int count = 0;
        while (bucket < 0 && l < dmax && guard < kRaycastIterCap) {
            rv = f3add(rv, f3smul(vbl, dir));
            l = __fadd_rn(l, vbl);
            block_of(g, rv, bx, by, bz);
            bucket = find_block(g, bx, by, bz);
            count++;
            guard++;
        }
        if (l >= dmax) break;
        if (count > 0) {
            const float back = __fsub_rn(vbl, dtr);
            rv = f3sub(rv, f3smul(back, dir));
            l = __fsub_rn(l, back);
            block_of(g, rv, bx, by, bz);
            bucket = find_block(g, bx, by, bz);
            while (bucket < 0 && l < dmax && guard < kRaycastIterCap) {
                rv = f3add(rv, f3smul(dtr, dir));
                l = __fadd_rn(l, dtr);
                block_of(g, rv, bx, by, bz);
                bucket = find_block(g, bx, by, bz);
                guard++;
            }
        }
        if (l >= dmax) break;
        if (guard >= kRaycastIterCap) break;
        // vb = value_at(index); oldvbInd = vbInd (GPUVoxelGrid.cpp:633-635)
        const int cur = bucket;
        const int ox = bx, oy = by, oz = bz;
        int v = voxel_in_block(g, rv, bx, by, bz);
        while (!done && l < dmax && ox == bx && oy == by && oz == bz && !Fn) {
            if (++guard >= kRaycastIterCap) break;
            const VoxelRead cv = read_voxel<kStorage>(g, cur, v);
            if (cv.w > 0) {
                if (cv.sdf > 0) {
                    Lp = true;
                    rv = f3add(rv, f3smul(vl, dir));
                    l = __fadd_rn(l, vl);
                    block_of(g, rv, bx, by, bz);
                    v = voxel_in_block(g, rv, bx, by, bz);
                } else if (Lp) {
                    done = true;  // zero crossing (GPUVoxelGrid.cpp:655-689)
                    const F3 vm_in = voxel_mid(g, v, bx, by, bz);
                    rv = f3sub(rv, f3smul(vl, dir));
                    l = __fsub_rn(l, vl);
                    int qx, qy, qz;
                    block_of(g, rv, qx, qy, qz);
                    const int vo = voxel_in_block(g, rv, qx, qy, qz);
                    const F3 vm_out = voxel_mid(g, vo, qx, qy, qz);
                    const int ob = (qx == ox && qy == oy && qz == oz) ? cur : find_block(g, qx, qy, qz);
                    VoxelRead o{0.f, 0.f};
                    float orr = 0.f, og = 0.f, obb = 0.f;
                    if (ob >= 0) {  // missing block: reads as an empty voxel (reference: value_at(invalid))
                        o = read_voxel<kStorage>(g, ob, vo);
                        if (out_col && g.rgb) {
                            const float *pl = g.rgb + (size_t)ob * 3 * kBlockVoxels + vo;
                            orr = pl[0];
                            og = pl[kBlockVoxels];
                            obb = pl[2 * kBlockVoxels];
                        }
                    }
                    // x = (w_o*sdf_o/vl + w_i*(1 - sdf_i/vl)) / (w_i + w_o)  (GPUVoxelGrid.cpp:678)
                    const float x = __fdiv_rn(
                        __fadd_rn(__fdiv_rn(__fmul_rn(o.w, o.sdf), vl), __fmul_rn(cv.w, __fsub_rn(1.f, __fdiv_rn(cv.sdf, vl)))),
                        __fadd_rn(cv.w, o.w));
                    const F3 p = f3add(vm_out, f3smul(x, f3sub(vm_in, vm_out)));
                    const float sproj = __fsub_rn(f3dot(p, dir), f3dot(rv, dir));
                    hit = f3add(rv, f3smul(sproj, dir));  // point on the ray (GPUVoxelGrid.cpp:681)
                    if (out_col && g.rgb) {
                        const float *pl = g.rgb + (size_t)cur * 3 * kBlockVoxels + v;
                        cr = (float)((0.5 * (double)orr + 0.5 * (double)pl[0]) / 255.0);
                        cg = (float)((0.5 * (double)og + 0.5 * (double)pl[kBlockVoxels]) / 255.0);
                        cb = (float)((0.5 * (double)obb + 0.5 * (double)pl[2 * kBlockVoxels]) / 255.0);
                    }
                } else {
                    Fn = true;
                }
            } else {
                Lp = false;
                rv = f3add(rv, f3smul(vl, dir));
                l = __fadd_rn(l, vl);
                block_of(g, rv, bx, by, bz);
                v = voxel_in_block(g, rv, bx, by, bz);
            }
        }
        if (guard >= kRaycastIterCap) break;
    }
    if (guard >= kRaycastIterCap) atomicOr(&g.ctr->status, kStTimeout);
    const size_t pix = (size_t)i * g.resj + j;
    if (!done) hit = F3{0.f, 0.f, 0.f};
    out_pcd[pix * 3 + 0] = hit.x;
    out_pcd[pix * 3 + 1] = hit.y;
    out_pcd[pix * 3 + 2] = hit.z;
    if (out_col) {
        out_col[pix * 3 + 0] = done ? cr : 0.f;
        out_col[pix * 3 + 1] = done ? cg : 0.f;
        out_col[pix * 3 + 2] = done ? cb : 0.f;
    }
}


// ------------------------------------------------------------------------
// Trilinear raycast (the per-frame pipeline's model view): depth, vertex and
// normal maps with at most max_steps march steps per ray.
//
// Ray of pixel (i, j): direction ((j - cj)/fx, (i - ci)/fy, 1) in the camera
// (not normalised, so the ray parameter t is the camera-frame depth). Steps:
//  * the ray point lies in a super-block (8^3 blocks) without any allocated
//    block: jump to the exit of that super-block's box;
//  * the ray point lies in a block that is not allocated: jump to the exit of
//    that block's box (empty-space skip);
//  * the trilinear TSDF sample is invalid (a corner voxel unobserved or in a
//    missing block): advance one voxel;
//  * the sample is positive: advance max(vl, 0.8 f) (f in metres);
//  * the sample is negative after a positive one: zero crossing; two
//    regula-falsi refinements on the bracket, then the hit;
//  * the sample is negative with no positive predecessor: no hit (back face).
// With a depth hint (the frame just fused at this pose, so the same rays), a
// ray whose pixel has depth d searches only [d - margin, d + margin]; a pixel
// without depth (dropout) starts at the smallest depth of its warp's 32-pixel
// row segment minus margin and marches on as usual. Where the fused frame saw
// d, a crossing outside that window contradicts the frame just fused (it
// shows up at silhouettes, through gaps of the thin band the trilinear
// validity test leaves there), so the window loses no consistent surface and
// keeps every lane of a warp within a few steps of the others.
// Every sample or skip counts as one step. The normal is the normalised
// gradient of the trilinear interpolant at the hit (world frame, pointing
// out of the surface). Outputs: vmap[i][j] = (x, y, z world, depth) and
// nmap[i][j] = (nx, ny, nz, 0); misses are all-zero.
struct TriSample {
    bool valid;
    float f;
    float gx, gy, gz;  // d f / d (world x, y, z)
};

struct BlockCache {
    int x, y, z, bucket;
    unsigned lookups;  // hash-table finds issued (cache misses)
    unsigned voxels;   // voxel words loaded
};

template <int kStorage>
__device__ __forceinline__ float2 voxel_sw(const GridView &g, int bucket, int v) {
    const size_t vi = (size_t)bucket * kBlockVoxels + v;
    if (kStorage == SS_STORAGE_F32) {
        return __ldg(g.vox32 + vi);
    } else {
        const uint32_t word = __ldg(g.vox16 + vi);
        return make_float2(__half2float(__ushort_as_half((unsigned short)(word & 0xffffu))) * g.trunc,
                           (float)(word >> 16));
    }
}

__device__ __forceinline__ int cached_lookup(const GridView &g, BlockCache &c, int bx, int by, int bz) {
    if (bx == c.x && by == c.y && bz == c.z) return c.bucket;
    c.x = bx;
    c.y = by;
    c.z = bz;
    c.lookups++;
    c.bucket = packable(bx, by, bz) ? table_find(g, prime_hash(bx, by, bz)) : -1;
    return c.bucket;
}

template <int kStorage, bool kGrad>
__device__ __forceinline__ TriSample trilinear(const GridView &g, float px, float py, float pz, float inv_vl,
                                               BlockCache &c) {
    TriSample r{false, 0.f, 0.f, 0.f, 0.f};
    const float ux = fmaf(px, inv_vl, -0.5f), uy = fmaf(py, inv_vl, -0.5f), uz = fmaf(pz, inv_vl, -0.5f);
    const float fx0 = floorf(ux), fy0 = floorf(uy), fz0 = floorf(uz);
    const int ix = (int)fx0, iy = (int)fy0, iz = (int)fz0;
    const float ax = ux - fx0, ay = uy - fy0, az = uz - fz0;
    float s[8];
    if ((ix & 7) != 7 && (iy & 7) != 7 && (iz & 7) != 7) {
        // all 8 corners in one block: one lookup, fixed offsets +1, +8, +64
        const int b = cached_lookup(g, c, ix >> 3, iy >> 3, iz >> 3);
        if (b < 0) return r;
        const int v0 = (ix & 7) + 8 * (iy & 7) + 64 * (iz & 7);
        float2 sw[8];
#pragma unroll
        for (int k = 0; k < 8; k++) sw[k] = voxel_sw<kStorage>(g, b, v0 + (k & 1) + 8 * ((k >> 1) & 1) + 64 * (k >> 2));
        c.voxels += 8;
        bool ok = true;
#pragma unroll
        for (int k = 0; k < 8; k++) {
            ok &= sw[k].y > 0.f;
            s[k] = sw[k].x;
        }
        if (!ok) return r;
    } else {
#pragma unroll
        for (int k = 0; k < 8; k++) {
            const int vx = ix + (k & 1), vy = iy + ((k >> 1) & 1), vz = iz + (k >> 2);
            const int bx = vx >> 3, by = vy >> 3, bz = vz >> 3;  // floor(v / 8)
            const int b = cached_lookup(g, c, bx, by, bz);
            if (b < 0) return r;
            const float2 sw = voxel_sw<kStorage>(g, b, (vx & 7) + 8 * (vy & 7) + 64 * (vz & 7));
            c.voxels++;
            if (!(sw.y > 0.f)) return r;
            s[k] = sw.x;
        }
    }
    // lerp along x, then y, then z
    const float s00 = fmaf(ax, s[1] - s[0], s[0]), s10 = fmaf(ax, s[3] - s[2], s[2]);
    const float s01 = fmaf(ax, s[5] - s[4], s[4]), s11 = fmaf(ax, s[7] - s[6], s[6]);
    const float s0 = fmaf(ay, s10 - s00, s00), s1 = fmaf(ay, s11 - s01, s01);
    r.valid = true;
    r.f = fmaf(az, s1 - s0, s0);
    if (kGrad) {
        const float dx00 = s[1] - s[0], dx10 = s[3] - s[2], dx01 = s[5] - s[4], dx11 = s[7] - s[6];
        const float dx0 = fmaf(ay, dx10 - dx00, dx00), dx1 = fmaf(ay, dx11 - dx01, dx01);
        r.gx = fmaf(az, dx1 - dx0, dx0) * inv_vl;
        r.gy = fmaf(az, s11 - s01 - (s10 - s00), s10 - s00) * inv_vl;
        r.gz = (s1 - s0) * inv_vl;
    }
    return r;
}

// One ray march from t0; returns true on a zero crossing (t = hit depth).
template <int kStorage>
__device__ __forceinline__ bool march(const GridView &g, float ox, float oy, float oz, float dx, float dy, float dz,
                                      float inv_len, float t0, float t_max, int max_steps, int &steps, float &t,
                                      BlockCache &cache) {
    const float vl = g.vl, inv_vl = 1.f / g.vl, inv_vbl = 1.f / g.vbl;
    const float rdx = 1.f / dx, rdy = 1.f / dy, rdz = 1.f / dz;
    const float sbl = g.vbl * (float)(1 << kSuperShift);
    t = t0;
    float t_prev = 0.f, f_prev = 0.f;
    bool prev_valid = false;
    int csx = INT_MIN, csy = INT_MIN, csz = INT_MIN;
    bool cocc = false;
    while (steps < max_steps && t < t_max) {
        const float px = fmaf(t, dx, ox), py = fmaf(t, dy, oy), pz = fmaf(t, dz, oz);
        const int bx = (int)floorf(px * inv_vbl), by = (int)floorf(py * inv_vbl), bz = (int)floorf(pz * inv_vbl);
        steps++;
        const int sx = bx >> kSuperShift, sy = by >> kSuperShift, sz = bz >> kSuperShift;
        if (sx != csx || sy != csy || sz != csz) {
            csx = sx;
            csy = sy;
            csz = sz;
            cocc = super_occupied(g, sx, sy, sz);
            cache.lookups++;
        }
        if (!cocc) {  // exit of this empty super-block's box along the ray
            const float ex = ((float)(sx + (dx > 0.f)) * sbl - ox) * rdx;
            const float ey = ((float)(sy + (dy > 0.f)) * sbl - oy) * rdy;
            const float ez = ((float)(sz + (dz > 0.f)) * sbl - oz) * rdz;
            const float te = fminf(fminf(dx != 0.f ? ex : INFINITY, dy != 0.f ? ey : INFINITY),
                                   dz != 0.f ? ez : INFINITY);
            t = fmaxf(te, t) + 1e-4f * vl * inv_len;
            prev_valid = false;
            continue;
        }
        if (cached_lookup(g, cache, bx, by, bz) < 0) {  // exit of this empty block's box
            const float ex = ((float)(bx + (dx > 0.f)) * g.vbl - ox) * rdx;
            const float ey = ((float)(by + (dy > 0.f)) * g.vbl - oy) * rdy;
            const float ez = ((float)(bz + (dz > 0.f)) * g.vbl - oz) * rdz;
            const float te = fminf(fminf(dx != 0.f ? ex : INFINITY, dy != 0.f ? ey : INFINITY),
                                   dz != 0.f ? ez : INFINITY);
            t = fmaxf(te, t) + 1e-4f * vl * inv_len;
            prev_valid = false;
            continue;
        }
        const TriSample sm = trilinear<kStorage, false>(g, px, py, pz, inv_vl, cache);
        if (!sm.valid) {
            prev_valid = false;
            t += vl * inv_len;
            continue;
        }
        if (sm.f < 0.f) {
            if (!(prev_valid && f_prev > 0.f)) return false;  // back face
            float ta = t_prev, fa = f_prev, tb = t, fb = sm.f;
            for (int r = 0; r < 2; r++) {
                const float tc = ta + (tb - ta) * fa / (fa - fb);
                const TriSample q = trilinear<kStorage, false>(g, fmaf(tc, dx, ox), fmaf(tc, dy, oy),
                                                               fmaf(tc, dz, oz), inv_vl, cache);
                if (!q.valid) break;
                if (q.f > 0.f) {
                    ta = tc;
                    fa = q.f;
                } else {
                    tb = tc;
                    fb = q.f;
                }
            }
            t = ta + (tb - ta) * fa / (fa - fb);
            return true;
        }
        prev_valid = true;
        t_prev = t;
        f_prev = sm.f;
        t += fmaxf(vl, 0.8f * sm.f) * inv_len;
    }
    return false;
}

template <int kStorage>
__global__ void __launch_bounds__(256) raycast_maps_kernel(GridView g, Mat34 T, const FramePose *__restrict__ pose,
                                                           int max_steps, float t_min, float t_max,
                                                           float4 *__restrict__ vmap, float4 *__restrict__ nmap,
                                                           unsigned long long *__restrict__ counters,
                                                           const uint16_t *__restrict__ hint, float hint_margin) {
    const int j = blockIdx.x * 32 + threadIdx.x;
    const int i = blockIdx.y * blockDim.y + threadIdx.y;
    const bool inside = i < g.resi && j < g.resj;
    BlockCache cache{INT_MIN, INT_MIN, INT_MIN, -1, 0u, 0u};
    int steps = 0;
    bool hit = false;
    // Depth hint of this ray: the fused frame's depth at this pixel, or, where
    // that is missing (dropout), the smallest depth of the 32 pixels of this
    // warp's row segment, so that no lane of the warp marches the whole ray.
    unsigned hint_mm = 0;
    if (hint) {
        const unsigned own = inside ? (unsigned)__ldg(hint + (size_t)i * g.resj + j) : 0u;
        const unsigned wmin = __reduce_min_sync(0xffffffffu, own ? own : 0xffffffffu);
        hint_mm = own ? own : (wmin != 0xffffffffu ? wmin : 0u);
    }
    if (inside) {
    if (pose) {
#pragma unroll
        for (int k = 0; k < 12; k++) T.m[k] = __ldg(&pose->E.m[k]);
    }
    const float dcx = ((float)j - g.in.cj) / g.in.fx, dcy = ((float)i - g.in.ci) / g.in.fy;
    const float dx = fmaf(T.m[0], dcx, fmaf(T.m[1], dcy, T.m[2]));
    const float dy = fmaf(T.m[4], dcx, fmaf(T.m[5], dcy, T.m[6]));
    const float dz = fmaf(T.m[8], dcx, fmaf(T.m[9], dcy, T.m[10]));
    const float ox = T.m[3], oy = T.m[7], oz = T.m[11];
    const float inv_len = rsqrtf(fmaf(dx, dx, fmaf(dy, dy, dz * dz)));  // world length of dt = 1
    const float inv_vl = 1.f / g.vl;

    float t = t_min;
    const float t_hint = (float)hint_mm * 1e-3f - hint_margin;
    if (hint && t_hint > t_min) {
        // a pixel with its own depth d searches [d - margin, d + margin]; a
        // dropout pixel starts at its warp's smallest depth and marches on
        const bool own = __ldg(hint + (size_t)i * g.resj + j) != 0;
        const float t_end = own ? fminf(t_max, t_hint + 2.f * hint_margin) : t_max;
        hit = march<kStorage>(g, ox, oy, oz, dx, dy, dz, inv_len, t_hint, t_end, max_steps, steps, t, cache);
    } else {
        hit = march<kStorage>(g, ox, oy, oz, dx, dy, dz, inv_len, t_min, t_max, max_steps, steps, t, cache);
    }
    const size_t pix = (size_t)i * g.resj + j;
    float4 v = make_float4(0.f, 0.f, 0.f, 0.f), n = make_float4(0.f, 0.f, 0.f, 0.f);
    if (hit) {
        const float px = fmaf(t, dx, ox), py = fmaf(t, dy, oy), pz = fmaf(t, dz, oz);
        const TriSample q = trilinear<kStorage, true>(g, px, py, pz, inv_vl, cache);
        const float gn = q.valid ? sqrtf(q.gx * q.gx + q.gy * q.gy + q.gz * q.gz) : 0.f;
        if (gn > 0.f) {
            v = make_float4(px, py, pz, t);
            n = make_float4(q.gx / gn, q.gy / gn, q.gz / gn, 0.f);
        }
    }
    vmap[pix] = v;
    nmap[pix] = n;
    }
    if (counters) {  // algorithmic-traffic counters (profiling only), one atomic per warp and field
        const unsigned full = 0xffffffffu;
        const unsigned l = __reduce_add_sync(full, cache.lookups), vx = __reduce_add_sync(full, cache.voxels);
        const unsigned st = __reduce_add_sync(full, (unsigned)steps), h = __reduce_add_sync(full, hit ? 1u : 0u);
        if ((threadIdx.x & 31) == 0) {
            atomicAdd(counters + 0, (unsigned long long)l);
            atomicAdd(counters + 1, (unsigned long long)vx);
            atomicAdd(counters + 2, (unsigned long long)st);
            atomicAdd(counters + 3, (unsigned long long)h);
        }
    }
}

ss_status launch_raycast_maps(ss_grid *g, const Mat34 &T, const FramePose *dpose, int max_steps, float t_min,
                              float t_max, float4 *vmap, float4 *nmap, cudaStream_t s, unsigned long long *counters,
                              const uint16_t *hint, float hint_margin) {
    const dim3 blk(32, 8), grid((g->p.resj + 31) / 32, (g->p.resi + 7) / 8);
    if (g->p.storage == SS_STORAGE_F32)
        raycast_maps_kernel<SS_STORAGE_F32><<<grid, blk, 0, s>>>(g->v, T, dpose, max_steps, t_min, t_max, vmap, nmap,
                                                                 counters, hint, hint_margin);
    else
        raycast_maps_kernel<SS_STORAGE_F16><<<grid, blk, 0, s>>>(g->v, T, dpose, max_steps, t_min, t_max, vmap, nmap,
                                                                 counters, hint, hint_margin);
    SS_LAUNCH_CHECK();
    return SS_OK;
}

}  // namespace ss

using namespace ss;

extern "C" ss_status ss_raycast(ss_grid *g, const float extr[16], float *ray_pcd, float *ray_color,
                                ss_stream_t stream) {
    if (!g || !extr || !ray_pcd) return SS_ERR_ARG;
    if (!g->intr_set) return SS_ERR_STATE;
    for (int k = 0; k < 16; k++)
        if (!std::isfinite(extr[k])) return SS_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    const dim3 blk(32, 8), grid((g->p.resj + 31) / 32, (g->p.resi + 7) / 8);
    const Mat34 Er = mat34_from(extr);
    if (g->p.storage == SS_STORAGE_F32)
        raycast_ref_kernel<SS_STORAGE_F32><<<grid, blk, 0, s>>>(g->v, Er, ray_pcd, ray_color);
    else
        raycast_ref_kernel<SS_STORAGE_F16><<<grid, blk, 0, s>>>(g->v, Er, ray_pcd, ray_color);
    SS_LAUNCH_CHECK();
    return SS_OK;
}

extern "C" ss_status ss_raycast_maps(ss_grid *g, const float extr[16], int32_t max_steps, float t_min, float t_max,
                                     const uint16_t *hint_depth, float hint_margin, float *vertex_depth,
                                     float *normal, ss_stream_t stream) {
    if (!g || !extr || !vertex_depth || !normal || max_steps <= 0 || !(t_max > t_min)) return SS_ERR_ARG;
    if (!g->intr_set) return SS_ERR_STATE;
    for (int k = 0; k < 16; k++)
        if (!std::isfinite(extr[k])) return SS_ERR_ARG;
    return launch_raycast_maps(g, mat34_from(extr), nullptr, max_steps, t_min, t_max, (float4 *)vertex_depth,
                               (float4 *)normal, (cudaStream_t)stream, nullptr, hint_depth, hint_margin);
}
