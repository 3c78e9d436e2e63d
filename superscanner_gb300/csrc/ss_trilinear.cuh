// ss_trilinear.cuh — trilinear TSDF sampling and the model-view ray march,
// shared by the raycast (ss_raycast.cu) and its adjoint (ss_raydiff.cu).
#pragma once

#include <climits>

#include "ss_internal.cuh"

namespace ss {

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

}  // namespace ss
