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
    // the last sampled cell (its lowest voxel) and its 8 corner values
    int cx = INT_MIN, cy = INT_MIN, cz = INT_MIN;
    bool cok = false;
    float cs[8];
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

// Uncached find of a neighbouring block (counted as a lookup).
__device__ __forceinline__ int block_find(const GridView &g, BlockCache &c, int bx, int by, int bz) {
    c.lookups++;
    return packable(bx, by, bz) ? table_find(g, prime_hash(bx, by, bz)) : -1;
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
    if (ix == c.cx && iy == c.cy && iz == c.cz) {  // same cell as the last sample: its corners again
        if (!c.cok) return r;
#pragma unroll
        for (int k = 0; k < 8; k++) s[k] = c.cs[k];
    } else {
        // The cell's 8 corners: one lookup of the cell's lowest block, and,
        // for a cell straddling block faces, one find of each further block
        // (corner (a, b, c) lies in block offset (a sx, b sy, c sz)). One code
        // path for both kinds of cell, so that the corner loads of a warp
        // whose lanes hold both kinds are issued together.
        c.cx = ix, c.cy = iy, c.cz = iz, c.cok = false;
        const int bx0 = ix >> 3, by0 = iy >> 3, bz0 = iz >> 3;
        const bool sx = (ix & 7) == 7, sy = (iy & 7) == 7, sz = (iz & 7) == 7;
        int bk[8];
        bk[0] = cached_lookup(g, c, bx0, by0, bz0);
        if (bk[0] < 0) return r;
#pragma unroll
        for (int k = 1; k < 8; k++) bk[k] = bk[0];
        if (sx | sy | sz) {
            if (sx) bk[1] = block_find(g, c, bx0 + 1, by0, bz0);
            if (sy) bk[2] = block_find(g, c, bx0, by0 + 1, bz0);
            if (sz) bk[4] = block_find(g, c, bx0, by0, bz0 + 1);
            bk[3] = (sx && sy) ? block_find(g, c, bx0 + 1, by0 + 1, bz0) : (sx ? bk[1] : bk[2]);
            bk[5] = (sx && sz) ? block_find(g, c, bx0 + 1, by0, bz0 + 1) : (sx ? bk[1] : bk[4]);
            bk[6] = (sy && sz) ? block_find(g, c, bx0, by0 + 1, bz0 + 1) : (sy ? bk[2] : bk[4]);
            bk[7] = (sx && sy && sz) ? block_find(g, c, bx0 + 1, by0 + 1, bz0 + 1)
                                     : (sx && sy ? bk[3] : (sx && sz ? bk[5] : (sy && sz ? bk[6] : (sx ? bk[1] : (sy ? bk[2] : bk[4])))));
        }
        bool ok = true;
#pragma unroll
        for (int k = 0; k < 8; k++) ok &= bk[k] >= 0;
        if (!ok) return r;
        float2 sw[8];
#pragma unroll
        for (int k = 0; k < 8; k++) {
            const int vx = ix + (k & 1), vy = iy + ((k >> 1) & 1), vz = iz + (k >> 2);
            sw[k] = voxel_sw<kStorage>(g, bk[k], (vx & 7) + 8 * (vy & 7) + 64 * (vz & 7));
        }
        c.voxels += 8;
#pragma unroll
        for (int k = 0; k < 8; k++) {
            ok &= sw[k].y > 0.f;
            s[k] = sw[k].x;
            c.cs[k] = s[k];
        }
        c.cok = ok;
        if (!ok) return r;
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

// Regula falsi on a bracket (ta, fa > 0) .. (tb, fb < 0) of the trilinear
// field along the ray: two refinements, then the secant root.
template <int kStorage>
__device__ __forceinline__ float refine_crossing(const GridView &g, float ox, float oy, float oz, float dx, float dy,
                                                 float dz, float ta, float fa, float tb, float fb, BlockCache &cache) {
    const float inv_vl = 1.f / g.vl;
    for (int r = 0; r < 2; r++) {
        const float tc = ta + (tb - ta) * fa / (fa - fb);
        const TriSample q =
            trilinear<kStorage, false>(g, fmaf(tc, dx, ox), fmaf(tc, dy, oy), fmaf(tc, dz, oz), inv_vl, cache);
        if (!q.valid) break;
        if (q.f > 0.f) {
            ta = tc;
            fa = q.f;
        } else {
            tb = tc;
            fb = q.f;
        }
    }
    return ta + (tb - ta) * fa / (fa - fb);
}

constexpr int kRayForward = 0;  // march forward from t0 to t_hi
constexpr int kRaySeek = 1;     // search near a depth hint t0 within [t_lo, t_hi]

// Ray search, one loop with one trilinear sample per iteration for every
// mode, so lanes of a warp in different modes still share the sampling code:
//  forward: in a super-block without allocated blocks, or a block that is not
//    allocated, jump to the exit of its box; an invalid sample (unobserved
//    corner) advances one voxel; a positive one advances max(vl, 0.8 f); a
//    negative one after a positive one brackets the crossing, a negative one
//    without a positive predecessor is a back face (no hit);
//  seek (window [t_lo, t_hi]): one sample at the hint t0; unobserved: no
//    hit; positive: forward from there to t_hi (that sample is the
//    predecessor); negative:
//  back: steps back by max(vl, 0.8 |f|) until a positive sample brackets the
//    crossing (an unobserved sample, or passing t_lo, first: no hit).
// Forward marching ends at t_hi. Every sample or skip counts as one step. A
// bracket is refined by two regula-falsi steps, then the secant root is the
// hit (t).
template <int kStorage>
__device__ __forceinline__ bool ray_search(const GridView &g, float ox, float oy, float oz, float dx, float dy,
                                           float dz, float inv_len, int mode, float t0, float t_lo, float t_hi,
                                           int max_steps, int &steps, float &t, BlockCache &cache) {
    constexpr int kBack = 2;
    const float vl = g.vl, inv_vl = 1.f / g.vl, inv_vbl = 1.f / g.vbl;
    const float rdx = 1.f / dx, rdy = 1.f / dy, rdz = 1.f / dz;
    const float sbl = g.vbl * (float)(1 << kSuperShift);
    t = t0;
    bool prev_valid = false, found = false;
    float t_prev = 0.f, f_prev = 0.f;  // forward: last valid sample; back: last (negative) sample
    float ta = 0.f, fa = 0.f, tb = 0.f, fb = 0.f;  // bracket: f(ta) > 0 > f(tb)
    int csx = INT_MIN, csy = INT_MIN, csz = INT_MIN;
    bool cocc = false;
    while (steps < max_steps) {
        if (mode == kRayForward && !(t < t_hi)) break;
        const float px = fmaf(t, dx, ox), py = fmaf(t, dy, oy), pz = fmaf(t, dz, oz);
        steps++;
        if (mode == kRayForward) {
            const int bx = (int)floorf(px * inv_vbl), by = (int)floorf(py * inv_vbl), bz = (int)floorf(pz * inv_vbl);
            const int sx = bx >> kSuperShift, sy = by >> kSuperShift, sz = bz >> kSuperShift;
            if (sx != csx || sy != csy || sz != csz) {
                csx = sx;
                csy = sy;
                csz = sz;
                cocc = super_occupied(g, sx, sy, sz);
                cache.lookups++;
            }
            const bool empty_super = !cocc;
            if (empty_super || cached_lookup(g, cache, bx, by, bz) < 0) {
                // exit of the empty super-block's (or block's) box along the ray
                const float box = empty_super ? sbl : g.vbl;
                const int cx = empty_super ? sx : bx, cy = empty_super ? sy : by, cz = empty_super ? sz : bz;
                const float ex = ((float)(cx + (dx > 0.f)) * box - ox) * rdx;
                const float ey = ((float)(cy + (dy > 0.f)) * box - oy) * rdy;
                const float ez = ((float)(cz + (dz > 0.f)) * box - oz) * rdz;
                const float te = fminf(fminf(dx != 0.f ? ex : INFINITY, dy != 0.f ? ey : INFINITY),
                                       dz != 0.f ? ez : INFINITY);
                t = fmaxf(te, t) + 1e-4f * vl * inv_len;
                prev_valid = false;
                continue;
            }
        }
        const TriSample sm = trilinear<kStorage, false>(g, px, py, pz, inv_vl, cache);
        if (mode == kRayForward) {
            if (!sm.valid) {
                prev_valid = false;
                t += vl * inv_len;
                continue;
            }
            if (sm.f < 0.f) {
                found = prev_valid && f_prev > 0.f;  // else a back face
                ta = t_prev;
                fa = f_prev;
                tb = t;
                fb = sm.f;
                break;
            }
            prev_valid = true;
            t_prev = t;
            f_prev = sm.f;
            t += fmaxf(vl, 0.8f * sm.f) * inv_len;
        } else if (mode == kRaySeek) {
            if (!sm.valid) break;  // unobserved at the hint (a gap in the band): no hit
            t_prev = t;
            f_prev = sm.f;
            if (sm.f >= 0.f) {
                mode = kRayForward;
                prev_valid = true;
                // a valid sample's corner blocks exist, so the super-block of its
                // point is occupied: the first forward step needs no probe for it
                // (should rounding put the point in a neighbouring block, the march
                // only falls back from a super-block skip to a block skip)
                csx = (int)floorf(px * inv_vbl) >> kSuperShift;
                csy = (int)floorf(py * inv_vbl) >> kSuperShift;
                csz = (int)floorf(pz * inv_vbl) >> kSuperShift;
                cocc = true;
                t += fmaxf(vl, 0.8f * sm.f) * inv_len;
            } else {
                mode = kBack;
                t -= fmaxf(vl, -0.8f * sm.f) * inv_len;
                if (t < t_lo) break;
            }
        } else {  // back
            if (sm.valid && sm.f > 0.f) {
                found = true;
                ta = t;
                fa = sm.f;
                tb = t_prev;
                fb = f_prev;
                break;
            }
            if (!sm.valid) break;
            t_prev = t;
            f_prev = sm.f;
            t -= fmaxf(vl, -0.8f * sm.f) * inv_len;
            if (t < t_lo) break;
        }
    }
    if (found) t = refine_crossing<kStorage>(g, ox, oy, oz, dx, dy, dz, ta, fa, tb, fb, cache);
    return found;
}

// One forward ray march from t0 to t_max; returns true on a zero crossing (t = hit depth).
template <int kStorage>
__device__ __forceinline__ bool march(const GridView &g, float ox, float oy, float oz, float dx, float dy, float dz,
                                      float inv_len, float t0, float t_max, int max_steps, int &steps, float &t,
                                      BlockCache &cache) {
    return ray_search<kStorage>(g, ox, oy, oz, dx, dy, dz, inv_len, kRayForward, t0, t0, t_max, max_steps, steps, t,
                                cache);
}

}  // namespace ss
