// ss_raycast.cu — reference-semantics raycast (raycastingTag,
// src/VoxelGrid/GPUVoxelGrid.cpp:561-715) and its C-ABI entry point.
//
// One thread per pixel, 32x8 pixel tiles, each warp an 8 x 4 patch of
// neighbouring rays, which stay coherent through the block-skip loop. The unit ray
// table normPcd (createNormPcdTag, :717-722) is recomputed in registers
// instead of being read from a 3.7 MB image.
#include <climits>

#include "ss_grid_impl.cuh"
#include "ss_trilinear.cuh"

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

// getVBIndeces (GPUVoxelGrid.h:162-189): the index rule of each coordinate
// (by multiplication where that is provably the IEEE quotient's result).
__device__ __forceinline__ void block_of(const GridView &g, F3 p, int &bx, int &by, int &bz) {
    bx = idx_rule_fast(p.x, g.vbl, g.rvbl);
    by = idx_rule_fast(p.y, g.vbl, g.rvbl);
    bz = idx_rule_fast(p.z, g.vbl, g.rvbl);
}

// getVinVBIndeces (GPUVoxelGrid.h:192-221): p - vbl * vbInd, then the index rule.
__device__ __forceinline__ int voxel_in_block(const GridView &g, F3 p, int bx, int by, int bz) {
    const F3 q = f3sub(p, F3{__fmul_rn(g.vbl, (float)bx), __fmul_rn(g.vbl, (float)by), __fmul_rn(g.vbl, (float)bz)});
    const int vx = idx_rule_fast(q.x, g.vl, g.rvl), vy = idx_rule_fast(q.y, g.vl, g.rvl),
              vz = idx_rule_fast(q.z, g.vl, g.rvl);
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

// Block finds of the reference raycast (UnorderedMap::find of the prime hash,
// GPUVoxelGrid.cpp:590-630). When `skip` holds, a block whose super-block
// holds no allocated block is known to be absent without a table probe: the
// super-block is looked up once per super-block the ray enters. That is exact
// only where no prime-hash collision can make another block answer the find
// (see raycast_ref_kernel).
struct SuperCache {
    int sx = INT_MIN, sy = INT_MIN, sz = INT_MIN;
    bool occ = false;
};

__device__ __forceinline__ int find_block(const GridView &g, int bx, int by, int bz, int &finds, bool skip,
                                          SuperCache &sc) {
    if (skip) {
        const int sx = bx >> kSuperShift, sy = by >> kSuperShift, sz = bz >> kSuperShift;
        if (sx != sc.sx || sy != sc.sy || sz != sc.sz) {
            sc.sx = sx;
            sc.sy = sy;
            sc.sz = sz;
            sc.occ = super_occupied(g, sx, sy, sz);
            finds++;
        }
        if (!sc.occ) return -1;
    }
    finds++;
    return table_find(g, prime_hash(bx, by, bz));
}

// The shortest difference between two block coordinates with the same prime
// hash (73856093 dx + 19349669 dy + 83492791 dz = 0 mod 2^32, dx, dy, dz not
// all zero) is 951 blocks along some axis (exhaustive search of |dx|, |dy| <=
// 3000 for the dz that solves it): blocks within 950 of each other along
// every axis never share a key.
constexpr int kHashCollisionFree = 950;

template <int kStorage>
__global__ void __launch_bounds__(256) raycast_ref_kernel(GridView g, Mat34 Er, float *__restrict__ out_pcd,
                                                          float *__restrict__ out_col, int iter_cap) {
    // warp w of the 32 x 8 tile marches an 8 x 4 pixel patch: neighbouring rays
    // in both directions take more similar paths than a 32-pixel row segment
    // (0.351 vs 0.388 ms per call at 640 x 480)
    const int w = threadIdx.y, ln = threadIdx.x;
    const int j = blockIdx.x * 32 + (w & 3) * 8 + (ln & 7);
    const int i = blockIdx.y * blockDim.y + (w >> 2) * 4 + (ln >> 3);
    if (i >= g.resi || j >= g.resj) return;
    const float vl = g.vl, vbl = g.vbl, dtr = g.trunc, dmax = g.d_max;

    const F3 np = f3normalized(get_point(g.in, i, j, 1.0f));
    F3 rv = xform(Er, np);
    const F3 dir = f3sub(rv, F3{Er.m[3], Er.m[7], Er.m[11]});
    float l = 0.1f;
    rv = f3sub(rv, f3smul(__fsub_rn(1.f, l), dir));

    bool done = false, Fn = false, Lp = false;
    int guard = 0, finds = 0, voxels = 0;  // work counters: hash and super-block finds, voxel reads

    // Skip the table probe in empty super-blocks when this ray's blocks and
    // every allocated block (within the super-blocks' bounding box) lie within
    // the collision-free extent: then a find answers only for the block itself.
    bool skip = false;
    {
        const int lo0 = __ldcg(&g.ctr->sb_lo[0]), lo1 = __ldcg(&g.ctr->sb_lo[1]), lo2 = __ldcg(&g.ctr->sb_lo[2]);
        const int hi0 = __ldcg(&g.ctr->sb_hi[0]), hi1 = __ldcg(&g.ctr->sb_hi[1]), hi2 = __ldcg(&g.ctr->sb_hi[2]);
        const float reach = dmax + 2.f * vbl;  // the march ends within d_max plus a step of the start
        const float e[3] = {Er.m[3] + reach * dir.x, Er.m[7] + reach * dir.y, Er.m[11] + reach * dir.z};
        const float c[3] = {Er.m[3], Er.m[7], Er.m[11]};
        const int lo[3] = {lo0, lo1, lo2}, hi[3] = {hi0, hi1, hi2};
        skip = true;
#pragma unroll
        for (int a = 0; a < 3; a++) {
            const float mn = fminf(c[a], e[a]), mx = fmaxf(c[a], e[a]);
            if (!(fabsf(mn) < 1e6f && fabsf(mx) < 1e6f)) skip = false;
            const long long rb_lo = (long long)floorf(mn / vbl) - 1, rb_hi = (long long)floorf(mx / vbl) + 1;
            long long bl = rb_lo, bh = rb_hi;
            if (lo[a] <= hi[a]) {  // allocated blocks lie in super-blocks lo..hi
                bl = min(bl, (long long)lo[a] * 8);
                bh = max(bh, (long long)hi[a] * 8 + 7);
            }
            if (bh - bl > kHashCollisionFree) skip = false;
        }
    }
    SuperCache sc;
    F3 hit{0.f, 0.f, 0.f};
    float cr = 0.f, cg = 0.f, cb = 0.f;

    while (!done && !Fn && l < dmax) {
        int bx, by, bz;
        block_of(g, rv, bx, by, bz);
        int bucket = find_block(g, bx, by, bz, finds, skip, sc);
        int count = 0;
        while (bucket < 0 && l < dmax && guard < iter_cap) {
            rv = f3add(rv, f3smul(vbl, dir));
            l = __fadd_rn(l, vbl);
            block_of(g, rv, bx, by, bz);
            bucket = find_block(g, bx, by, bz, finds, skip, sc);
            count++;
            guard++;
        }
        if (l >= dmax) break;
        if (count > 0) {
            const float back = __fsub_rn(vbl, dtr);
            rv = f3sub(rv, f3smul(back, dir));
            l = __fsub_rn(l, back);
            block_of(g, rv, bx, by, bz);
            bucket = find_block(g, bx, by, bz, finds, skip, sc);
            while (bucket < 0 && l < dmax && guard < iter_cap) {
                rv = f3add(rv, f3smul(dtr, dir));
                l = __fadd_rn(l, dtr);
                block_of(g, rv, bx, by, bz);
                bucket = find_block(g, bx, by, bz, finds, skip, sc);
                guard++;
            }
        }
        if (l >= dmax) break;
        if (guard >= iter_cap) break;
        // vb = value_at(index); oldvbInd = vbInd (GPUVoxelGrid.cpp:633-635)
        const int cur = bucket;
        const int ox = bx, oy = by, oz = bz;
        int v = voxel_in_block(g, rv, bx, by, bz);
        while (!done && l < dmax && ox == bx && oy == by && oz == bz && !Fn) {
            if (++guard >= iter_cap) break;
            const VoxelRead cv = read_voxel<kStorage>(g, cur, v);
            voxels++;
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
                    const int ob = (qx == ox && qy == oy && qz == oz) ? cur : find_block(g, qx, qy, qz, finds, skip, sc);
                    VoxelRead o{0.f, 0.f};
                    float orr = 0.f, og = 0.f, obb = 0.f;
                    if (ob >= 0) {  // missing block: reads as an empty voxel (reference: value_at(invalid))
                        o = read_voxel<kStorage>(g, ob, vo);
                        voxels++;
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
        if (guard >= iter_cap) break;
    }
    if (guard >= iter_cap) atomicOr(&g.ctr->status, kStTimeout);
    {  // the warp's work counts, one atomic pair per warp
        const unsigned m = __activemask();
        const unsigned f = __reduce_add_sync(m, (unsigned)finds), vx = __reduce_add_sync(m, (unsigned)voxels);
        if ((threadIdx.x & 31) == __ffs(m) - 1) {
            atomicAdd(&g.ctr->ray_finds, (unsigned long long)f);
            atomicAdd(&g.ctr->ray_voxels, (unsigned long long)vx);
        }
    }
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
// ray whose pixel has depth d searches only [d - margin, d + margin], and
// starts at d: one sample there; in front of the surface (f >= 0) the march
// goes on forward, behind it (f < 0) it steps back by max(vl, 0.8 |f|) until a
// positive sample brackets the crossing (an unobserved sample, or leaving the
// window, first: no hit); an unobserved sample at d (a gap of the band at a
// silhouette) is no hit. A pixel without depth (dropout) takes as d the
// smaller depth of the nearest pixels with depth to its left and right in its
// warp's 32-pixel row segment. Where the fused frame saw d, a crossing
// outside the window contradicts the frame just fused, so the window loses no
// consistent surface; starting at d skips the unobserved voxels in front of
// the band, which a plain march would cross one voxel at a time, and keeps
// the lanes of a warp within a few steps of each other (marching the window
// where the sample at d is unobserved recovers 0.3 % of the hits on the
// synthetic room sequence at 2.3x the warp time).
// Every sample or skip counts as one step. The normal is the normalised
// gradient of the trilinear interpolant at the hit (world frame, pointing
// out of the surface). Outputs: vmap[i][j] = (x, y, z world, depth) and
// nmap[i][j] = (nx, ny, nz, 0); misses are all-zero.
#ifdef SS_RAYCAST_TIMING
// Per-warp SM cycles of the hint, the search (with its refinement) and the
// final sample and stores, and the warps' largest and summed step counts,
// for tuning builds only.
__device__ unsigned long long g_raycast_timing[8];
#define SS_RT_NOW(v) long long v = clock64()
#define SS_RT_ADD(slot, val)                                                                 \
    do {                                                                                     \
        if ((threadIdx.x & 31) == 0) atomicAdd(&g_raycast_timing[slot], (unsigned long long)(val)); \
    } while (0)
extern "C" int ss_debug_raycast_timing(unsigned long long *out, int reset) {
    int e = (int)cudaMemcpyFromSymbol(out, g_raycast_timing, sizeof(g_raycast_timing));
    if (reset) {
        unsigned long long z[8] = {};
        cudaMemcpyToSymbol(g_raycast_timing, z, sizeof(z));
    }
    return e;
}
#else
#define SS_RT_NOW(v)
#define SS_RT_ADD(slot, val) \
    do {                     \
    } while (0)
#endif

template <int kStorage>
__global__ void __launch_bounds__(512, 2) raycast_maps_kernel(GridView g, Mat34 T, const FramePose *__restrict__ pose,
                                                           int max_steps, float t_min, float t_max,
                                                           float4 *__restrict__ vmap, float4 *__restrict__ nmap,
                                                           unsigned long long *__restrict__ counters,
                                                           const uint16_t *__restrict__ hint, float hint_margin,
                                                           Counters *end) {
    const int j = blockIdx.x * 32 + threadIdx.x;
    const int i = blockIdx.y * blockDim.y + threadIdx.y;
    const bool inside = i < g.resi && j < g.resj;
    BlockCache cache{INT_MIN, INT_MIN, INT_MIN, -1, 0u, 0u};
    int steps = 0;
    bool hit = false;
    SS_RT_NOW(rt0);
    // Depth hint of this ray: the fused frame's depth at this pixel, or, where
    // that is missing (dropout), the smaller depth of the nearest pixels with
    // depth to its left and right within this warp's 32-pixel row segment.
    unsigned hint_mm = 0;
    if (hint) {
        const unsigned full = 0xffffffffu;
        const int lane = threadIdx.x & 31;
        const unsigned own = inside ? (unsigned)__ldg(hint + (size_t)i * g.resj + j) : 0u;
        const unsigned have = __ballot_sync(full, own != 0u);
        const unsigned left = have & ((1u << lane) - 1u), right = lane < 31 ? have & (full << (lane + 1)) : 0u;
        const int li = left ? 31 - __clz(left) : lane, ri = right ? __ffs(right) - 1 : lane;
        const unsigned dl = __shfl_sync(full, own, li), dr = __shfl_sync(full, own, ri);
        hint_mm = own ? own : (left && right ? min(dl, dr) : (left ? dl : (right ? dr : 0u)));
    }
    // the hint is the frame's depth, an input; the volume, the pose and the
    // call's counters come from the kernels before this one
    pdl_wait();
    if (end && blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0 && threadIdx.y == 0) end_call(end);
    SS_RT_NOW(rt1);
    long long rt2 = 0;
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
        // seek from the hint d within [d - margin, d + margin]
        hit = ray_search<kStorage>(g, ox, oy, oz, dx, dy, dz, inv_len, kRaySeek, t_hint + hint_margin, t_hint,
                                   fminf(t_max, t_hint + 2.f * hint_margin), max_steps, steps, t, cache);
    } else {
        hit = march<kStorage>(g, ox, oy, oz, dx, dy, dz, inv_len, t_min, t_max, max_steps, steps, t, cache);
    }
#ifdef SS_RAYCAST_TIMING
    rt2 = clock64();
#endif
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
#ifdef SS_RAYCAST_TIMING
    {
        const long long rt3 = clock64();
        const unsigned full = 0xffffffffu;
        // lanes outside the image leave rt2 at 0: take the warp's latest search end
        const long long e2 = (long long)__reduce_max_sync(full, (unsigned)(rt2 ? rt2 - rt1 : 0));
        SS_RT_ADD(0, rt1 - rt0);
        SS_RT_ADD(1, e2);
        SS_RT_ADD(2, rt3 - rt1 - e2);
        const unsigned smax = __reduce_max_sync(full, (unsigned)steps), ssum = __reduce_add_sync(full, (unsigned)steps);
        SS_RT_ADD(3, smax);
        SS_RT_ADD(4, ssum);
        SS_RT_ADD(5, 1);
    }
#endif
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
                              const uint16_t *hint, float hint_margin, Counters *end) {
    const int rr = g->lc.raycast_rows;
    const dim3 blk(32, rr), grid((g->p.resj + 31) / 32, (g->p.resi + rr - 1) / rr);
    if (g->p.storage == SS_STORAGE_F32)
        SS_CUDA_TRY(launch_kernel(raycast_maps_kernel<SS_STORAGE_F32>, grid, blk, 0, s, g->pdl, g->v, T, dpose, max_steps,
                                  t_min, t_max, vmap, nmap, counters, hint, hint_margin, end));
    else
        SS_CUDA_TRY(launch_kernel(raycast_maps_kernel<SS_STORAGE_F16>, grid, blk, 0, s, g->pdl, g->v, T, dpose, max_steps,
                                  t_min, t_max, vmap, nmap, counters, hint, hint_margin, end));
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
    const int cap = g->raycast_cap > 0 ? g->raycast_cap : kRaycastIterCap;
    if (g->p.storage == SS_STORAGE_F32) {
        raycast_ref_kernel<SS_STORAGE_F32><<<grid, blk, 0, s>>>(g->v, Er, ray_pcd, ray_color, cap);
    } else {
        raycast_ref_kernel<SS_STORAGE_F16><<<grid, blk, 0, s>>>(g->v, Er, ray_pcd, ray_color, cap);
    }
    SS_LAUNCH_CHECK();
    return SS_OK;
}

extern "C" ss_status ss_grid_test_raycast_cap(ss_grid *g, int32_t cap) {
    if (!g || cap < 0) return SS_ERR_ARG;
    g->raycast_cap = cap;
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
