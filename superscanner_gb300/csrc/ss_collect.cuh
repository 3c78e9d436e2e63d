// ss_collect.cuh — block collection of one 32 x rows pixel tile
// (depthToPcdTag + vbCollectionTag, GPUVoxelGrid.h:303-307,
// GPUVoxelGrid.cpp:471-514), shared by the per-call collection
// (collect_kernel, ss_grid.cu) and the batched re-fusion's
// (refuse_collect_kernel, ss_refuse.cu). One thread per pixel, two phases:
//  1. every pixel's candidates, the cube of blocks its truncation band
//     overlaps (GPUVoxelGrid.cpp:485-489), go into a shared-memory hash set,
//     so the tile's candidates are deduplicated on chip: the lanes of a warp
//     are grouped by cube (__match_any_sync on corner and extent; neighbouring
//     pixels mostly share one), and the distinct cubes' blocks are spread
//     over the lanes, 32 per step, each inserted with at most one 32-bit CAS
//     (typically one or two steps per warp instead of one per candidate of a
//     pixel). A key is the block's
//     offset from the camera's block, 10 bits per axis ([-512, 511] blocks,
//     +-16 m at 32 mm blocks); 128 slots per tile row (a tile row at 4 m and
//     4 mm voxels meets about 20 distinct blocks). Most candidates are in the
//     set already, so a plain load of the slot precedes the CAS (shared
//     atomics, not arithmetic, bound this phase). A candidate outside the
//     key range, or one the set cannot place, is visited directly;
//  2. each warp compacts its slice of the set (ballots, no atomics) and
//     visits its distinct blocks; the visits that append a block to the
//     call's list are aggregated per warp.
// The set of allocated blocks is the union of every pixel's candidates, as in
// the reference; only the number of global probes and atomics changes (one
// per distinct block per tile). 8 bytes of shared memory per slot (set and
// per-warp lists; 12 with a tagged set's tags) and 512 bytes per warp for its
// cubes: 6 KB per 4-row tile (8 KB tagged).
//
// A visitor is a callable bool (int bx, int by, int bz, unsigned tag, int
// &bucket): it finds or inserts the block, marks it, and returns true when
// this visit is the one that appends bucket to the list. A tagged set (the
// batched re-fusion's) keeps per slot the OR of the tags (2 bits) of the
// fills that entered the key, so several fills of one tile (a keyframe's two
// phases) share the set and each distinct block is visited once with the tags
// of all of them.
#pragma once

#include "ss_internal.cuh"

namespace ss {

constexpr unsigned kSetEmpty = 0xffffffffu;
constexpr int kSetSlotsPerRow = 128;
constexpr int kSetOff = 512;  // key offsets per axis: [-kSetOff, kSetOff) blocks

// Dynamic shared memory of a tile of `rows` pixel rows (rows warps): the
// set, the per-warp lists, per warp 32 cube entries of 16 bytes, and for a
// tagged set the slots' tags.
inline size_t tile_set_bytes(int rows, bool tagged = false) {
    return (size_t)kSetSlotsPerRow * rows * (tagged ? 3 : 2) * sizeof(unsigned) + (size_t)rows * 32 * sizeof(int4);
}

// The slots' tags of a tagged set (after the cube entries).
__device__ __forceinline__ unsigned *tile_tags(unsigned *cset, int slots) {
    return cset + 2 * slots + blockDim.y * 32 * 4;
}

// The camera's block, about (the origin of the set's keys) of pose E: any
// value works as long as every thread of the tile computes the same one.
__device__ __forceinline__ void camera_block(const GridView &g, const Mat34 &E, int &cbx, int &cby, int &cbz) {
    cbx = (int)floorf(E.m[3] * g.rvbl);
    cby = (int)floorf(E.m[7] * g.rvbl);
    cbz = (int)floorf(E.m[11] * g.rvbl);
}

// One visit outside the tile's set, with its own append.
template <class Visit>
__device__ __forceinline__ void visit_one(const GridView &g, int bx, int by, int bz, unsigned tag, Visit &visit) {
    int bucket = -1;
    if (!visit(bx, by, bz, tag, bucket)) return;
    const int idx = atomicAdd(&g.ctr->list_count, 1);
    if (idx <= (int)g.mask) g.list[idx] = bucket;
    else atomicOr(&g.ctr->status, kStListOverflow);
}

// The camera-frame point of pixel (i, j) (depthToPcdTag, GPUVoxelGrid.h:303-307)
// and whether it takes part (inside the image, z > rmin): the part of a
// pixel's collection that does not depend on the pose.
__device__ __forceinline__ bool tile_point(const GridView &g, const uint16_t *__restrict__ depth, int i, int j, F3 &p) {
    p = F3{0.f, 0.f, 0.f};
    if (!(i < g.resi && j < g.resj)) return false;
    p = get_point_t(g, i, j, depth_m(__ldg(depth + (size_t)i * g.resj + j)));
    return p.z > g.rmin;
}

// Phase 1 for a pixel of the tile with camera-frame point p (valid: from
// tile_point) at pose E (every thread of the CTA calls it; the set, and a
// tagged set's tags, must be cleared and the CTA synced before; fills of a
// tagged set may follow one another without a barrier).
template <bool kTagged, class Visit>
__device__ __forceinline__ void tile_fill_set(const GridView &g, F3 p, bool valid, const Mat34 &E, unsigned *cset,
                                              int slots, int cbx, int cby, int cbz, unsigned tag, Visit &visit) {
    const unsigned FULL = 0xffffffffu;
    __syncwarp();  // the warp's lanes are done with its cube entries of an earlier fill
    int lox = 0, loy = 0, loz = 0, nx = 0, ny = 0, nz = 0;
    if (valid) {
        const F3 pt = xform(E, p);
        const F3 t{g.trunc, g.trunc, g.trunc};
        const F3 lo = f3sub(pt, t), hi = f3add(pt, t);
        int hix, hiy, hiz;
        block_range(lo, hi, g.vbl, g.rvbl, lox, loy, loz, hix, hiy, hiz);
        nx = hix - lox + 1;
        ny = hiy - loy + 1;
        nz = hiz - loz + 1;
        if (nx < 1 || ny < 1 || nz < 1 || nx > 8 || ny > 8 || nz > 8) {
            atomicOr(&g.ctr->status, kStRange);  // non-finite pose or truncation > 3.5 blocks
            nx = ny = nz = 0;
        }
    }
    const int total = nx * ny * nz;
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    const int lane = tid & 31, wid = tid >> 5;
    const unsigned lt = (1u << lane) - 1u;
    const uint32_t hmask = (uint32_t)(slots - 1);
    const int hshift = __clz(slots) + 1;  // 32 - log2(slots)
    // Neighbouring pixels mostly share their whole cube of candidates: lanes
    // are grouped by cube (corner and extent), each group's leader enters its
    // cube in the warp's table, and the cubes' blocks are then spread over the
    // lanes, 32 per step. A cube is enumerated over its extents rounded up to
    // powers of two (x outer, z inner), so an item's offsets are shifts and
    // masks; items past an extent are skipped (none while the truncation band
    // spans at most two blocks per axis, the usual case).
    const bool small = abs(lox) < (1 << 16) && abs(loy) < (1 << 16) && abs(loz) < (1 << 16);
    unsigned long long cube = ~0ull - (unsigned long long)lane;  // no cube, or one not grouped: its own key
    if (total > 0 && small)
        cube = ((unsigned long long)(lox & 0x1ffff) << 46) | ((unsigned long long)(loy & 0x1ffff) << 29) |
               ((unsigned long long)(loz & 0x1ffff) << 12) | (unsigned long long)((nx - 1) | (ny - 1) << 4 | (nz - 1) << 8);
    const unsigned peers = __match_any_sync(FULL, cube);
    const bool leader = total > 0 && __ffs(peers) - 1 == lane;
    const unsigned lmask = __ballot_sync(FULL, leader);
    // log2 of the padded extents: 1 -> 0, 2 -> 1, 3-4 -> 2, 5-8 -> 3
    const int ly = 32 - __clz(max(ny - 1, 0)), lz = 32 - __clz(max(nz - 1, 0));
    const int padded = leader ? (1 << (32 - __clz(max(nx - 1, 0)) + ly + lz)) : 0;
    int incl = padded;  // inclusive scan of the leaders' padded block counts
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(FULL, incl, o);
        if (lane >= o) incl += t;
    }
    const int work = __shfl_sync(FULL, incl, 31);
    const int first = incl - padded;  // a leader's first item
    int4 *cubes = reinterpret_cast<int4 *>(cset + 2 * slots) + wid * 32;
    if (leader)
        cubes[__popc(lmask & lt)] =
            make_int4(lox, loy, loz, first << 16 | lz << 11 | ly << 9 | (nz - 1) << 6 | (ny - 1) << 3 | (nx - 1));
    __syncwarp();
    for (int base = 0; base < work; base += 32) {
        // the cube of item w: the leaders that started before this step, plus
        // those starting in it at or before w (one bit per starting item)
        const unsigned starts =
            __reduce_or_sync(FULL, leader && first >= base && first < base + 32 ? 1u << (first - base) : 0u);
        const int before = __popc(__ballot_sync(FULL, leader && first < base));
        const int w = base + lane;
        unsigned key = kSetEmpty;
        bool direct = false;
        int cx = 0, cy = 0, cz = 0;
        if (w < work) {
            const int4 cb = cubes[before + __popc(starts & (0xffffffffu >> (31 - lane))) - 1];
            const int c = w - (cb.w >> 16), sz = (cb.w >> 11) & 3, sy = (cb.w >> 9) & 3;
            const int dz = c & ((1 << sz) - 1), dy = (c >> sz) & ((1 << sy) - 1), dx = c >> (sz + sy);
            if (dx <= (cb.w & 7) && dy <= ((cb.w >> 3) & 7) && dz <= ((cb.w >> 6) & 7)) {
                cx = cb.x + dx;
                cy = cb.y + dy;
                cz = cb.z + dz;
                if (packable(cx, cy, cz)) {
                    const unsigned ox = (unsigned)(cx - cbx + kSetOff), oy = (unsigned)(cy - cby + kSetOff),
                                   oz = (unsigned)(cz - cbz + kSetOff);
                    if (ox < 2u * kSetOff && oy < 2u * kSetOff && oz < 2u * kSetOff) key = (ox << 20) | (oy << 10) | oz;
                    else direct = true;
                } else {
                    atomicOr(&g.ctr->status, kStRange);
                }
            }
        }
        if (direct) visit_one(g, cx, cy, cz, tag, visit);  // outside the key range
        if (key == kSetEmpty) continue;
        // most blocks are already in the set (another warp or step put them
        // there): a plain load finds those without an atomic
        uint32_t h = (key * 0x9E3779B1u) >> hshift;  // the product's top bits (multiplicative hashing)
        int at = -1;
        for (int probe = 0; probe < slots / 2 && at < 0; probe++) {
            h &= hmask;
            unsigned cur = ((volatile unsigned *)cset)[h];
            if (cur == kSetEmpty) cur = atomicCAS(cset + h, kSetEmpty, key);
            if (cur == kSetEmpty || cur == key) at = (int)h;
            h++;
        }
        if (at < 0) {
            visit_one(g, cx, cy, cz, tag, visit);  // set too crowded
        } else if (kTagged) {
            unsigned *tg = tile_tags(cset, slots) + at;
            if ((*(volatile unsigned *)tg & tag) != tag) atomicOr(tg, tag);
        }
    }
}

// Phase 2 (every thread of the CTA calls it after a CTA barrier that follows
// phase 1): warp w compacts slots [w per, (w + 1) per) into its list (a key
// has 30 bits; a tagged set's tag rides in the top two) and visits its
// distinct blocks, appending with one atomic per warp step.
template <bool kTagged, class Visit>
__device__ __forceinline__ void tile_flush_set(const GridView &g, unsigned *cset, int slots, int cbx, int cby,
                                               int cbz, Visit &visit) {
    const unsigned FULL = 0xffffffffu;
    const int tid = threadIdx.y * blockDim.x + threadIdx.x, nthreads = blockDim.x * blockDim.y;
    const int lane = tid & 31, wid = tid >> 5, nw = nthreads >> 5, per = slots / nw;
    const unsigned lt = (1u << lane) - 1u;
    unsigned *wlist = cset + slots + wid * per;
    int cnt = 0;
    for (int r = 0; r < per; r += 32) {
        const unsigned key = cset[wid * per + r + lane];
        const bool present = key != kSetEmpty;
        const unsigned b = __ballot_sync(FULL, present);
        if (present)
            wlist[cnt + __popc(b & lt)] = kTagged ? key | tile_tags(cset, slots)[wid * per + r + lane] << 30 : key;
        cnt += __popc(b);
    }
    __syncwarp();
    for (int base = 0; base < cnt; base += 32) {
        const int e = base + lane;
        bool append = false;
        int bucket = -1;
        if (e < cnt) {
            const unsigned key = wlist[e];
            append = visit(cbx + (int)((key >> 20) & 1023u) - kSetOff, cby + (int)((key >> 10) & 1023u) - kSetOff,
                           cbz + (int)(key & 1023u) - kSetOff, kTagged ? key >> 30 : 1u, bucket);
        }
        const unsigned ap = __ballot_sync(FULL, append);
        if (ap) {
            const int leader = __ffs(ap) - 1;
            int b0 = 0;
            if (lane == leader) b0 = atomicAdd(&g.ctr->list_count, __popc(ap));
            b0 = __shfl_sync(FULL, b0, leader);
            if (append) {
                const int idx = b0 + __popc(ap & lt);
                if (idx <= (int)g.mask) g.list[idx] = bucket;
                else atomicOr(&g.ctr->status, kStListOverflow);
            }
        }
    }
}

// Find or insert a block, then stamp it with this call's epoch: the first
// visitor of the epoch appends it (replaces alreadyIntegrated and the
// O(capacity) "Reset booleans" pass); the 64-bit atomicMax on (epoch, packed
// coordinates) also fixes an aliased entry's coordinates canonically (the
// largest packed coordinate of the call). Most visits find the block in its
// home bucket, already stamped by an earlier tile: the home bucket's key and
// stamp (and, with a side array, the block's word of it) are loaded together,
// so such a visit costs one round trip to L2 and no atomic. A stamp that
// already holds this call's value or a larger one would not change, and its
// epoch says "not first", so skipping the atomicMax then changes nothing.
// With a side array (words per bucket `side_stride`), the block's word
// `side_word` gets the bits `side_bit` ORed in (a load first: they are
// usually set; the atomic unless all of them are).
template <bool kSide = false>
__device__ __forceinline__ bool find_and_stamp(const GridView &g, uint32_t epoch, int bx, int by, int bz, int &bucket,
                                               uint32_t *side = nullptr, int side_stride = 0, int side_word = 0,
                                               uint32_t side_bit = 0) {
    const unsigned long long key = prime_hash(bx, by, bz);
    const unsigned long long val = ((unsigned long long)epoch << kEpochShift) | pack_coords(bx, by, bz);
    const uint32_t home = home_bucket(key, g.mask);
    const unsigned long long k0 = ld_relaxed(g.keys + home);
    const unsigned long long s0 = ld_relaxed(g.stamp + home);
    uint32_t m0 = 0;
    if (kSide) m0 = ld_relaxed_u32(side + (size_t)home * side_stride + side_word);
    bool append = false;
    if (k0 == key) {
        bucket = (int)home;
        if (s0 < val) append = (uint32_t)(atomicMax(g.stamp + home, val) >> kEpochShift) != epoch;
    } else {
        bool inserted = false;
        bucket = table_find_or_insert(g, key, &inserted);
        if (inserted) super_insert(g, bx, by, bz);
        if (bucket < 0) return false;
        append = (uint32_t)(atomicMax(g.stamp + bucket, val) >> kEpochShift) != epoch;
        if (kSide) m0 = ld_relaxed_u32(side + (size_t)bucket * side_stride + side_word);
    }
    if (kSide && (m0 & side_bit) != side_bit) atomicOr(side + (size_t)bucket * side_stride + side_word, side_bit);
    return append;
}

}  // namespace ss
