// ss_grid.cu — voxel-hash TSDF: block allocation (hash insertion),
// integrate / deintegrate, clean, export / import, and their C-ABI.
//
// Reference: src/VoxelGrid/GPUVoxelGrid.{h,cpp} of Pandia3DPublic/SuperScanner.
//
// Layout in HBM (bucket b of a power-of-two table owns payload b, like
// Kokkos::UnorderedMap::value_at):
//   keys   u64[B]          prime-hash key, kEmptyKey, or kTombKey
//   stamp  u64[B]          epoch of the last call that touched b | packed block coords
//   vox32  float2[B][512]  (sdf, w)                       plain form, 8 B/voxel
//   vox16  u32[B][512]     half(sdf/trunc) | u16(w) << 16 precision form, 4 B/voxel
//   rgb    f32[B][3][512]  colour planes (optional)
//   list   i32[B]          buckets touched by the current call (deduplicated)
// One 8^3 block is 4 KB (plain) or 2 KB (precision) contiguous: a warp reads a
// whole block as 16 fully coalesced 256/128-byte rows.
#include <climits>
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "ss_collect.cuh"
#include "ss_fuse.cuh"
#include "ss_grid_impl.cuh"

namespace ss {

static thread_local std::string g_last_error;

void set_last_error(const char *where, cudaError_t e) {
    g_last_error = std::string(where) + ": " + cudaGetErrorString(e);
}
void set_last_error_text(const std::string &s) { g_last_error = s; }

ss_status status_from_bits(int bits) {
    if (bits & kStTableFull) return SS_ERR_TABLE_FULL;
    if (bits & kStListOverflow) return SS_ERR_LIST_OVERFLOW;
    if (bits & kStTimeout) return SS_ERR_TIMEOUT;
    if (bits & kStRange) return SS_ERR_RANGE;
    return SS_OK;
}

Mat34 mat34_from(const float E[16]) {
    Mat34 m;
    for (int k = 0; k < 12; k++) m.m[k] = E[k];
    return m;
}

// Inverse of a 4x4 float matrix, row-major: the adjugate over the
// determinant, each cofactor a 3x3 minor expanded along its first row, all in
// double, rounded to float once (GPUVoxelGrid.cpp:55 inverts with Eigen in
// float; Eigen is not available).
static double det3_rowmajor(const double a[9]) {
    return a[0] * (a[4] * a[8] - a[5] * a[7]) - a[1] * (a[3] * a[8] - a[5] * a[6]) +
           a[2] * (a[3] * a[7] - a[4] * a[6]);
}

void inverse4_rounded(const float Ef[16], float out[16]) {
    double m[16], cof[16];
    for (int k = 0; k < 16; k++) m[k] = Ef[k];
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) {
            double sub[9];
            int n = 0;
            for (int r = 0; r < 4; r++)
                if (r != i)
                    for (int c = 0; c < 4; c++)
                        if (c != j) sub[n++] = m[4 * r + c];
            const double d = det3_rowmajor(sub);
            cof[4 * i + j] = ((i + j) & 1) ? -d : d;
        }
    const double det = m[0] * cof[0] + m[1] * cof[1] + m[2] * cof[2] + m[3] * cof[3];
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) out[4 * j + i] = (float)(cof[4 * i + j] / det);
}

int persistent_ctas(const ss_grid *g, int per_sm) { return g->num_sms * per_sm; }

// ------------------------------------------------------------------ kernels

__global__ void fill_u64_kernel(unsigned long long *p, size_t n, unsigned long long v) {
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x)
        p[t] = v;
}

// Block collection of one call (vbCollectionTag, GPUVoxelGrid.cpp:471-514,
// fused with depthToPcdTag; the two tile phases are in ss_collect.cuh).
// Registers are capped at 32 so that every tile of a 640x480 frame is
// resident at once (16 tiles of 4 rows per SM); the few bytes this spills
// cost less than a second wave of tiles (collect 0.024 -> 0.022 ms per frame).
#ifdef SS_COLLECT_TIMING
// Phase timestamps of every CTA (global timer, ns) for tuning builds only:
// start, candidates computed, set filled, tile synced, end.
constexpr int kCollectTimingCtas = 4096;
__device__ unsigned long long g_collect_timing[kCollectTimingCtas * 5];
#define SS_CT(phase)                                                                                    \
    do {                                                                                                \
        const unsigned cta_ = blockIdx.y * gridDim.x + blockIdx.x;                                      \
        if (threadIdx.x == 0 && threadIdx.y == 0 && cta_ < kCollectTimingCtas) {                        \
            unsigned long long t_;                                                                      \
            asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t_));                                      \
            g_collect_timing[cta_ * 5 + (phase)] = t_;                                                  \
        }                                                                                               \
    } while (0)
extern "C" int ss_debug_collect_timing(unsigned long long *out) {
    return (int)cudaMemcpyFromSymbol(out, g_collect_timing, sizeof(g_collect_timing));
}
#else
#define SS_CT(phase) \
    do {             \
    } while (0)
#endif

// A block visited by the per-call collection: find or insert, stamp.
struct CollectVisit {
    GridView g;
    uint32_t epoch;
    __device__ __forceinline__ bool operator()(int bx, int by, int bz, unsigned, int &bucket) {
        return find_and_stamp(g, epoch, bx, by, bz, bucket);
    }
};

__global__ void __launch_bounds__(256, 8) collect_kernel(GridView g, const uint16_t *__restrict__ depth, Mat34 E,
                                                         const FramePose *__restrict__ pose) {
    extern __shared__ unsigned cset[];  // [slots] keys, then [slots] per-warp lists
    const int slots = kSetSlotsPerRow * blockDim.y;
    const int tid = threadIdx.y * blockDim.x + threadIdx.x, nthreads = blockDim.x * blockDim.y;
    for (int q = tid; q < slots; q += nthreads) cset[q] = kSetEmpty;
    // the frame's depth is an input, not an output of the kernel before this one
    F3 p;
    const bool valid = tile_point(g, depth, blockIdx.y * blockDim.y + threadIdx.y, blockIdx.x * 32 + threadIdx.x, p);
    pdl_wait();  // the pose (tracker) and the table (previous calls)
    if (pose) {
#pragma unroll
        for (int k = 0; k < 12; k++) E.m[k] = __ldg(&pose->E.m[k]);
    }
    CollectVisit visit{g, *(volatile uint32_t *)&g.ctr->epoch};
    int cbx, cby, cbz;
    camera_block(g, E, cbx, cby, cbz);
    SS_CT(0);
    __syncthreads();
    tile_fill_set<false>(g, p, valid, E, cset, slots, cbx, cby, cbz, 1u, visit);
    SS_CT(2);
    pdl_trigger();  // the fuse kernel may launch once every tile has filled its set
    __syncthreads();
    SS_CT(3);
    tile_flush_set<false>(g, cset, slots, cbx, cby, cbz, visit);
    SS_CT(4);
}

// Integrate / deintegrate the touched blocks. A work item is a quarter of a
// block (128 voxels): one warp, 4 voxels per lane, voxel v = lane + 32 r, so
// every load and store of the warp is one contiguous row of the block and the
// 4 voxels of a lane are independent (their loads and depth gathers overlap).
// Persistent: warps stride over 4 x (device-side list length) items, so the
// launch needs no host read of the block count (the reference copies it to
// the host every call, GPUVoxelGrid.cpp:62-63).
// Voxel centres: the reference computes pzero + (k + 0.5) * vl in double and
// rounds to float (GPUVoxelGrid.cpp:521); that double sum is exact for
// |pzero| < 2^20 m, so one fmaf (single rounding of the exact value) gives the
// identical float. Registers are capped at 32 (8 CTAs, 64 warps per SM: the
// kernel waits on dependent loads, and the few spilled bytes cost less than
// the lost occupancy; 0.0164 -> 0.0154 ms per frame).
template <int kStorage, bool kColor, bool kDeint, bool kExact>
__global__ void __launch_bounds__(256, 8) fuse_kernel(GridView g, const uint16_t *__restrict__ depth,
                                                   const uint8_t *__restrict__ rgb, Mat34 E, Mat34 Einv, F3 Ez,
                                                   const FramePose *__restrict__ pose) {
    pdl_wait();     // the block list (collection) and the pose (tracker)
    pdl_trigger();  // the raycast may launch: its CTAs take the SMs this grid leaves
    if (pose) load_pose(pose, E, Einv, Ez.x, Ez.y, Ez.z);
    const int lane = threadIdx.x & 31;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    const int n = 4 * *(volatile int *)&g.ctr->list_count;
    const int k = lane & 7, l0 = lane >> 3;
    const float inv_trunc = 1.0f / g.trunc;
    // the list entry of a warp's next item is loaded while it works on the
    // current one, so an item's chain of dependent loads starts at the stamp
    int next = warp < n ? __ldg(g.list + (warp >> 2)) : 0;
    for (int t = warp; t < n; t += nwarps) {
        const int bucket = next;
        if (t + nwarps < n) next = __ldg(g.list + ((t + nwarps) >> 2));
        const int r0 = (t & 3) * 4;
        // this lane's 4 voxel words, loaded before they are known to be
        // observed: their loads overlap the stamp load and the depth gathers
        float2 sw32[4];
        uint32_t sw16[4];
#pragma unroll
        for (int rr = 0; rr < 4; rr++) {
            const size_t vi = (size_t)bucket * kBlockVoxels + lane + 32 * (r0 + rr);
            if (kStorage == SS_STORAGE_F32) sw32[rr] = g.vox32[vi];
            else sw16[rr] = g.vox16[vi];
        }
        int bx, by, bz;
        unpack_coords(__ldg(g.stamp + bucket), bx, by, bz);
        // pzero = vbl * Kvec3f(x, y, z) (GPUVoxelGrid.cpp:501)
        const float pzx = __fmul_rn(g.vbl, (float)bx), pzy = __fmul_rn(g.vbl, (float)by),
                    pzz = __fmul_rn(g.vbl, (float)bz);
        const float cx = __fmaf_rn((float)k + 0.5f, g.vl, pzx);
        F3 qf[4];  // fast path: the four camera-frame points (ss_fuse.cuh)
        if (!kExact)
            quad_points_fast(Einv, F3{cx, __fmaf_rn((float)l0 + 0.5f, g.vl, pzy), __fmaf_rn((float)(r0 >> 1) + 0.5f, g.vl, pzz)},
                             g.vl, qf);
#pragma unroll
        for (int rr = 0; rr < 4; rr++) {
            const int r = r0 + rr;
            const int l = l0 + 4 * (r & 1), m = r >> 1;
            const int v = lane + 32 * r;  // == k + 8 l + 64 m
            const F3 vm{cx, __fmaf_rn((float)l + 0.5f, g.vl, pzy), __fmaf_rn((float)m + 0.5f, g.vl, pzz)};
            const size_t vi = (size_t)bucket * kBlockVoxels + v;
            float obs;
            int pix;
            if (kExact ? !voxel_observe(g, depth, E, Einv, Ez, vm, obs, pix)
                       : !observe_fast(g, depth, qf[rr], obs, pix))
                continue;
            float s, w;
            if (kStorage == SS_STORAGE_F32) {
                s = sw32[rr].x;
                w = sw32[rr].y;
            } else {
                const uint32_t word = sw16[rr];
                s = __half2float(__ushort_as_half((unsigned short)(word & 0xffffu))) * g.trunc;
                w = (float)(word >> 16);
            }
            if (kStorage == SS_STORAGE_F16 && kDeint && w == 0.f) continue;  // u16 weight cannot go negative
            const float w_old = w;
            running_average<kDeint, kExact>(s, w, obs, g.max_weight);
            if (kStorage == SS_STORAGE_F32) {
                g.vox32[vi] = make_float2(s, w);
            } else {
                const float wc = fminf(w, 65535.f);
                const unsigned short hs = __half_as_ushort(__float2half_rn(s * inv_trunc));
                g.vox16[vi] = (uint32_t)hs | ((uint32_t)wc << 16);
            }
            if (kColor) {
                const uint8_t *c = rgb + (size_t)pix * 3;
                float *pl = g.rgb + (size_t)bucket * 3 * kBlockVoxels + v;
#pragma unroll
                for (int ch = 0; ch < 3; ch++) {
                    float cv = pl[ch * kBlockVoxels];
                    color_average<kDeint, kExact>(cv, w_old, (float)c[ch]);
                    pl[ch * kBlockVoxels] = cv;
                }
            }
        }
    }
}

// Ends a call: remembers and resets the list, advances the epoch (after the
// fuse kernel, of which it may be a programmatic dependent).
__global__ void finalize_kernel(Counters *ctr) {
    pdl_wait();
    end_call(ctr);
}

// Clears the epoch field of every stamp (run when the epoch counter wraps).
__global__ void rebase_epoch_kernel(GridView g) {
    for (size_t b = blockIdx.x * (size_t)blockDim.x + threadIdx.x; b <= g.mask; b += (size_t)gridDim.x * blockDim.x)
        g.stamp[b] &= ((1ull << kEpochShift) - 1ull);
    if (blockIdx.x == 0 && threadIdx.x == 0) g.ctr->epoch = 1u;
}

// cleanTag (GPUVoxelGrid.cpp:785-805): one warp per bucket; a block whose 512
// weights are all zero is erased (tombstone) and its payload zeroed so the
// bucket can be reused as a default-constructed block.
template <int kStorage>
__global__ void __launch_bounds__(256) clean_kernel(GridView g) {
    const int lane = threadIdx.x & 31;
    const size_t warp = (blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5;
    const size_t nwarps = ((size_t)gridDim.x * blockDim.x) >> 5;
    for (size_t b = warp; b <= g.mask; b += nwarps) {
        const unsigned long long key = g.keys[b];
        if (key == kEmptyKey || key == kTombKey) continue;
        bool nz = false;
        for (int r = 0; r < 16; r++) {
            const size_t vi = b * kBlockVoxels + lane + 32 * r;
            if (kStorage == SS_STORAGE_F32) nz |= g.vox32[vi].y != 0.f;
            else nz |= (g.vox16[vi] >> 16) != 0u;
        }
        if (__any_sync(0xffffffffu, nz)) continue;
        for (int r = 0; r < 16; r++) {
            const size_t vi = b * kBlockVoxels + lane + 32 * r;
            if (kStorage == SS_STORAGE_F32) g.vox32[vi] = make_float2(0.f, 0.f);
            else g.vox16[vi] = 0u;
            if (g.rgb) {
                float *pl = g.rgb + b * 3 * kBlockVoxels + lane + 32 * r;
                pl[0] = 0.f;
                pl[kBlockVoxels] = 0.f;
                pl[2 * kBlockVoxels] = 0.f;
            }
        }
        if (lane == 0) {
            g.stamp[b] = 0ull;
            g.keys[b] = kTombKey;
            atomicSub(&g.ctr->live_blocks, 1);
        }
    }
}

// Empties the super-blocks' bounding box (before a rebuild re-derives it).
__global__ void super_bbox_reset_kernel(Counters *c) {
    if (threadIdx.x < 3) {
        c->sb_lo[threadIdx.x] = INT_MAX;
        c->sb_hi[threadIdx.x] = INT_MIN;
    }
}

// Re-derives the super-block set from the live blocks (after clean).
__global__ void super_rebuild_kernel(GridView g) {
    for (size_t b = blockIdx.x * (size_t)blockDim.x + threadIdx.x; b <= g.mask; b += (size_t)gridDim.x * blockDim.x) {
        const unsigned long long key = g.keys[b];
        if (key == kEmptyKey || key == kTombKey) continue;
        int x, y, z;
        unpack_coords(g.stamp[b] & ((1ull << kEpochShift) - 1ull), x, y, z);
        super_insert(g, x, y, z);
    }
}

// Gathers the payload of listed buckets into compact FP32 arrays (export).
template <int kStorage>
__global__ void gather_blocks_kernel(GridView g, const int *__restrict__ buckets, int n, float *sdf, float *w,
                                     float *rgb) {
    const size_t total = (size_t)n * kBlockVoxels;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
        const int q = (int)(t / kBlockVoxels), v = (int)(t % kBlockVoxels);
        const size_t vi = (size_t)buckets[q] * kBlockVoxels + v;
        if (kStorage == SS_STORAGE_F32) {
            const float2 sw = g.vox32[vi];
            if (sdf) sdf[t] = sw.x;
            if (w) w[t] = sw.y;
        } else {
            const uint32_t word = g.vox16[vi];
            if (sdf) sdf[t] = __half2float(__ushort_as_half((unsigned short)(word & 0xffffu))) * g.trunc;
            if (w) w[t] = (float)(word >> 16);
        }
        if (rgb && g.rgb) {
            const float *pl = g.rgb + (size_t)buckets[q] * 3 * kBlockVoxels + v;
            float *o = rgb + (size_t)q * 3 * kBlockVoxels + v;
            o[0] = pl[0];
            o[kBlockVoxels] = pl[kBlockVoxels];
            o[2 * kBlockVoxels] = pl[2 * kBlockVoxels];
        }
    }
}

// Inserts imported blocks and writes their payload (import / resume).
template <int kStorage>
__global__ void import_blocks_kernel(GridView g, const int *__restrict__ coords, int n, const float *sdf,
                                     const float *w, const float *rgb) {
    const int lane = threadIdx.x & 31;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    for (int q = warp; q < n; q += nwarps) {
        const int x = coords[q * 3], y = coords[q * 3 + 1], z = coords[q * 3 + 2];
        int bucket = -1;
        if (lane == 0) {
            if (packable(x, y, z)) {
                bucket = table_find_or_insert(g, prime_hash(x, y, z));
                if (bucket >= 0) {
                    g.stamp[bucket] = pack_coords(x, y, z);
                    super_insert(g, x, y, z);
                }
            } else {
                atomicOr(&g.ctr->status, kStRange);
            }
        }
        bucket = __shfl_sync(0xffffffffu, bucket, 0);
        if (bucket < 0) continue;
        for (int r = 0; r < 16; r++) {
            const int v = lane + 32 * r;
            const size_t src = (size_t)q * kBlockVoxels + v, vi = (size_t)bucket * kBlockVoxels + v;
            if (kStorage == SS_STORAGE_F32) {
                g.vox32[vi] = make_float2(sdf[src], w[src]);
            } else {
                const float wc = fminf(fmaxf(w[src], 0.f), 65535.f);
                g.vox16[vi] = (uint32_t)__half_as_ushort(__float2half_rn(sdf[src] / g.trunc)) | ((uint32_t)wc << 16);
            }
            if (rgb && g.rgb) {
                float *pl = g.rgb + (size_t)bucket * 3 * kBlockVoxels + v;
                const float *s = rgb + (size_t)q * 3 * kBlockVoxels + v;
                pl[0] = s[0];
                pl[kBlockVoxels] = s[kBlockVoxels];
                pl[2 * kBlockVoxels] = s[2 * kBlockVoxels];
            }
        }
    }
}

// --------------------------------------------------------------- launchers

FramePose frame_pose_from(const float extr[16]) {
    FramePose fp;
    float Einv16[16];
    inverse4_rounded(extr, Einv16);
    fp.E = mat34_from(extr);
    fp.Einv = mat34_from(Einv16);
    // Ez: normalized third column of extr (GPUVoxelGrid.cpp:52-53), Kvec3f::normalize in float
    const float ex = extr[2], ey = extr[6], ez = extr[10];
    const float len = std::sqrt(ex * ex + ey * ey + ez * ez);
    fp.Ez[0] = ex / len;
    fp.Ez[1] = ey / len;
    fp.Ez[2] = ez / len;
    fp.pad = 0.f;
    return fp;
}

ss_status rebase_epoch(ss_grid *g, cudaStream_t s) {
    rebase_epoch_kernel<<<persistent_ctas(g, 4), 256, 0, s>>>(g->v);
    SS_LAUNCH_CHECK();
    g->host_epoch = 1;
    return SS_OK;
}

ss_status launch_fuse(ss_grid *g, const uint16_t *depth, const uint8_t *rgb, const FramePose &hp,
                      const FramePose *dpose, bool color, bool deint, bool exact, cudaStream_t s,
                      bool manage_epoch, cudaEvent_t after_collect, cudaEvent_t after_fuse, bool finalize) {
    const Mat34 E = hp.E, Einv = hp.Einv;
    const F3 Ez{hp.Ez[0], hp.Ez[1], hp.Ez[2]};

    if (manage_epoch && g->host_epoch >= kEpochMax) {
        ss_status st = rebase_epoch(g, s);
        if (st != SS_OK) return st;
    }
    const int cr = g->lc.collect_rows;
    const dim3 cblk(32, cr), cgrid((g->p.resj + 31) / 32, (g->p.resi + cr - 1) / cr);
    // shared set of packed coordinates + the list of its distinct entries
    const size_t csmem = tile_set_bytes(cr);  // <= 12 KB (8 rows)
    // The collection reads the depth before it waits for the kernel before it,
    // so it is a programmatic dependent only where that kernel is known not to
    // write the depth (g->pdl: the per-frame pipeline); the fuse and finalize
    // kernels wait before they read anything and follow this call's own
    // kernels, so they always are (unless an event sits between).
    SS_CUDA_TRY(launch_kernel(collect_kernel, cgrid, cblk, csmem, s, g->pdl, g->v, depth, E, dpose));
    if (after_collect) SS_CUDA_TRY(cudaEventRecord(after_collect, s));
    const int ctas = persistent_ctas(g, g->lc.fuse_ctas_per_sm);
    const bool fuse_pdl = g->pdl || !after_collect;
#define SS_FUSE(ST, C, D, X) \
    SS_CUDA_TRY(launch_kernel(fuse_kernel<ST, C, D, X>, dim3(ctas), dim3(256), 0, s, fuse_pdl, g->v, depth, rgb, E, Einv, Ez, dpose))
#define SS_FUSE_X(ST, C, D) \
    do {                    \
        if (exact) SS_FUSE(ST, C, D, true); else SS_FUSE(ST, C, D, false); \
    } while (0)
#define SS_FUSE_D(ST, C) \
    do {                 \
        if (deint) SS_FUSE_X(ST, C, true); else SS_FUSE_X(ST, C, false); \
    } while (0)
    if (g->p.storage == SS_STORAGE_F32) {
        if (color) SS_FUSE_D(SS_STORAGE_F32, true); else SS_FUSE_D(SS_STORAGE_F32, false);
    } else {
        if (color) SS_FUSE_D(SS_STORAGE_F16, true); else SS_FUSE_D(SS_STORAGE_F16, false);
    }
#undef SS_FUSE_D
#undef SS_FUSE_X
#undef SS_FUSE
    SS_LAUNCH_CHECK();
    if (after_fuse) SS_CUDA_TRY(cudaEventRecord(after_fuse, s));
    if (finalize) SS_CUDA_TRY(launch_kernel(finalize_kernel, dim3(1), dim3(1), 0, s, !after_fuse, g->v.ctr));
    if (manage_epoch) g->host_epoch++;
    return SS_OK;
}

}  // namespace ss

using namespace ss;

extern "C" {

const char *ss_last_error(void) { return g_last_error.c_str(); }

ss_status ss_params_default(ss_params *p, uint32_t capacity_voxels, float trunc, float voxel_length, int32_t resi,
                            int32_t resj) {
    if (!p || voxel_length <= 0.f || trunc <= 0.f || resi <= 0 || resj <= 0) return SS_ERR_ARG;
    uint32_t blocks = capacity_voxels / kBlockVoxels;
    uint32_t b = 1024;
    while (b < blocks && b < (1u << 30)) b <<= 1;
    p->voxel_length = voxel_length;
    p->truncation = trunc;
    p->resi = resi;
    p->resj = resj;
    p->hash_buckets = b;
    p->storage = SS_STORAGE_F32;
    p->with_color = 1;
    p->max_weight = 0.f;
    p->rmin = 0.2f;
    p->d_max = 10.0f;
    return SS_OK;
}

ss_status ss_grid_get_launch_config(const ss_grid *g, ss_launch_config *c) {
    if (!g || !c) return SS_ERR_ARG;
    *c = g->lc;
    return SS_OK;
}

ss_status ss_grid_set_launch_config(ss_grid *g, const ss_launch_config *c) {
    if (!g || !c) return SS_ERR_ARG;
    if (c->collect_rows < 1 || c->collect_rows > 8 || c->raycast_rows < 1 || c->raycast_rows > 16 ||
        c->fuse_ctas_per_sm < 1 || c->fuse_ctas_per_sm > 32 || c->refuse_ctas_per_sm < 1 ||
        c->refuse_ctas_per_sm > 32 || c->track_ctas_per_sm < 1 || c->track_ctas_per_sm > 2)
        return SS_ERR_ARG;
    g->lc = *c;
    g->launch_gen++;
    return SS_OK;
}

ss_status ss_grid_reset(ss_grid *g, ss_stream_t stream) {
    if (!g) return SS_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    const size_t B = (size_t)g->p.hash_buckets;
    fill_u64_kernel<<<persistent_ctas(g, 4), 256, 0, s>>>(g->v.keys, B, kEmptyKey);
    fill_u64_kernel<<<persistent_ctas(g, 1), 256, 0, s>>>(g->v.sbkeys, (size_t)g->v.sbmask + 1, kSuperEmpty);
    SS_LAUNCH_CHECK();
    SS_CUDA_TRY(cudaMemsetAsync(g->v.stamp, 0, B * 8, s));
    if (g->v.vox32) SS_CUDA_TRY(cudaMemsetAsync(g->v.vox32, 0, B * kBlockVoxels * sizeof(float2), s));
    if (g->v.vox16) SS_CUDA_TRY(cudaMemsetAsync(g->v.vox16, 0, B * kBlockVoxels * sizeof(uint32_t), s));
    if (g->v.rgb) SS_CUDA_TRY(cudaMemsetAsync(g->v.rgb, 0, B * 3 * kBlockVoxels * sizeof(float), s));
    Counters c;
    std::memset(&c, 0, sizeof(c));
    c.epoch = 1;
    for (int a = 0; a < 3; a++) {
        c.sb_lo[a] = INT_MAX;
        c.sb_hi[a] = INT_MIN;
    }
    SS_CUDA_TRY(cudaMemcpyAsync(g->v.ctr, &c, sizeof(c), cudaMemcpyHostToDevice, s));
    SS_CUDA_TRY(cudaStreamSynchronize(s));
    g->host_epoch = 1;
    return SS_OK;
}

ss_status ss_grid_create(const ss_params *p, ss_grid **out) {
    if (!p || !out) return SS_ERR_ARG;
    *out = nullptr;
    if (p->hash_buckets < 32 || (p->hash_buckets & (p->hash_buckets - 1)) != 0 || p->hash_buckets > (1u << 30))
        return SS_ERR_ARG;
    if (!(p->voxel_length > 0.f) || !(p->truncation > 0.f) || p->resi <= 0 || p->resj <= 0) return SS_ERR_ARG;
    if (p->storage != SS_STORAGE_F32 && p->storage != SS_STORAGE_F16) return SS_ERR_ARG;
    ss_grid *g = new ss_grid;
    g->p = *p;
    std::memset(&g->v, 0, sizeof(g->v));
    SS_CUDA_TRY(cudaGetDevice(&g->device));
    SS_CUDA_TRY(cudaDeviceGetAttribute(&g->num_sms, cudaDevAttrMultiProcessorCount, g->device));
    const size_t B = (size_t)p->hash_buckets;
    bool ok = cudaMalloc((void **)&g->v.ray_u, (size_t)p->resj * sizeof(float)) == cudaSuccess &&
              cudaMalloc((void **)&g->v.ray_v, (size_t)p->resi * sizeof(float)) == cudaSuccess &&
              cudaMalloc(&g->v.keys, B * 8) == cudaSuccess && cudaMalloc(&g->v.stamp, B * 8) == cudaSuccess &&
              cudaMalloc(&g->v.list, B * 4) == cudaSuccess && cudaMalloc(&g->v.ctr, sizeof(Counters)) == cudaSuccess;
    // super-block set: as many entries as the table has buckets, so it cannot
    // fill before the table does (scattered depths put every block in a
    // super-block of its own); at least 4096
    const size_t SB = std::max<size_t>(4096, B);
    if (ok) ok = cudaMalloc(&g->v.sbkeys, SB * 8) == cudaSuccess;
    g->v.sbmask = (uint32_t)(SB - 1);
    if (ok && p->storage == SS_STORAGE_F32)
        ok = cudaMalloc(&g->v.vox32, B * kBlockVoxels * sizeof(float2)) == cudaSuccess;
    if (ok && p->storage == SS_STORAGE_F16)
        ok = cudaMalloc(&g->v.vox16, B * kBlockVoxels * sizeof(uint32_t)) == cudaSuccess;
    if (ok && p->with_color) ok = cudaMalloc(&g->v.rgb, B * 3 * kBlockVoxels * sizeof(float)) == cudaSuccess;
    if (!ok) {
        cudaGetLastError();
        ss_grid_destroy(g);
        set_last_error_text("ss_grid_create: device allocation failed");
        return SS_ERR_NOMEM;
    }
    g->v.mask = p->hash_buckets - 1;
    g->v.vl = p->voxel_length;
    g->v.vbl = kEdge * p->voxel_length;  // GPUVoxelGrid.cpp:15
    g->v.rvbl = 1.0f / g->v.vbl;
    g->v.rvl = 1.0f / g->v.vl;
    g->v.trunc = p->truncation;
    g->v.rmin = p->rmin;
    g->v.d_max = p->d_max;
    g->v.max_weight = p->max_weight;
    g->v.resi = p->resi;
    g->v.resj = p->resj;
    ss_status st = ss_grid_reset(g, nullptr);
    if (st != SS_OK) {
        ss_grid_destroy(g);
        return st;
    }
    *out = g;
    return SS_OK;
}

ss_status ss_grid_destroy(ss_grid *g) {
    if (!g) return SS_ERR_ARG;
    cudaFree(g->v.keys);
    cudaFree(g->v.stamp);
    cudaFree(g->v.list);
    cudaFree(g->v.ctr);
    cudaFree(g->v.vox32);
    cudaFree(g->v.vox16);
    cudaFree(g->v.rgb);
    cudaFree(g->v.sbkeys);
    cudaFree((void *)g->v.ray_u);
    cudaFree((void *)g->v.ray_v);
    cudaFree(g->phase_mask);
    cudaFree(g->mesh_count);
    cudaFree(g->batch_poses);
    cudaFree((void *)g->batch_depths);
    delete g;
    return SS_OK;
}

ss_status ss_grid_set_intrinsic(ss_grid *g, float fx, float fy, float cx, float cy) {
    if (!g || !(fx != 0.f) || !(fy != 0.f)) return SS_ERR_ARG;
    g->fx = fx;
    g->fy = fy;
    g->cx = cx;
    g->cy = cy;
    g->v.in.fx = fx;
    g->v.in.fy = fy;
    g->v.in.ci = (float)g->p.resi - cy;  // ci = resi - cy (GPUVoxelGrid.cpp:259)
    g->v.in.cj = cx;                     // cj = cx (GPUVoxelGrid.cpp:260)
    // getPoint's quotients per column and row (float operations, as on the device)
    std::vector<float> u(g->p.resj), v(g->p.resi);
    for (int j = 0; j < g->p.resj; j++) u[j] = ((float)j - g->v.in.cj) / fx;
    for (int i = 0; i < g->p.resi; i++) v[i] = ((float)i - g->v.in.ci) / fy;
    SS_CUDA_TRY(cudaMemcpy((void *)g->v.ray_u, u.data(), u.size() * sizeof(float), cudaMemcpyHostToDevice));
    SS_CUDA_TRY(cudaMemcpy((void *)g->v.ray_v, v.data(), v.size() * sizeof(float), cudaMemcpyHostToDevice));
    g->intr_set = true;
    return SS_OK;
}

static ss_status fuse_entry(ss_grid *g, const uint16_t *depth, const uint8_t *rgb, const float extr[16],
                            int32_t with_color, bool deint, ss_stream_t s) {
    if (!g || !depth || !extr) return SS_ERR_ARG;
    if (!g->intr_set) return SS_ERR_STATE;
    const bool color = with_color != 0;
    if (color && (!rgb || !g->v.rgb)) return SS_ERR_ARG;
    for (int k = 0; k < 16; k++)
        if (!std::isfinite(extr[k])) return SS_ERR_ARG;
    return launch_fuse(g, depth, rgb, frame_pose_from(extr), nullptr, color, deint, /*exact=*/true, (cudaStream_t)s);
}

ss_status ss_integrate(ss_grid *g, const uint16_t *depth, const uint8_t *rgb, const float extr[16],
                       int32_t with_color, ss_stream_t s) {
    return fuse_entry(g, depth, rgb, extr, with_color, false, s);
}

ss_status ss_deintegrate(ss_grid *g, const uint16_t *depth, const uint8_t *rgb, const float extr[16],
                         int32_t with_color, ss_stream_t s) {
    return fuse_entry(g, depth, rgb, extr, with_color, true, s);
}

// Variant used by the per-frame pipeline: same kernels, FMA-contracted fast
// arithmetic and nearest-pixel association in the voxel update (block
// allocation stays reference-exact).
ss_status ss_integrate_fast(ss_grid *g, const uint16_t *depth, const uint8_t *rgb, const float extr[16],
                            int32_t with_color, int32_t deint, ss_stream_t s) {
    if (!g || !depth || !extr) return SS_ERR_ARG;
    if (!g->intr_set) return SS_ERR_STATE;
    const bool color = with_color != 0;
    if (color && (!rgb || !g->v.rgb)) return SS_ERR_ARG;
    return launch_fuse(g, depth, rgb, frame_pose_from(extr), nullptr, color, deint != 0, /*exact=*/false,
                       (cudaStream_t)s);
}

ss_status ss_clean_memory(ss_grid *g, ss_stream_t stream) {
    if (!g) return SS_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    if (g->p.storage == SS_STORAGE_F32) clean_kernel<SS_STORAGE_F32><<<persistent_ctas(g, 8), 256, 0, s>>>(g->v);
    else clean_kernel<SS_STORAGE_F16><<<persistent_ctas(g, 8), 256, 0, s>>>(g->v);
    SS_LAUNCH_CHECK();
    fill_u64_kernel<<<persistent_ctas(g, 1), 256, 0, s>>>(g->v.sbkeys, (size_t)g->v.sbmask + 1, kSuperEmpty);
    super_bbox_reset_kernel<<<1, 32, 0, s>>>(g->v.ctr);
    super_rebuild_kernel<<<persistent_ctas(g, 4), 256, 0, s>>>(g->v);
    SS_LAUNCH_CHECK();
    return SS_OK;
}

ss_status ss_grid_sync(ss_grid *g, ss_stream_t stream) {
    if (!g) return SS_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    SS_CUDA_TRY(cudaStreamSynchronize(s));
    int bits = 0;
    SS_CUDA_TRY(cudaMemcpy(&bits, &g->v.ctr->status, sizeof(int), cudaMemcpyDeviceToHost));
    if (bits) {
        int zero = 0;
        SS_CUDA_TRY(cudaMemcpy(&g->v.ctr->status, &zero, sizeof(int), cudaMemcpyHostToDevice));
    }
    return status_from_bits(bits);
}

ss_status ss_grid_block_count(ss_grid *g, ss_stream_t stream, int32_t *count) {
    if (!g || !count) return SS_ERR_ARG;
    SS_CUDA_TRY(cudaStreamSynchronize((cudaStream_t)stream));
    SS_CUDA_TRY(cudaMemcpy(count, &g->v.ctr->live_blocks, sizeof(int), cudaMemcpyDeviceToHost));
    return SS_OK;
}

// Host copy of the counters (last_touched, touched_total, calls, live blocks).
ss_status ss_grid_counters(ss_grid *g, ss_stream_t stream, int64_t out[6]) {
    if (!g || !out) return SS_ERR_ARG;
    SS_CUDA_TRY(cudaStreamSynchronize((cudaStream_t)stream));
    Counters c;
    SS_CUDA_TRY(cudaMemcpy(&c, g->v.ctr, sizeof(c), cudaMemcpyDeviceToHost));
    out[0] = c.live_blocks;
    out[1] = c.last_touched;
    out[2] = (int64_t)c.touched_total;
    out[3] = (int64_t)c.calls;
    out[4] = c.status;
    out[5] = c.epoch;
    return SS_OK;
}

ss_status ss_grid_raycast_counters(ss_grid *g, ss_stream_t stream, int64_t out[2]) {
    if (!g || !out) return SS_ERR_ARG;
    SS_CUDA_TRY(cudaStreamSynchronize((cudaStream_t)stream));
    Counters c;
    SS_CUDA_TRY(cudaMemcpy(&c, g->v.ctr, sizeof(c), cudaMemcpyDeviceToHost));
    out[0] = (int64_t)c.ray_finds;
    out[1] = (int64_t)c.ray_voxels;
    return SS_OK;
}

ss_status ss_grid_export_blocks(ss_grid *g, ss_stream_t stream, int32_t max_blocks, uint64_t *keys, int32_t *coords,
                                float *sdf, float *weight, float *rgb, int32_t *n_out) {
    if (!g || !n_out || max_blocks < 0) return SS_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    SS_CUDA_TRY(cudaStreamSynchronize(s));
    const size_t B = (size_t)g->p.hash_buckets;
    std::vector<unsigned long long> hk(B), hs(B);
    SS_CUDA_TRY(cudaMemcpy(hk.data(), g->v.keys, B * 8, cudaMemcpyDeviceToHost));
    SS_CUDA_TRY(cudaMemcpy(hs.data(), g->v.stamp, B * 8, cudaMemcpyDeviceToHost));
    std::vector<std::pair<unsigned long long, int>> items;
    for (size_t b = 0; b < B; b++)
        if (hk[b] != kEmptyKey && hk[b] != kTombKey) items.push_back({hk[b], (int)b});
    std::sort(items.begin(), items.end());
    const int n = (int)std::min<size_t>(items.size(), (size_t)max_blocks);
    *n_out = (int)items.size();
    if (n == 0) return SS_OK;
    std::vector<int> buckets(n);
    for (int q = 0; q < n; q++) {
        buckets[q] = items[q].second;
        if (keys) keys[q] = items[q].first;
        if (coords) {
            const unsigned long long p = hs[items[q].second] & ((1ull << kEpochShift) - 1ull);
            coords[q * 3 + 0] = (int)((p >> 28) & 0x3fff) - kCoordBias;
            coords[q * 3 + 1] = (int)((p >> 14) & 0x3fff) - kCoordBias;
            coords[q * 3 + 2] = (int)(p & 0x3fff) - kCoordBias;
        }
    }
    if (!sdf && !weight && !rgb) return SS_OK;
    int *d_buckets = nullptr;
    float *d_sdf = nullptr, *d_w = nullptr, *d_rgb = nullptr;
    const size_t nv = (size_t)n * kBlockVoxels;
    ss_status st = SS_OK;
    if (cudaMalloc(&d_buckets, n * sizeof(int)) != cudaSuccess || cudaMalloc(&d_sdf, nv * 4) != cudaSuccess ||
        cudaMalloc(&d_w, nv * 4) != cudaSuccess || (rgb && g->v.rgb && cudaMalloc(&d_rgb, nv * 12) != cudaSuccess)) {
        cudaGetLastError();
        st = SS_ERR_NOMEM;
    }
    if (st == SS_OK) {
        cudaMemcpy(d_buckets, buckets.data(), n * sizeof(int), cudaMemcpyHostToDevice);
        if (g->p.storage == SS_STORAGE_F32)
            gather_blocks_kernel<SS_STORAGE_F32><<<persistent_ctas(g, 4), 256, 0, s>>>(g->v, d_buckets, n, d_sdf, d_w, d_rgb);
        else
            gather_blocks_kernel<SS_STORAGE_F16><<<persistent_ctas(g, 4), 256, 0, s>>>(g->v, d_buckets, n, d_sdf, d_w, d_rgb);
        cudaError_t e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) {
            set_last_error("gather_blocks", e);
            st = SS_ERR_CUDA;
        }
    }
    if (st == SS_OK) {
        if (sdf) cudaMemcpy(sdf, d_sdf, nv * 4, cudaMemcpyDeviceToHost);
        if (weight) cudaMemcpy(weight, d_w, nv * 4, cudaMemcpyDeviceToHost);
        if (rgb) {
            if (d_rgb) cudaMemcpy(rgb, d_rgb, nv * 12, cudaMemcpyDeviceToHost);
            else std::memset(rgb, 0, nv * 12);
        }
    }
    cudaFree(d_buckets);
    cudaFree(d_sdf);
    cudaFree(d_w);
    cudaFree(d_rgb);
    return st;
}

ss_status ss_grid_export_buckets(ss_grid *g, ss_stream_t stream, int32_t max_blocks, int32_t *buckets,
                                 int32_t *n_out) {
    if (!g || !n_out || max_blocks < 0) return SS_ERR_ARG;
    SS_CUDA_TRY(cudaStreamSynchronize((cudaStream_t)stream));
    const size_t B = (size_t)g->p.hash_buckets;
    std::vector<unsigned long long> hk(B);
    SS_CUDA_TRY(cudaMemcpy(hk.data(), g->v.keys, B * 8, cudaMemcpyDeviceToHost));
    std::vector<std::pair<unsigned long long, int>> items;
    for (size_t b = 0; b < B; b++)
        if (hk[b] != kEmptyKey && hk[b] != kTombKey) items.push_back({hk[b], (int)b});
    std::sort(items.begin(), items.end());
    *n_out = (int)items.size();
    for (int q = 0; q < (int)items.size() && q < max_blocks; q++)
        if (buckets) buckets[q] = items[q].second;
    return SS_OK;
}

ss_status ss_grid_import_blocks(ss_grid *g, ss_stream_t stream, int32_t n, const int32_t *coords, const float *sdf,
                                const float *weight, const float *rgb) {
    if (!g || n < 0 || (n > 0 && (!coords || !sdf || !weight))) return SS_ERR_ARG;
    if (n == 0) return SS_OK;
    cudaStream_t s = (cudaStream_t)stream;
    const size_t nv = (size_t)n * kBlockVoxels;
    int *d_c = nullptr;
    float *d_s = nullptr, *d_w = nullptr, *d_rgb = nullptr;
    ss_status st = SS_OK;
    if (cudaMalloc(&d_c, (size_t)n * 12) != cudaSuccess || cudaMalloc(&d_s, nv * 4) != cudaSuccess ||
        cudaMalloc(&d_w, nv * 4) != cudaSuccess || (rgb && cudaMalloc(&d_rgb, nv * 12) != cudaSuccess)) {
        cudaGetLastError();
        st = SS_ERR_NOMEM;
    }
    if (st == SS_OK) {
        cudaMemcpy(d_c, coords, (size_t)n * 12, cudaMemcpyHostToDevice);
        cudaMemcpy(d_s, sdf, nv * 4, cudaMemcpyHostToDevice);
        cudaMemcpy(d_w, weight, nv * 4, cudaMemcpyHostToDevice);
        if (rgb) cudaMemcpy(d_rgb, rgb, nv * 12, cudaMemcpyHostToDevice);
        if (g->p.storage == SS_STORAGE_F32)
            import_blocks_kernel<SS_STORAGE_F32><<<persistent_ctas(g, 4), 256, 0, s>>>(g->v, d_c, n, d_s, d_w, d_rgb);
        else
            import_blocks_kernel<SS_STORAGE_F16><<<persistent_ctas(g, 4), 256, 0, s>>>(g->v, d_c, n, d_s, d_w, d_rgb);
        cudaError_t e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) {
            set_last_error("import_blocks", e);
            st = SS_ERR_CUDA;
        }
    }
    cudaFree(d_c);
    cudaFree(d_s);
    cudaFree(d_w);
    cudaFree(d_rgb);
    if (st != SS_OK) return st;
    return ss_grid_sync(g, stream);
}

}  // extern "C"
