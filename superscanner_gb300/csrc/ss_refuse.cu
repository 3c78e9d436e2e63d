// ss_refuse.cu — batched loop-closure re-fusion: for keyframes k = 0..n-1 in
// order, deintegrate depth k at its old pose and integrate it at its new one
// (the reference does these as 2n separate deIntegrate / integrate calls,
// src/core/integrate.cpp:109-113 and src/postprocessing/postprocessing.cpp:64-76,
// each with a block collection, a D2H count read and a device fence).
//
// Two launches for the whole batch:
//  1. refuse_collect_kernel, grid (tiles, keyframes): phase 2k deintegrates
//     and 2k+1 integrates keyframe k. Each tile's candidate blocks are
//     deduplicated in shared memory and found or inserted as in
//     collect_kernel (ss_collect.cuh); the first visitor of the batch appends
//     the block to the list, and every phase ORs its bit into the block's
//     512-bit phase mask.
//  2. refuse_apply_kernel, persistent: warps pull quarter-block items from an
//     atomic counter (blocks carry very different numbers of phases when
//     keyframes are partly occluded), keep their 4 voxels per lane in
//     registers and apply the block's phases in ascending order.
// Every voxel thus sees exactly the updates of the 2n sequential calls, in
// the same order, with the same arithmetic, so the volume is bit-identical to
// them (precision form included: the value is re-quantised to half after
// every phase as a sequential store would). Only the aliasing rule differs:
// an aliased entry takes the largest packed coordinate of the whole batch.
#include "ss_collect.cuh"
#include "ss_fuse.cuh"
#include "ss_grid_impl.cuh"

namespace ss {

// A block visited by the batched collection for one or both phases of a
// keyframe (tag bit 0: phase 2k, bit 1: phase 2k + 1, the same mask word):
// find or insert, stamp with the batch's epoch, OR the phases' bits into the
// block's mask (a load first, with the home bucket's key and stamp: other
// tiles have mostly set them already).
struct RefuseVisit {
    GridView g;
    uint32_t epoch;
    uint32_t *phase_mask;
    int word, shift;  // phase 2k's word and bit
    __device__ __forceinline__ bool operator()(int bx, int by, int bz, unsigned tag, int &bucket) {
        return find_and_stamp<true>(g, epoch, bx, by, bz, bucket, phase_mask, kPhaseWords, word, tag << shift);
    }
};

// Grid (tiles, tiles, keyframes): the tile phases of collect_kernel
// (ss_collect.cuh) for both phases of one keyframe, which share its depth
// image: the tile's depth and camera-frame points are read once, the
// deintegration phase (old pose) and the integration phase (new pose) fill one
// tagged set (keys relative to the old pose's camera block), and each distinct
// block is visited once with the bits of the phases that reach it. Registers
// capped as in collect_kernel.
__global__ void __launch_bounds__(256, 8) refuse_collect_kernel(GridView g, const uint16_t *const *__restrict__ depths,
                                                                const FramePose *__restrict__ poses,
                                                                uint32_t *__restrict__ phase_mask) {
    extern __shared__ unsigned cset[];  // [slots] keys, [slots] per-warp lists, cube entries, [slots] tags
    const int slots = kSetSlotsPerRow * blockDim.y;
    const int tid = threadIdx.y * blockDim.x + threadIdx.x, nthreads = blockDim.x * blockDim.y;
    unsigned *tags = tile_tags(cset, slots);
    for (int q = tid; q < slots; q += nthreads) {
        cset[q] = kSetEmpty;
        tags[q] = 0u;
    }
    const int phase0 = 2 * blockIdx.z;
    F3 p;
    const bool valid =
        tile_point(g, depths[blockIdx.z], blockIdx.y * blockDim.y + threadIdx.y, blockIdx.x * 32 + threadIdx.x, p);
    RefuseVisit visit{g, *(volatile uint32_t *)&g.ctr->epoch, phase_mask, phase0 >> 5, phase0 & 31};
    Mat34 E;
#pragma unroll
    for (int k = 0; k < 12; k++) E.m[k] = __ldg(&poses[phase0].E.m[k]);
    int cbx, cby, cbz;
    camera_block(g, E, cbx, cby, cbz);
    __syncthreads();
    tile_fill_set<true>(g, p, valid, E, cset, slots, cbx, cby, cbz, 1u, visit);
#pragma unroll
    for (int k = 0; k < 12; k++) E.m[k] = __ldg(&poses[phase0 + 1].E.m[k]);
    tile_fill_set<true>(g, p, valid, E, cset, slots, cbx, cby, cbz, 2u, visit);
    __syncthreads();
    tile_flush_set<true>(g, cset, slots, cbx, cby, cbz, visit);
}

template <int kStorage, bool kExact>
__global__ void __launch_bounds__(256) refuse_apply_kernel(GridView g, const uint16_t *const *__restrict__ depths,
                                                           const FramePose *__restrict__ poses,
                                                           const uint32_t *__restrict__ phase_mask) {
    const int lane = threadIdx.x & 31;
    const int n = 4 * *(volatile int *)&g.ctr->list_count;
    const int k = lane & 7, l0 = lane >> 3;
    const float inv_trunc = 1.0f / g.trunc;
    for (;;) {
        int t = 0;
        if (lane == 0) t = atomicAdd(&g.ctr->work, 1);
        t = __shfl_sync(0xffffffffu, t, 0);
        if (t >= n) break;
        const int bucket = __ldg(g.list + (t >> 2));
        const int r0 = (t & 3) * 4;
        int bx, by, bz;
        unpack_coords(__ldg(g.stamp + bucket) & ((1ull << kEpochShift) - 1ull), bx, by, bz);
        const float pzx = __fmul_rn(g.vbl, (float)bx), pzy = __fmul_rn(g.vbl, (float)by),
                    pzz = __fmul_rn(g.vbl, (float)bz);
        const float cx = __fmaf_rn((float)k + 0.5f, g.vl, pzx);
        F3 vm[4];
        float s[4], w[4];
        bool changed[4];
#pragma unroll
        for (int rr = 0; rr < 4; rr++) {
            const int r = r0 + rr, l = l0 + 4 * (r & 1), m = r >> 1;
            vm[rr] = F3{cx, __fmaf_rn((float)l + 0.5f, g.vl, pzy), __fmaf_rn((float)m + 0.5f, g.vl, pzz)};
            const size_t vi = (size_t)bucket * kBlockVoxels + lane + 32 * r;
            if (kStorage == SS_STORAGE_F32) {
                const float2 sw = g.vox32[vi];
                s[rr] = sw.x;
                w[rr] = sw.y;
            } else {
                const uint32_t word = g.vox16[vi];
                s[rr] = __half2float(__ushort_as_half((unsigned short)(word & 0xffffu))) * g.trunc;
                w[rr] = (float)(word >> 16);
            }
            changed[rr] = false;
        }
        const uint32_t *mask = phase_mask + (size_t)bucket * kPhaseWords;
        for (int wi = 0; wi < kPhaseWords; wi++) {
            uint32_t bits = __ldg(mask + wi);
            while (bits) {
                const int phase = wi * 32 + __ffs(bits) - 1;
                bits &= bits - 1;
                const bool deint = (phase & 1) == 0;
                const FramePose fp = poses[phase];
                const uint16_t *depth = depths[phase >> 1];
                F3 qf[4];  // fast path: the four camera-frame points, as fuse_kernel computes them
                if (!kExact) quad_points_fast(fp.Einv, vm[0], g.vl, qf);
#pragma unroll
                for (int rr = 0; rr < 4; rr++) {
                    float obs;
                    int pix;
                    if (kExact ? !voxel_observe(g, depth, fp.E, fp.Einv, F3{fp.Ez[0], fp.Ez[1], fp.Ez[2]}, vm[rr],
                                                      obs, pix)
                               : !observe_fast(g, depth, qf[rr], obs, pix))
                        continue;
                    if (kStorage == SS_STORAGE_F16 && deint && w[rr] == 0.f) continue;
                    float sv = s[rr], wv = w[rr];
                    if (deint)
                        running_average<true, kExact>(sv, wv, obs, g.max_weight);
                    else
                        running_average<false, kExact>(sv, wv, obs, g.max_weight);
                    if (kStorage == SS_STORAGE_F16) {  // the value a sequential call would have stored
                        sv = __half2float(__float2half_rn(sv * inv_trunc)) * g.trunc;
                        wv = fminf(wv, 65535.f);
                    }
                    s[rr] = sv;
                    w[rr] = wv;
                    changed[rr] = true;
                }
            }
        }
#pragma unroll
        for (int rr = 0; rr < 4; rr++) {
            if (!changed[rr]) continue;
            const size_t vi = (size_t)bucket * kBlockVoxels + lane + 32 * (r0 + rr);
            if (kStorage == SS_STORAGE_F32) {
                g.vox32[vi] = make_float2(s[rr], w[rr]);
            } else {
                const unsigned short hs = __half_as_ushort(__float2half_rn(s[rr] * inv_trunc));
                g.vox16[vi] = (uint32_t)hs | ((uint32_t)w[rr] << 16);
            }
        }
    }
}

// Clears the phase masks of the listed blocks, then ends the call like finalize_kernel.
__global__ void refuse_finalize_kernel(GridView g, uint32_t *phase_mask) {
    const int n = *(volatile int *)&g.ctr->list_count;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n * kPhaseWords; t += gridDim.x * blockDim.x)
        phase_mask[(size_t)g.list[t / kPhaseWords] * kPhaseWords + t % kPhaseWords] = 0u;
}

__global__ void refuse_counters_kernel(Counters *ctr) {
    const int n = ctr->list_count;
    ctr->last_touched = n;
    ctr->touched_total += (unsigned long long)n;
    ctr->calls += 1ull;
    ctr->list_count = 0;
    ctr->work = 0;
    ctr->epoch = ctr->epoch + 1u;
}

}  // namespace ss

using namespace ss;

extern "C" ss_status ss_refuse_batch(ss_grid *g, int32_t n, const uint16_t *const *depths, const float *T_old,
                                     const float *T_new, int32_t exact, ss_stream_t stream) {
    if (!g || n < 0 || (n > 0 && (!depths || !T_old || !T_new))) return SS_ERR_ARG;
    if (!g->intr_set) return SS_ERR_STATE;
    if (2 * n > kMaxPhases) return SS_ERR_DIMS;
    for (int k = 0; k < n; k++) {
        if (!depths[k]) return SS_ERR_ARG;
        for (int q = 0; q < 16; q++)
            if (!std::isfinite(T_old[k * 16 + q]) || !std::isfinite(T_new[k * 16 + q])) return SS_ERR_ARG;
    }
    cudaStream_t s = (cudaStream_t)stream;
    if (!g->phase_mask) {
        const size_t B = (size_t)g->p.hash_buckets;
        if (cudaMalloc(&g->phase_mask, B * kPhaseWords * sizeof(uint32_t)) != cudaSuccess ||
            cudaMalloc(&g->batch_poses, kMaxPhases * sizeof(FramePose)) != cudaSuccess ||
            cudaMalloc(&g->batch_depths, (kMaxPhases / 2) * sizeof(uint16_t *)) != cudaSuccess) {
            cudaGetLastError();
            return SS_ERR_NOMEM;
        }
        SS_CUDA_TRY(cudaMemsetAsync(g->phase_mask, 0, B * kPhaseWords * sizeof(uint32_t), s));
    }
    if (n == 0) return SS_OK;
    if (g->host_epoch >= kEpochMax) {
        ss_status st = rebase_epoch(g, s);
        if (st != SS_OK) return st;
    }
    FramePose hp[kMaxPhases];
    for (int k = 0; k < n; k++) {
        hp[2 * k] = frame_pose_from(T_old + 16 * k);
        hp[2 * k + 1] = frame_pose_from(T_new + 16 * k);
    }
    SS_CUDA_TRY(cudaMemcpyAsync(g->batch_poses, hp, 2 * n * sizeof(FramePose), cudaMemcpyHostToDevice, s));
    SS_CUDA_TRY(cudaMemcpyAsync(g->batch_depths, depths, n * sizeof(uint16_t *), cudaMemcpyHostToDevice, s));
    SS_CUDA_TRY(cudaMemsetAsync(&g->v.ctr->work, 0, sizeof(int), s));
    constexpr int kRows = 4;
    const dim3 cblk(32, kRows), cgrid((g->p.resj + 31) / 32, (g->p.resi + kRows - 1) / kRows, n);
    refuse_collect_kernel<<<cgrid, cblk, tile_set_bytes(kRows, true), s>>>(g->v, g->batch_depths, g->batch_poses,
                                                                     g->phase_mask);
    SS_LAUNCH_CHECK();
    const int ctas = persistent_ctas(g, g->lc.refuse_ctas_per_sm);
    const bool f32 = g->p.storage == SS_STORAGE_F32;
    if (f32 && exact) refuse_apply_kernel<SS_STORAGE_F32, true><<<ctas, 256, 0, s>>>(g->v, g->batch_depths, g->batch_poses, g->phase_mask);
    else if (f32) refuse_apply_kernel<SS_STORAGE_F32, false><<<ctas, 256, 0, s>>>(g->v, g->batch_depths, g->batch_poses, g->phase_mask);
    else if (exact) refuse_apply_kernel<SS_STORAGE_F16, true><<<ctas, 256, 0, s>>>(g->v, g->batch_depths, g->batch_poses, g->phase_mask);
    else refuse_apply_kernel<SS_STORAGE_F16, false><<<ctas, 256, 0, s>>>(g->v, g->batch_depths, g->batch_poses, g->phase_mask);
    SS_LAUNCH_CHECK();
    refuse_finalize_kernel<<<persistent_ctas(g, 2), 256, 0, s>>>(g->v, g->phase_mask);
    refuse_counters_kernel<<<1, 1, 0, s>>>(g->v.ctr);
    SS_LAUNCH_CHECK();
    g->host_epoch++;
    return SS_OK;
}
