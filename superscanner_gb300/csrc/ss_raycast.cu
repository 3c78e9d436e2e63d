// ss_raycast.cu — reference-semantics raycast (raycastingTag,
// src/VoxelGrid/GPUVoxelGrid.cpp:561-715) and its C-ABI entry point.
//
// One thread per pixel, 32x8 pixel tiles (a warp marches 32 neighbouring rays
// of one row, which stay coherent through the block-skip loop). The unit ray
// table normPcd (createNormPcdTag, :717-722) is recomputed in registers
// instead of being read from a 3.7 MB image.
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
