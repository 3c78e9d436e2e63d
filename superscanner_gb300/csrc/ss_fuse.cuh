// ss_fuse.cuh — the per-voxel observation and running-average update of
// integrate / deintegrate, shared by the per-frame fuse kernel (ss_grid.cu)
// and the batched re-fusion (ss_refuse.cu), so that a batched re-fusion gives
// bit for bit the volume of the sequential calls.
#pragma once

#include "ss_internal.cuh"

namespace ss {

// One voxel of integrationCore[Color]Tag / deIntegrationCore[Color]Tag
// (GPUVoxelGrid.cpp:345-469, 516-550) in the reference's arithmetic. Returns
// true when the voxel changes; pixel (cori, corj) and the observed sdf come
// back through the references.
__device__ __forceinline__ bool voxel_observe(const GridView &g, const uint16_t *__restrict__ depth, const Mat34 &E,
                                              const Mat34 &Einv, const F3 &Ez, F3 vm, float &sdf, int &pix) {
    const F3 q = xform(Einv, vm);
    const float c0 = __fadd_rn(__fdiv_rn(__fmul_rn(q.y, g.in.fy), q.z), g.in.ci);  // getCoordinate (GPUVoxelGrid.h:234-237)
    const float c1 = __fadd_rn(__fdiv_rn(__fmul_rn(q.x, g.in.fx), q.z), g.in.cj);
    // the reference's (int) cast (GPUVoxelGrid.cpp:348-349), which picks the pixel half a pixel off the projection
    const int cori = __float2int_rz(c0);
    const int corj = __float2int_rz(c1);
    if (!(cori < g.resi && corj < g.resj && cori >= 0 && corj >= 0)) return false;
    pix = cori * g.resj + corj;
    F3 vpt = get_point(g.in, cori, corj, depth_m(__ldg(depth + pix)));
    if (!(vpt.z > g.rmin)) return false;
    vpt = xform(E, vpt);
    sdf = f3dot(f3sub(vpt, vm), Ez);
    return fabsf(sdf) < g.trunc;
}

// The fast path's observation of a voxel from its camera-frame point q =
// Einv vm: the nearest pixel (the reference's truncation picks the pixel half
// a pixel off the projection, which makes frame-to-model tracking drift),
// within the image, with the half pixel of the rounding folded into the
// principal point and the projection from an approximate reciprocal (the
// pixel choice only needs it to ~1 ulp); its depth d > rmin; and the
// projective sdf d - q.z within the truncation: for a rigid E, (E p - vm) . Ez
// with p the pixel's point at depth d is d - q.z, the distance along the
// camera axis (a voxel behind the camera gets d + |q.z| > trunc).
__device__ __forceinline__ bool observe_fast(const GridView &g, const uint16_t *__restrict__ depth, F3 q, float &sdf,
                                             int &pix) {
    float rz;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(rz) : "f"(q.z));
    const int cori = __float2int_rd(fmaf(q.y * g.in.fy, rz, g.in.ci + 0.5f));
    const int corj = __float2int_rd(fmaf(q.x * g.in.fx, rz, g.in.cj + 0.5f));
    if (!(cori < g.resi && corj < g.resj && cori >= 0 && corj >= 0)) return false;
    pix = cori * g.resj + corj;
    const float d = (float)__ldg(depth + pix) * 1.0e-3f;
    if (!(d > g.rmin)) return false;
    sdf = d - q.z;
    return fabsf(sdf) < g.trunc;
}

// Camera-frame points of a lane's four voxels r0 .. r0 + 3 (r0 even: voxel
// (l0, m0) of vm0, then (l0 + 4, m0), (l0, m0 + 1), (l0 + 4, m0 + 1)) for the
// fast path: the first as Einv vm0, the others by adding the transformed
// voxel steps (4 vl along y, vl along z), with rounded operations that are
// never contracted, so every kernel computes the same values (the per-frame
// fusion and the batched re-fusion stay bit-identical).
__device__ __forceinline__ void quad_points_fast(const Mat34 &Einv, F3 vm0, float vl, F3 q[4]) {
    q[0].x = fmaf(vm0.x, Einv.m[0], fmaf(vm0.y, Einv.m[1], fmaf(vm0.z, Einv.m[2], Einv.m[3])));
    q[0].y = fmaf(vm0.x, Einv.m[4], fmaf(vm0.y, Einv.m[5], fmaf(vm0.z, Einv.m[6], Einv.m[7])));
    q[0].z = fmaf(vm0.x, Einv.m[8], fmaf(vm0.y, Einv.m[9], fmaf(vm0.z, Einv.m[10], Einv.m[11])));
    const float sy = __fmul_rn(4.f, vl);
    const F3 dy{__fmul_rn(Einv.m[1], sy), __fmul_rn(Einv.m[5], sy), __fmul_rn(Einv.m[9], sy)};
    const F3 dz{__fmul_rn(Einv.m[2], vl), __fmul_rn(Einv.m[6], vl), __fmul_rn(Einv.m[10], vl)};
    q[1] = F3{__fadd_rn(q[0].x, dy.x), __fadd_rn(q[0].y, dy.y), __fadd_rn(q[0].z, dy.z)};
    q[2] = F3{__fadd_rn(q[0].x, dz.x), __fadd_rn(q[0].y, dz.y), __fadd_rn(q[0].z, dz.z)};
    q[3] = F3{__fadd_rn(q[2].x, dy.x), __fadd_rn(q[2].y, dy.y), __fadd_rn(q[2].z, dy.z)};
}

// Running-average update of one voxel (sdf, weight) in FP32.
template <bool kDeint, bool kExact>
__device__ __forceinline__ void running_average(float &s, float &w, float obs, float max_weight) {
    if (!kDeint) {
        const float w1 = kExact ? __fadd_rn(w, 1.f) : w + 1.f;
        s = kExact ? __fdiv_rn(__fadd_rn(__fmul_rn(s, w), obs), w1) : __fdividef(fmaf(s, w, obs), w1);
        w = (max_weight > 0.f && w1 > max_weight) ? max_weight : w1;
    } else {
        if (w != 1.f) {
            const float w1 = kExact ? __fsub_rn(w, 1.f) : w - 1.f;
            s = kExact ? __fdiv_rn(__fsub_rn(__fmul_rn(s, w), obs), w1) : __fdividef(fmaf(s, w, -obs), w1);
            w = w1;
        } else {
            w = 0.f;
            s = 0.f;
        }
    }
}

template <bool kDeint, bool kExact>
__device__ __forceinline__ void color_average(float &c, float w_old, float obs) {
    if (!kDeint) {
        c = kExact ? __fdiv_rn(__fadd_rn(__fmul_rn(c, w_old), obs), __fadd_rn(w_old, 1.f))
                   : __fdividef(fmaf(c, w_old, obs), w_old + 1.f);
    } else {
        if (w_old != 1.f) {
            c = kExact ? __fdiv_rn(__fsub_rn(__fmul_rn(c, w_old), obs), __fsub_rn(w_old, 1.f))
                       : __fdividef(fmaf(c, w_old, -obs), w_old - 1.f);
        } else {
            c = 0.f;
        }
    }
}

}  // namespace ss
