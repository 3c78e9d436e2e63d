// ss_raydiff.cu — differentiable raycast: a depth / point-to-plane loss of the
// rendered model view against an observed depth image, and its hand-written
// adjoint with respect to the camera pose (se(3), left increment) and to the
// TSDF values of the voxels the rays hit. No reference counterpart (the
// reference raycast, GPUVoxelGrid.cpp:561-715, is not differentiable).
//
// Forward, per pixel: the ray of the pipeline's trilinear raycast (same march,
// <= max_steps steps), then Newton steps on f(o + t d) = 0 to the root of the
// trilinear field, so the hit depth t* is a smooth function of the pose and of
// the 8 corner values of its cell. With r = t* - d_obs and c = n.d (n the unit
// TSDF gradient), a valid pixel adds r^2 + lambda (r c)^2 (the second term is
// the squared distance of the observed point p_obs = o + d_obs d to the
// rendered tangent plane). Valid: hit, observed depth present, |r| < r_max,
// c < -0.05 (surface facing the ray).
//
// Backward recomputes the march (no march state is stored) and uses implicit
// differentiation of f(p*) = 0, with g = grad f, H its Hessian (trilinear:
// zero diagonal), m = (I - n n^T) d / |g|, h = H m, a = dL/dt*, b = dL/dc,
// e = (a + b h.d) / (g.d):
//   dL/d omega   = -e (p x g) + b (p x h + d x n)
//   dL/d upsilon = -e g + b h
//   dL/d s_k     = -e w_k + b (m . grad w_k)
// The pose gradient is reduced per CTA (FP32), the CTAs' values added exactly
// in fixed point with integer atomics (order-independent), the last CTA
// takes the totals as doubles; voxel gradients are scattered with atomicAdd
// into a caller buffer laid out like the TSDF payload ([buckets][512] floats).
#include "ss_grid_impl.cuh"
#include "ss_trilinear.cuh"

namespace ss {

constexpr int kDiffSums = 8;  // loss, dL/domega (3), dL/dupsilon (3), valid pixels

struct CellSample {
    bool valid;
    float f, g[3], Hxy, Hxz, Hyz;
    float a, b, c;  // fractional position in the cell (x, y, z)
    int bucket[8], vox[8];
};

// Trilinear value, gradient and Hessian of the cell holding p, with the
// corners' addresses (for the scatter of voxel gradients).
template <int kStorage>
__device__ __forceinline__ void cell_sample(const GridView &g, float px, float py, float pz, float inv_vl,
                                            BlockCache &cache, CellSample &cs) {
    cs.valid = false;
    const float ux = fmaf(px, inv_vl, -0.5f), uy = fmaf(py, inv_vl, -0.5f), uz = fmaf(pz, inv_vl, -0.5f);
    const float fx0 = floorf(ux), fy0 = floorf(uy), fz0 = floorf(uz);
    const int ix = (int)fx0, iy = (int)fy0, iz = (int)fz0;
    cs.a = ux - fx0;
    cs.b = uy - fy0;
    cs.c = uz - fz0;
    float s[8];
#pragma unroll
    for (int k = 0; k < 8; k++) {
        const int vx = ix + (k & 1), vy = iy + ((k >> 1) & 1), vz = iz + (k >> 2);
        const int b = cached_lookup(g, cache, vx >> 3, vy >> 3, vz >> 3);
        if (b < 0) return;
        const int v = (vx & 7) + 8 * (vy & 7) + 64 * (vz & 7);
        const float2 sw = voxel_sw<kStorage>(g, b, v);
        if (!(sw.y > 0.f)) return;
        s[k] = sw.x;
        cs.bucket[k] = b;
        cs.vox[k] = v;
    }
    const float a = cs.a, bb = cs.b, c = cs.c;
    float f = 0.f, ga = 0.f, gb = 0.f, gc = 0.f, hab = 0.f, hac = 0.f, hbc = 0.f;
#pragma unroll
    for (int k = 0; k < 8; k++) {
        const float wx = (k & 1) ? a : 1.f - a, wy = ((k >> 1) & 1) ? bb : 1.f - bb, wz = (k >> 2) ? c : 1.f - c;
        const float sx = (k & 1) ? 1.f : -1.f, sy = ((k >> 1) & 1) ? 1.f : -1.f, sz = (k >> 2) ? 1.f : -1.f;
        f += s[k] * wx * wy * wz;
        ga += s[k] * sx * wy * wz;
        gb += s[k] * wx * sy * wz;
        gc += s[k] * wx * wy * sz;
        hab += s[k] * sx * sy * wz;
        hac += s[k] * sx * wy * sz;
        hbc += s[k] * wx * sy * sz;
    }
    cs.f = f;
    cs.g[0] = ga * inv_vl;
    cs.g[1] = gb * inv_vl;
    cs.g[2] = gc * inv_vl;
    const float iv2 = inv_vl * inv_vl;
    cs.Hxy = hab * iv2;
    cs.Hxz = hac * iv2;
    cs.Hyz = hbc * iv2;
    cs.valid = true;
}

template <int kStorage, bool kBackward>
__global__ void __launch_bounds__(256) raydiff_kernel(GridView g, Mat34 T, const uint16_t *__restrict__ obs,
                                                      int max_steps, float t_min, float t_max, float lambda_n,
                                                      float r_max, unsigned long long *__restrict__ facc,
                                                      double *result, int *ticket,
                                                      float *__restrict__ grad_vox,
                                                      float *__restrict__ depth_out,
                                                      const uint8_t *__restrict__ mask) {
    const int j = blockIdx.x * 32 + threadIdx.x;
    const int i = blockIdx.y * blockDim.y + threadIdx.y;
    float acc[kDiffSums];
#pragma unroll
    for (int k = 0; k < kDiffSums; k++) acc[k] = 0.f;
    if (i < g.resi && j < g.resj) {
        const float dcx = ((float)j - g.in.cj) / g.in.fx, dcy = ((float)i - g.in.ci) / g.in.fy;
        const float dx = fmaf(T.m[0], dcx, fmaf(T.m[1], dcy, T.m[2]));
        const float dy = fmaf(T.m[4], dcx, fmaf(T.m[5], dcy, T.m[6]));
        const float dz = fmaf(T.m[8], dcx, fmaf(T.m[9], dcy, T.m[10]));
        const float ox = T.m[3], oy = T.m[7], oz = T.m[11];
        const float inv_len = rsqrtf(fmaf(dx, dx, fmaf(dy, dy, dz * dz)));
        const float inv_vl = 1.f / g.vl;
        BlockCache cache{INT_MIN, INT_MIN, INT_MIN, -1, 0u, 0u};
        int steps = 0;
        float t = t_min;
        bool hit = march<kStorage>(g, ox, oy, oz, dx, dy, dz, inv_len, t_min, t_max, max_steps, steps, t, cache);
        CellSample cs;
        cs.valid = false;
        if (hit) {
            // Newton steps to the root of the trilinear field (bounded, safeguarded)
            for (int it = 0; it < 6; it++) {
                cell_sample<kStorage>(g, fmaf(t, dx, ox), fmaf(t, dy, oy), fmaf(t, dz, oz), inv_vl, cache, cs);
                if (!cs.valid) break;
                const float gd = cs.g[0] * dx + cs.g[1] * dy + cs.g[2] * dz;
                if (!(gd < 0.f)) {
                    cs.valid = false;
                    break;
                }
                const float dt = -cs.f / gd;
                if (fabsf(dt) > 2.f * g.vl * inv_len) {
                    cs.valid = false;
                    break;
                }
                t += dt;
                if (fabsf(dt) < 1e-7f * t) break;
            }
            if (cs.valid) cell_sample<kStorage>(g, fmaf(t, dx, ox), fmaf(t, dy, oy), fmaf(t, dz, oz), inv_vl, cache, cs);
        }
        const size_t pix = (size_t)i * g.resj + j;
        if (depth_out) depth_out[pix] = cs.valid ? t : 0.f;
        const float d_obs = (float)__ldg(obs + pix) * 1e-3f;
        if (cs.valid && d_obs > g.rmin && (!mask || __ldg(mask + pix))) {
            const float gn = sqrtf(cs.g[0] * cs.g[0] + cs.g[1] * cs.g[1] + cs.g[2] * cs.g[2]);
            const float n[3] = {cs.g[0] / gn, cs.g[1] / gn, cs.g[2] / gn};
            const float d[3] = {dx, dy, dz};
            const float cdot = n[0] * dx + n[1] * dy + n[2] * dz;
            const float r = t - d_obs;
            if (fabsf(r) < r_max && cdot < -0.05f) {
                acc[0] = r * r + lambda_n * (r * cdot) * (r * cdot);
                acc[7] = 1.f;
                if (kBackward) {
                    const float p[3] = {fmaf(t, dx, ox), fmaf(t, dy, oy), fmaf(t, dz, oz)};
                    const float a = 2.f * r * (1.f + lambda_n * cdot * cdot);
                    const float b = 2.f * lambda_n * r * r * cdot;
                    const float gd = cs.g[0] * dx + cs.g[1] * dy + cs.g[2] * dz;
                    float m[3];
#pragma unroll
                    for (int q = 0; q < 3; q++) m[q] = (d[q] - n[q] * cdot) / gn;
                    const float h[3] = {cs.Hxy * m[1] + cs.Hxz * m[2], cs.Hxy * m[0] + cs.Hyz * m[2],
                                        cs.Hxz * m[0] + cs.Hyz * m[1]};
                    const float e = (a + b * (h[0] * dx + h[1] * dy + h[2] * dz)) / gd;
                    // p x g, p x h, d x n
                    const float pg[3] = {p[1] * cs.g[2] - p[2] * cs.g[1], p[2] * cs.g[0] - p[0] * cs.g[2],
                                         p[0] * cs.g[1] - p[1] * cs.g[0]};
                    const float ph[3] = {p[1] * h[2] - p[2] * h[1], p[2] * h[0] - p[0] * h[2], p[0] * h[1] - p[1] * h[0]};
                    const float dn[3] = {d[1] * n[2] - d[2] * n[1], d[2] * n[0] - d[0] * n[2], d[0] * n[1] - d[1] * n[0]};
#pragma unroll
                    for (int q = 0; q < 3; q++) {
                        acc[1 + q] = -e * pg[q] + b * (ph[q] + dn[q]);
                        acc[4 + q] = -e * cs.g[q] + b * h[q];
                    }
                    if (grad_vox) {
                        const float ca = cs.a, cb = cs.b, cc = cs.c;
#pragma unroll
                        for (int k = 0; k < 8; k++) {
                            const float wx = (k & 1) ? ca : 1.f - ca, wy = ((k >> 1) & 1) ? cb : 1.f - cb;
                            const float wz = (k >> 2) ? cc : 1.f - cc;
                            const float sx = (k & 1) ? 1.f : -1.f, sy = ((k >> 1) & 1) ? 1.f : -1.f;
                            const float sz = (k >> 2) ? 1.f : -1.f;
                            const float mdw = (m[0] * sx * wy * wz + m[1] * wx * sy * wz + m[2] * wx * wy * sz) * inv_vl;
                            const float gk = -e * (wx * wy * wz) + b * mdw;
                            atomicAdd(grad_vox + (size_t)cs.bucket[k] * kBlockVoxels + cs.vox[k], gk);
                        }
                    }
                }
            }
        }
    }
    // CTA reduction, the CTAs' values added in fixed point (words 3 v, 3 v + 1,
    // 3 v + 2 of value v; word 3 kDiffSums counts values out of range)
    __shared__ float red[8][kDiffSums];
    __shared__ bool last;
    const int lane = (threadIdx.y * blockDim.x + threadIdx.x) & 31, wid = (threadIdx.y * blockDim.x + threadIdx.x) >> 5;
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    const int nb = gridDim.x * gridDim.y;
#pragma unroll
    for (int k = 0; k < kDiffSums; k++) {
        float v = acc[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) red[wid][k] = v;
    }
    __syncthreads();
    if (tid < kDiffSums) {
        float v = 0.f;
        for (int w = 0; w < 8; w++) v += red[w][tid];
        __int128 q;
        if (fixed48_of_float(v, q)) fixed48_add(facc + 3 * tid, q);
        else atomicAdd(facc + 3 * kDiffSums, 1ull);
    }
    // the additions, ordered by the barrier, are released by thread 0's fence
    // before its ticket; the last CTA acquires them by a fence after its own
    __syncthreads();
    if (tid == 0) {
        __threadfence();
        const bool l = atomicAdd(ticket, 1) == nb - 1;
        if (l) __threadfence();
        last = l;
    }
    __syncthreads();
    if (!last || tid >= 32) return;
    // lane v < kDiffSums: total v as a double into the mapped host result; the
    // words cleared for the next call
    const bool bad = __ldcg(facc + 3 * kDiffSums) != 0ull;
    if (lane < kDiffSums) {
        unsigned long long *w = facc + 3 * lane;
        const unsigned long long s0 = __ldcg(w), s1 = __ldcg(w + 1), s2 = __ldcg(w + 2);
        w[0] = 0ull;
        w[1] = 0ull;
        w[2] = 0ull;
        const double t = bad ? __longlong_as_double(0x7ff8000000000000ll) : f64_of_fixed48(fixed48_total(s0, s1, s2));
        result[lane] = t;
    }
    __syncwarp();
    if (lane == 0) {
        facc[3 * kDiffSums] = 0ull;
        *ticket = 0;
    }
}

struct DiffScratch {
    unsigned long long *facc = nullptr;  // 3 kDiffSums fixed-point words and the out-of-range count
    double *result_host = nullptr, *result_mapped = nullptr;  // the totals: pinned host memory, mapped
    int *ticket = nullptr;
};

static ss_status diff_scratch(ss_grid *g, DiffScratch **out) {
    static DiffScratch per_device[64];
    if (g->device < 0 || g->device >= 64) return SS_ERR_ARG;
    DiffScratch &d = per_device[g->device];
    if (!d.facc) {
        const size_t words = 3 * kDiffSums + 1;
        if (cudaMalloc(&d.facc, words * sizeof(unsigned long long)) != cudaSuccess ||
            cudaMalloc(&d.ticket, sizeof(int)) != cudaSuccess ||
            cudaHostAlloc(&d.result_host, kDiffSums * sizeof(double), cudaHostAllocMapped) != cudaSuccess ||
            cudaHostGetDevicePointer(&d.result_mapped, d.result_host, 0) != cudaSuccess) {
            cudaGetLastError();
            cudaFree(d.facc);
            cudaFree(d.ticket);
            if (d.result_host) cudaFreeHost(d.result_host);
            d = DiffScratch{};
            return SS_ERR_NOMEM;
        }
        if (cudaMemset(d.facc, 0, words * sizeof(unsigned long long)) != cudaSuccess ||
            cudaMemset(d.ticket, 0, sizeof(int)) != cudaSuccess)
            return SS_ERR_CUDA;
    }
    *out = &d;
    return SS_OK;
}

static ss_status raydiff(ss_grid *g, const double T[16], const uint16_t *obs, float lambda_n, float r_max,
                         int32_t max_steps, bool backward, double *loss, double grad[6], int64_t *valid,
                         float *grad_vox, float *depth_out, cudaStream_t s, const uint8_t *mask = nullptr) {
    if (!g || !T || !obs || !loss || max_steps <= 0 || !(r_max > 0.f)) return SS_ERR_ARG;
    if (backward && !grad) return SS_ERR_ARG;
    if (!g->intr_set) return SS_ERR_STATE;
    float Tf[16];
    for (int k = 0; k < 16; k++) {
        if (!std::isfinite(T[k])) return SS_ERR_ARG;
        Tf[k] = (float)T[k];
    }
    const dim3 blk(32, 8), grid((g->p.resj + 31) / 32, (g->p.resi + 7) / 8);
    DiffScratch *d = nullptr;
    ss_status st = diff_scratch(g, &d);
    if (st != SS_OK) return st;
    const Mat34 M = mat34_from(Tf);
    const float t_min = g->p.rmin, t_max = g->p.d_max;
#define SS_RD(ST, BW)                                                                                           \
    raydiff_kernel<ST, BW><<<grid, blk, 0, s>>>(g->v, M, obs, max_steps, t_min, t_max, lambda_n, r_max, d->facc, \
                                                d->result_mapped, d->ticket, grad_vox, depth_out, mask)
    if (g->p.storage == SS_STORAGE_F32) {
        if (backward) SS_RD(SS_STORAGE_F32, true); else SS_RD(SS_STORAGE_F32, false);
    } else {
        if (backward) SS_RD(SS_STORAGE_F16, true); else SS_RD(SS_STORAGE_F16, false);
    }
#undef SS_RD
    SS_LAUNCH_CHECK();
    SS_CUDA_TRY(cudaStreamSynchronize(s));  // the last CTA wrote the totals into mapped host memory
    double h[kDiffSums];
    for (int k = 0; k < kDiffSums; k++) h[k] = ((volatile double *)d->result_host)[k];
    *loss = h[0];
    if (backward)
        for (int k = 0; k < 6; k++) grad[k] = h[1 + k];
    if (valid) *valid = (int64_t)h[7];
    return SS_OK;
}

}  // namespace ss

using namespace ss;

extern "C" {

ss_status ss_raycast_loss(ss_grid *g, const double T[16], const uint16_t *depth_obs, float lambda_n, float r_max,
                          int32_t max_steps, double *loss, int64_t *valid_pixels, float *depth_out,
                          ss_stream_t s) {
    return raydiff(g, T, depth_obs, lambda_n, r_max, max_steps, false, loss, nullptr, valid_pixels, nullptr,
                   depth_out, (cudaStream_t)s);
}

ss_status ss_raycast_loss_grad_masked(ss_grid *g, const double T[16], const uint16_t *depth_obs,
                                      const uint8_t *pixel_mask, float lambda_n, float r_max, int32_t max_steps,
                                      double *loss, double grad_pose[6], float *grad_voxels, int64_t *valid_pixels,
                                      ss_stream_t s) {
    if (!pixel_mask) return SS_ERR_ARG;
    return raydiff(g, T, depth_obs, lambda_n, r_max, max_steps, true, loss, grad_pose, valid_pixels, grad_voxels,
                   nullptr, (cudaStream_t)s, pixel_mask);
}

ss_status ss_raycast_loss_grad(ss_grid *g, const double T[16], const uint16_t *depth_obs, float lambda_n,
                               float r_max, int32_t max_steps, double *loss, double grad_pose[6],
                               float *grad_voxels, int64_t *valid_pixels, ss_stream_t s) {
    return raydiff(g, T, depth_obs, lambda_n, r_max, max_steps, true, loss, grad_pose, valid_pixels, grad_voxels,
                   nullptr, (cudaStream_t)s);
}

}  // extern "C"
