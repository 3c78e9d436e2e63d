// ss_track.cu — frame-to-model point-to-plane Gauss-Newton tracking.
//
// The reference tracks with keypoints and aligns frames in post-processing
// with kokkosICP (src/postprocessing/kokkosICP.cpp); the per-frame
// integrate -> raycast -> ICP pipeline tracks each new depth frame against
// the raycast model view instead (projective association, point-to-plane
// residual), over a 3-level pyramid of the source depth.
//
// Source pixels of level l are the level-0 pixels (i 2^l, j 2^l)
// back-projected with the level-0 intrinsics (no pyramid images are built).
// Each thread accumulates the 21 + 6 + 2 normal-equation sums in FP32 (four
// pixels' terms by FMA, then one Kahan-compensated add per group); warps
// combine (sum, compensation) pairs with TwoSum through shuffles, CTAs
// through shared memory. One warp then solves the 6x6 system and applies the
// SE(3) update in FP64 (ss_track_solve.cuh). Two launch forms: one
// cooperative launch per frame (CTA totals added exactly in fixed point with
// integer atomics, one grid barrier per iteration, every CTA solves
// redundantly), or one launch per iteration (CTA slots reduced with TwoSum in
// a fixed order by the last CTA to finish, which solves). No host
// synchronisation between iterations, levels or frames.
#include "ss_grid_impl.cuh"
#include "ss_track.cuh"
#include "ss_track_solve.cuh"

namespace ss {

constexpr int kTrackSums = 29;  // JtJ upper triangle (21), Jtr (6), r^2, count

__device__ __forceinline__ void kahan_add(float &s, float &c, float x) {
    const float y = x - c;
    const float t = s + y;
    c = (t - s) - y;
    s = t;
}

// (s1 + c1) + (s2 + c2) with the rounding error of s1 + s2 kept (TwoSum).
__device__ __forceinline__ void pair_add(float &s, float &c, float s2, float c2) {
    const float t = s + s2;
    const float bp = t - s;
    const float e = (s - (t - bp)) + (s2 - bp);
    s = t;
    c = c + c2 - e;  // compensation holds the negated error (kahan convention: value = s - c)
}

// pair_add of two independent pairs at once (packed: value 0 in the low
// halves), the same operations in the same order on each half.
__device__ __forceinline__ void pair_add2(f32x2 &s, f32x2 &c, f32x2 s2, f32x2 c2) {
    const f32x2 t = f2_add(s, s2);
    const f32x2 bp = f2_sub(t, s);
    const f32x2 e = f2_add(f2_sub(s, f2_sub(t, bp)), f2_sub(s2, bp));
    s = t;
    c = f2_sub(f2_add(c, c2), e);
}

__device__ void mat_from_T(const double *T, float *m) {
    for (int k = 0; k < 12; k++) m[k] = (float)T[k];
}

// Rigid inverse of a 4x4 double pose: [R^T, -R^T t].
__device__ void rigid_inverse(const double *T, double *Ti) {
    for (int r = 0; r < 3; r++) {
        for (int c = 0; c < 3; c++) Ti[r * 4 + c] = T[c * 4 + r];
        Ti[r * 4 + 3] = -(T[0 * 4 + r] * T[3] + T[1 * 4 + r] * T[7] + T[2 * 4 + r] * T[11]);
    }
    Ti[12] = Ti[13] = Ti[14] = 0.0;
    Ti[15] = 1.0;
}

// FramePose of a double pose: float E, float inverse, normalized z column.
__device__ void write_frame_pose(const double *T, FramePose *fp) {
    double Ti[16];
    rigid_inverse(T, Ti);
    for (int k = 0; k < 12; k++) {
        fp->E.m[k] = (float)T[k];
        fp->Einv.m[k] = (float)Ti[k];
    }
    const float ex = (float)T[2], ey = (float)T[6], ez = (float)T[10];
    const float len = sqrtf(ex * ex + ey * ey + ez * ez);
    fp->Ez[0] = ex / len;
    fp->Ez[1] = ey / len;
    fp->Ez[2] = ez / len;
    fp->pad = 0.f;
}

// Start of a frame: the model maps were raycast at the last pose T, so
// Tprev = T, and tracking starts from T (or from Tstart when one was set).
__global__ void track_begin_kernel(TrackState *st) {
    if (threadIdx.x != 0) return;
    double Ti[16];
    for (int k = 0; k < 16; k++) st->Tprev[k] = st->T[k];
    rigid_inverse(st->Tprev, Ti);
    for (int k = 0; k < 12; k++) st->Tprev_inv[k] = (float)Ti[k];
    if (st->has_start) {  // ICP start other than the model pose (one-shot)
        for (int k = 0; k < 16; k++) st->T[k] = st->Tstart[k];
        st->has_start = 0;
    }
    mat_from_T(st->T, st->Tf);
    st->ticket = 0;
    st->barrier = 0u;
    st->converged_level = -1;
    for (int l = 0; l < kMaxLevels; l++) {
        st->inliers[l] = 0;
        st->rmse[l] = 0.f;
    }
}

__global__ void pose_prep_kernel(TrackState *st) {
    if (threadIdx.x == 0) write_frame_pose(st->T, &st->pose);
}

// Accumulates this thread's share of one Gauss-Newton iteration at a level
// into Kahan (sum, compensation) pairs. The thread's pixels are visited in
// groups of kTrackGroup: all depth loads of a group, then all model-map loads,
// then the sums, so the two dependent memory round trips of a pixel overlap
// with those of the others. A group's terms are summed with plain FMAs, then
// added to the Kahan pairs once per group (the running sums stay compensated;
// a group adds at most kTrackGroup - 1 roundings).
constexpr int kTrackGroup = 4;

__device__ __forceinline__ void track_accumulate(const uint16_t *__restrict__ depth, int rows, int cols, Intr in,
                                                 const float4 *__restrict__ vmap, const float4 *__restrict__ nmap,
                                                 const float *T, const float *Pi, int level, float dist2, float rmin,
                                                 float dmax, int tid, int nthreads, float *s, float *c) {
    const int lr = (rows + (1 << level) - 1) >> level, lc = (cols + (1 << level) - 1) >> level;
    const int npix = lr * lc;
    const float rfx = 1.f / in.fx, rfy = 1.f / in.fy;
    for (int base = tid; base < npix; base += kTrackGroup * nthreads) {
        float d[kTrackGroup];
        int pi[kTrackGroup], pj[kTrackGroup];
#pragma unroll
        for (int g = 0; g < kTrackGroup; g++) {
            const int p = base + g * nthreads;
            pi[g] = (p / lc) << level;
            pj[g] = (p % lc) << level;
            d[g] = p < npix ? (float)__ldg(depth + (size_t)pi[g] * cols + pj[g]) * 1e-3f : 0.f;
        }
        float wv[kTrackGroup][3];
        float4 n[kTrackGroup], v[kTrackGroup];
        bool ok[kTrackGroup];
#pragma unroll
        for (int g = 0; g < kTrackGroup; g++) {
            const float dd = d[g];
            const float cx = ((float)pj[g] - in.cj) * rfx * dd, cy = ((float)pi[g] - in.ci) * rfy * dd;
            const float wx = fmaf(T[0], cx, fmaf(T[1], cy, fmaf(T[2], dd, T[3])));
            const float wy = fmaf(T[4], cx, fmaf(T[5], cy, fmaf(T[6], dd, T[7])));
            const float wz = fmaf(T[8], cx, fmaf(T[9], cy, fmaf(T[10], dd, T[11])));
            const float qx = fmaf(Pi[0], wx, fmaf(Pi[1], wy, fmaf(Pi[2], wz, Pi[3])));
            const float qy = fmaf(Pi[4], wx, fmaf(Pi[5], wy, fmaf(Pi[6], wz, Pi[7])));
            const float qz = fmaf(Pi[8], wx, fmaf(Pi[9], wy, fmaf(Pi[10], wz, Pi[11])));
            wv[g][0] = wx;
            wv[g][1] = wy;
            wv[g][2] = wz;
            bool good = (dd > rmin) && (dd < dmax) && (qz > 1e-3f);
            int ii = 0, jj = 0;
            if (good) {
                const float rq = 1.f / qz;
                ii = (int)floorf(fmaf(qy * in.fy, rq, in.ci) + 0.5f);
                jj = (int)floorf(fmaf(qx * in.fx, rq, in.cj) + 0.5f);
                good = ii >= 0 && ii < rows && jj >= 0 && jj < cols;
            }
            ok[g] = good;
            const size_t m = good ? (size_t)ii * cols + jj : 0;
            n[g] = good ? __ldg(nmap + m) : make_float4(0.f, 0.f, 0.f, 0.f);
            v[g] = good ? __ldg(vmap + m) : make_float4(0.f, 0.f, 0.f, 0.f);
        }
        float t[kTrackSums - 1];
#pragma unroll
        for (int q = 0; q < kTrackSums - 1; q++) t[q] = 0.f;
        bool any = false;
#pragma unroll
        for (int g = 0; g < kTrackGroup; g++) {
            if (!ok[g]) continue;
            const float4 nn = n[g], vv = v[g];
            if (nn.x == 0.f && nn.y == 0.f && nn.z == 0.f) continue;
            const float wx = wv[g][0], wy = wv[g][1], wz = wv[g][2];
            const float ex = wx - vv.x, ey = wy - vv.y, ez = wz - vv.z;
            if (ex * ex + ey * ey + ez * ez > dist2) continue;
            const float r = nn.x * ex + nn.y * ey + nn.z * ez;
            const float J[6] = {wy * nn.z - wz * nn.y, wz * nn.x - wx * nn.z, wx * nn.y - wy * nn.x, nn.x, nn.y, nn.z};
            int q = 0;
#pragma unroll
            for (int a = 0; a < 6; a++)
#pragma unroll
                for (int b = a; b < 6; b++) t[q] = fmaf(J[a], J[b], t[q]), q++;
#pragma unroll
            for (int a = 0; a < 6; a++) t[21 + a] = fmaf(J[a], r, t[21 + a]);
            t[27] = fmaf(r, r, t[27]);
            s[28] += 1.f;  // counts stay exact far below 2^24
            any = true;
        }
        if (any) {
#pragma unroll
            for (int q = 0; q < kTrackSums - 1; q++) kahan_add(s[q], c[q], t[q]);
        }
    }
}

// The persistent tracker keeps each thread's source points of a level in
// shared memory across the level's iterations (a pixel's camera-frame point
// does not depend on the pose): up to kCamCache pixels per thread.
constexpr int kCamCache = 8;

// Camera-frame points (x, y, d, valid) of this thread's pixels at a level,
// the same pixels in the same order as track_accumulate.
__device__ __forceinline__ void track_fill_cam(const uint16_t *__restrict__ depth, int rows, int cols, Intr in,
                                               int level, float rmin, float dmax, int tid, int nthreads, int m_count,
                                               float4 (*cam)[256]) {
    const int lc = (cols + (1 << level) - 1) >> level;
    const int npix = ((rows + (1 << level) - 1) >> level) * lc;
    const float rfx = 1.f / in.fx, rfy = 1.f / in.fy;
#pragma unroll
    for (int m = 0; m < kCamCache; m++) {
        if (m >= m_count) break;
        const int p = tid + m * nthreads;
        float4 cp = make_float4(0.f, 0.f, 0.f, 0.f);
        if (p < npix) {
            const int i = (p / lc) << level, j = (p % lc) << level;
            const float d = (float)__ldg(depth + (size_t)i * cols + j) * 1e-3f;
            if ((d > rmin) && (d < dmax))
                cp = make_float4(((float)j - in.cj) * rfx * d, ((float)i - in.ci) * rfy * d, d, 1.f);
        }
        cam[m][threadIdx.x] = cp;
    }
}

// track_accumulate over the cached camera points (groups of kG: all
// model-map loads of a group before its sums). A group's terms are summed
// with plain FMAs, then added to the Kahan pairs once per group (the running
// sums stay compensated; a group adds at most kG - 1 roundings). With
// kG = kCamCache the thread's points are one group: every gather of the
// iteration is in flight at once (one memory round trip), and the pairs are
// the group's sums with zero compensation.
template <int kG>
__device__ __forceinline__ void track_accumulate_cam(const float4 (*cam)[256], int m_count, int rows, int cols,
                                                     Intr in, const float4 *__restrict__ vmap,
                                                     const float4 *__restrict__ nmap, const float *T, const float *Pi,
                                                     float dist2, float *s, float *c) {
    for (int m0 = 0; m0 < m_count; m0 += kG) {
        float wv[kG][3];
        float4 n[kG], v[kG];
        bool ok[kG];
#pragma unroll
        for (int g = 0; g < kG; g++) {
            const float4 cp = (m0 + g < m_count) ? cam[m0 + g][threadIdx.x] : make_float4(0.f, 0.f, 0.f, 0.f);
            const float cx = cp.x, cy = cp.y, dd = cp.z;
            const float wx = fmaf(T[0], cx, fmaf(T[1], cy, fmaf(T[2], dd, T[3])));
            const float wy = fmaf(T[4], cx, fmaf(T[5], cy, fmaf(T[6], dd, T[7])));
            const float wz = fmaf(T[8], cx, fmaf(T[9], cy, fmaf(T[10], dd, T[11])));
            const float qx = fmaf(Pi[0], wx, fmaf(Pi[1], wy, fmaf(Pi[2], wz, Pi[3])));
            const float qy = fmaf(Pi[4], wx, fmaf(Pi[5], wy, fmaf(Pi[6], wz, Pi[7])));
            const float qz = fmaf(Pi[8], wx, fmaf(Pi[9], wy, fmaf(Pi[10], wz, Pi[11])));
            wv[g][0] = wx;
            wv[g][1] = wy;
            wv[g][2] = wz;
            bool good = (cp.w != 0.f) && (qz > 1e-3f);
            int ii = 0, jj = 0;
            if (good) {
                const float rq = 1.f / qz;
                ii = (int)floorf(fmaf(qy * in.fy, rq, in.ci) + 0.5f);
                jj = (int)floorf(fmaf(qx * in.fx, rq, in.cj) + 0.5f);
                good = ii >= 0 && ii < rows && jj >= 0 && jj < cols;
            }
            ok[g] = good;
            const size_t mi = good ? (size_t)ii * cols + jj : 0;
            n[g] = good ? __ldg(nmap + mi) : make_float4(0.f, 0.f, 0.f, 0.f);
            v[g] = good ? __ldg(vmap + mi) : make_float4(0.f, 0.f, 0.f, 0.f);
        }
        float t[kTrackSums - 1];
#pragma unroll
        for (int q = 0; q < kTrackSums - 1; q++) t[q] = 0.f;
        bool any = false;
#pragma unroll
        for (int g = 0; g < kG; g++) {
            if (!ok[g]) continue;
            const float4 nn = n[g], vv = v[g];
            if (nn.x == 0.f && nn.y == 0.f && nn.z == 0.f) continue;
            const float wx = wv[g][0], wy = wv[g][1], wz = wv[g][2];
            const float ex = wx - vv.x, ey = wy - vv.y, ez = wz - vv.z;
            if (ex * ex + ey * ey + ez * ez > dist2) continue;
            const float r = nn.x * ex + nn.y * ey + nn.z * ez;
            const float J[6] = {wy * nn.z - wz * nn.y, wz * nn.x - wx * nn.z, wx * nn.y - wy * nn.x, nn.x, nn.y, nn.z};
            int q = 0;
#pragma unroll
            for (int a = 0; a < 6; a++)
#pragma unroll
                for (int b = a; b < 6; b++) t[q] = fmaf(J[a], J[b], t[q]), q++;
#pragma unroll
            for (int a = 0; a < 6; a++) t[21 + a] = fmaf(J[a], r, t[21 + a]);
            t[27] = fmaf(r, r, t[27]);
            s[28] += 1.f;  // counts stay exact far below 2^24
            any = true;
        }
        if (kG >= kCamCache) {  // the only group
#pragma unroll
            for (int q = 0; q < kTrackSums - 1; q++) s[q] = t[q];
        } else if (any) {
#pragma unroll
            for (int q = 0; q < kTrackSums - 1; q++) kahan_add(s[q], c[q], t[q]);
        }
    }
}

// Reduces the CTA's pairs: thread v < kTrackSums returns the CTA's pair of
// value v. Within a warp, a transpose-reduce (recursive halving): at offset o
// each lane keeps the half of its remaining values selected by lane bit o and
// trades the other half with lane ^ o, adding with TwoSum, so after offsets
// 16, 8, 4, 2, 1 lane l holds the warp's pair of value l (31 exchanges per
// lane instead of 5 per value). Warps then combine through shared memory by a
// fixed tree (eight warps: three additions deep).
__device__ __forceinline__ float2 track_cta_pairs(float *s, float *c, float2 (*red)[kTrackSums]) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    float vs[32], vc[32];
#pragma unroll
    for (int k = 0; k < 32; k++) {
        vs[k] = k < kTrackSums ? s[k] : 0.f;
        vc[k] = k < kTrackSums ? c[k] : 0.f;
    }
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) {
        const bool upper = (lane & o) != 0;
        if (o >= 2) {  // two values per step in paired instructions (the same roundings)
#pragma unroll
            for (int k = 0; k < o; k += 2) {
                float ss[2], sc[2], ks[2], kc[2], rs[2], rc[2];
#pragma unroll
                for (int u = 0; u < 2; u++) {
                    ss[u] = upper ? vs[k + u] : vs[k + u + o];
                    sc[u] = upper ? vc[k + u] : vc[k + u + o];
                    ks[u] = upper ? vs[k + u + o] : vs[k + u];
                    kc[u] = upper ? vc[k + u + o] : vc[k + u];
                    rs[u] = __shfl_xor_sync(0xffffffffu, ss[u], o);
                    rc[u] = __shfl_xor_sync(0xffffffffu, sc[u], o);
                }
                f32x2 ps = f2_pack(ks[0], ks[1]), pc = f2_pack(kc[0], kc[1]);
                pair_add2(ps, pc, f2_pack(rs[0], rs[1]), f2_pack(rc[0], rc[1]));
                f2_unpack(ps, vs[k], vs[k + 1]);
                f2_unpack(pc, vc[k], vc[k + 1]);
            }
        } else {
            const float ss = upper ? vs[0] : vs[1], sc = upper ? vc[0] : vc[1];
            float ks = upper ? vs[1] : vs[0], kc = upper ? vc[1] : vc[0];
            const float rs = __shfl_xor_sync(0xffffffffu, ss, 1), rc = __shfl_xor_sync(0xffffffffu, sc, 1);
            pair_add(ks, kc, rs, rc);
            vs[0] = ks;
            vc[0] = kc;
        }
    }
    if (lane < kTrackSums) red[wid][lane] = make_float2(vs[0], vc[0]);
    __syncthreads();
    float a = 0.f, b = 0.f;
    if (threadIdx.x < kTrackSums) {
        if (blockDim.x == 256) {  // the eight warps' pairs by a tree, three additions deep
            float2 p[8];
#pragma unroll
            for (int w = 0; w < 8; w++) p[w] = red[w][threadIdx.x];
#pragma unroll
            for (int st = 1; st < 8; st <<= 1)
#pragma unroll
                for (int w = 0; w < 8; w += 2 * st) pair_add(p[w].x, p[w].y, p[w + st].x, p[w + st].y);
            a = p[0].x;
            b = p[0].y;
        } else {
            for (int w = 0; w < (int)(blockDim.x >> 5); w++) pair_add(a, b, red[w][threadIdx.x].x, red[w][threadIdx.x].y);
        }
    }
    return make_float2(a, b);
}

// The CTA's pairs into the value-major slots: slots[value][cta].
__device__ __forceinline__ void track_cta_to_slots(float *s, float *c, float2 (*red)[kTrackSums],
                                                   float2 *__restrict__ slots) {
    const float2 p = track_cta_pairs(s, c, red);
    if (threadIdx.x < kTrackSums) slots[(size_t)threadIdx.x * gridDim.x + blockIdx.x] = p;
}

// Cross-CTA sums of the persistent tracker in fixed point: each CTA's pair
// (sum - compensation) is converted exactly, up to a resolution of
// 2^-kTrackFixShift, to a signed integer below 2^96 in magnitude, split into
// three 32-bit chunks (two unsigned, the top one signed) and added with
// 64-bit integer atomics, so the total is exact and does not depend on the
// order in which CTAs arrive (the pose is bit-reproducible). A CTA value of
// magnitude >= 2^47 (or NaN) is not added; it counts in the overflow word
// (value kTrackSums) instead, and the iteration keeps its pose.
//
// Each atomic also adds 2^48, so every word counts its own contributions
// and no separate grid barrier is needed: a reader waits until each of its
// words has grown by gridDim.x contributions since it last read that buffer
// (a CTA's chunks add less than 2^41 per use, so the count field is exact).
// The words only grow during a frame (wrapping mod 2^64); readers take the
// difference to the value they read at the buffer's previous use. That is
// safe with three buffers in rotation: a CTA adds to iteration k + 3's use
// of a buffer only after it has read iteration k + 2, which needs every
// CTA's iteration-(k + 2) contribution, which each CTA makes only after it
// has read iteration k. The last CTA to leave zeroes the words for the next
// frame.
constexpr int kTrackFixShift = 48;
constexpr double kTrackFixUnit = (double)(1ull << kTrackFixShift);  // 1.0 in accumulator units
constexpr int kTrackCountShift = 48;
constexpr unsigned long long kTrackCountOne = 1ull << kTrackCountShift;

// f 2^kTrackFixShift truncated toward zero, for |f| < 2^47; false otherwise.
__device__ __forceinline__ bool fixed_of_float(float f, __int128 &q) {
    if (!(fabsf(f) < 0x1p47f)) return false;
    const unsigned u = __float_as_uint(f);
    const int ex = (int)((u >> 23) & 0xffu);
    if (ex == 0) {  // zero or subnormal: below the resolution
        q = 0;
        return true;
    }
    const unsigned long long m = (u & 0x7fffffu) | 0x800000u;  // f = m 2^(ex - 150)
    const int sh = ex - 150 + kTrackFixShift;                  // <= 71: m 2^sh < 2^95
    __int128 mag = 0;
    if (sh >= 0)
        mag = (__int128)m << sh;
    else if (sh > -24)
        mag = (__int128)(m >> -sh);
    q = (u >> 31) ? -mag : mag;
    return true;
}

// The CTA's totals into the counted words of one buffer: lane v < kTrackSums
// of warp 0 adds value v, lane kTrackSums the CTA's overflow count; every
// one of the buffer's words receives exactly one atomic per CTA.
__device__ __forceinline__ void track_cta_to_acc(float *s, float *c, float2 (*red)[kTrackSums],
                                                 unsigned long long *__restrict__ acc) {
    const float2 p = track_cta_pairs(s, c, red);
    if (threadIdx.x < 32) {
        const int v = threadIdx.x;
        __int128 qs = 0, qc = 0;
        const bool ok = v < kTrackSums && fixed_of_float(p.x, qs) && fixed_of_float(p.y, qc);
        const unsigned bad = __ballot_sync(0xffffffffu, v < kTrackSums && !ok);
        if (v < kTrackAccValues) {
            unsigned long long c0 = 0, c1 = 0, c2 = 0;
            if (ok) {
                const __int128 q = qs - qc;
                c0 = (unsigned long long)q & 0xffffffffull;
                c1 = (unsigned long long)(q >> 32) & 0xffffffffull;
                c2 = (unsigned long long)(long long)(q >> 64);
            }
            if (v == kTrackSums) c0 = (unsigned long long)__popc(bad);
            unsigned long long *w = acc + (size_t)v * kTrackAccChunks * kTrackAccStride;
            atomicAdd(w, c0 + kTrackCountOne);
            atomicAdd(w + kTrackAccStride, c1 + kTrackCountOne);
            atomicAdd(w + 2 * kTrackAccStride, c2 + kTrackCountOne);
        }
    }
}

// t rounded to the nearest double (ties to even), by integer operations (the
// FP64 pipe's conversions cost as much latency as an FMA); |t| < 2^127.
__device__ __forceinline__ double f64_rn_of_i128(__int128 t) {
    if (t == 0) return 0.0;
    const bool neg = t < 0;
    unsigned __int128 m = neg ? (unsigned __int128)(-t) : (unsigned __int128)t;
    const unsigned long long mh = (unsigned long long)(m >> 64), ml = (unsigned long long)m;
    const int lz = mh ? __clzll((long long)mh) : 64 + __clzll((long long)ml);
    m <<= lz;  // the leading one at bit 127
    const unsigned long long th = (unsigned long long)(m >> 64), tl = (unsigned long long)m;
    unsigned long long mant = th >> 11;  // 53 bits
    int ex = 127 - lz + 1023;
    if (((th >> 10) & 1ull) && ((th & 0x3ffull) || tl || (mant & 1ull))) {
        if (++mant >> 53) {
            mant >>= 1;
            ex++;
        }
    }
    return __longlong_as_double((long long)((neg ? 0x8000000000000000ull : 0ull) | ((unsigned long long)ex << 52) |
                                            (mant & 0xfffffffffffffull)));
}

__device__ __forceinline__ unsigned long long ld_relaxed_u64(const unsigned long long *p) {
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

// Warp 0: waits until all words of a buffer hold gridDim.x (+ extra) new
// contributions (relaxed loads, back-off, at most `polls` polls: 2^22 by
// default, about a second), then returns
// in lane v < kTrackAccValues value v of this use in FP64, in units of
// 2^-kTrackFixShift (the chunk increments recombined exactly into a 128-bit
// integer, then rounded once to the nearest double). prev: the buffer's 90 words as read
// at its previous use (shared), updated here. False on timeout.
__device__ __forceinline__ bool track_acc_wait(const unsigned long long *__restrict__ acc, unsigned long long *prev,
                                               double &value, int polls, int extra) {
    const int v = threadIdx.x & 31;
    const bool mine = v < kTrackAccValues;
    const unsigned long long *w = acc + (size_t)(mine ? v : 0) * kTrackAccChunks * kTrackAccStride;
    const unsigned long long p0 = mine ? prev[3 * v] : 0ull, p1 = mine ? prev[3 * v + 1] : 0ull,
                             p2 = mine ? prev[3 * v + 2] : 0ull;
    const unsigned long long want = (unsigned long long)gridDim.x + (unsigned long long)extra;
    unsigned long long w0 = 0, w1 = 0, w2 = 0;
    bool done = false;
    int spins = 0;
    do {
        if (mine) {
            w0 = ld_relaxed_u64(w);
            w1 = ld_relaxed_u64(w + kTrackAccStride);
            w2 = ld_relaxed_u64(w + 2 * kTrackAccStride);
        }
        const unsigned long long half = 1ull << (kTrackCountShift - 1);
        const bool complete = !mine || (((w0 - p0 + half) >> kTrackCountShift) == want &&
                                        ((w1 - p1 + half) >> kTrackCountShift) == want &&
                                        ((w2 - p2 + half) >> kTrackCountShift) == want);
        done = __all_sync(0xffffffffu, complete);
        if (done) break;
        __nanosleep(32);
    } while (++spins < polls);
    if (!done) return false;
    value = 0.0;
    if (mine) {
        prev[3 * v] = w0;
        prev[3 * v + 1] = w1;
        prev[3 * v + 2] = w2;
        const unsigned long long counted = want << kTrackCountShift;
        const long long s0 = (long long)(w0 - p0 - counted), s1 = (long long)(w1 - p1 - counted),
                        s2 = (long long)(w2 - p2 - counted);
        const __int128 t = (__int128)s2 * ((__int128)1 << 64) + (__int128)s1 * ((__int128)1 << 32) + (__int128)s0;
        value = f64_rn_of_i128(t);
    }
    return true;
}

// Reduces all CTA slots into (sum, compensation) pairs, TwoSum in FP32 in a
// fixed order: warp w takes values w, w + 8, w + 16, w + 24 (256 threads), each
// lane a strided share of the CTAs. The loads of up to kSlotChunks x 32 CTAs
// are all issued before the first addition (one L2 round trip).
constexpr int kSlotChunks = 8;

__device__ __forceinline__ void track_slots_to_pairs(const float2 *__restrict__ slots, float2 *tot) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    constexpr int kPer = (kTrackSums + 7) / 8;
    const unsigned n = gridDim.x;
    float a[kPer], b[kPer];
#pragma unroll
    for (int u = 0; u < kPer; u++) a[u] = b[u] = 0.f;
    for (unsigned q0 = 0; q0 < n; q0 += 32u * kSlotChunks) {
        float2 p[kSlotChunks][kPer];
#pragma unroll
        for (int ch = 0; ch < kSlotChunks; ch++) {
            const unsigned q = q0 + lane + 32u * ch;
#pragma unroll
            for (int u = 0; u < kPer; u++) {
                const int v = wid + 8 * u;
                p[ch][u] = (q < n && v < kTrackSums) ? __ldcg(slots + (size_t)v * n + q) : make_float2(0.f, 0.f);
            }
        }
#pragma unroll
        for (int ch = 0; ch < kSlotChunks; ch++)
#pragma unroll
            for (int u = 0; u < kPer; u++) pair_add(a[u], b[u], p[ch][u].x, p[ch][u].y);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
        for (int u = 0; u < kPer; u++) {
            const float a2 = __shfl_down_sync(0xffffffffu, a[u], o), b2 = __shfl_down_sync(0xffffffffu, b[u], o);
            pair_add(a[u], b[u], a2, b2);
        }
    }
    if (lane == 0) {
#pragma unroll
        for (int u = 0; u < kPer; u++)
            if (wid + 8 * u < kTrackSums) tot[wid + 8 * u] = make_float2(a[u], b[u]);
    }
}

// Value of a (sum, compensation) pair.
__device__ __forceinline__ float pair_value(float2 p) { return p.x - p.y; }

__global__ void __launch_bounds__(256) track_iter_kernel(const uint16_t *__restrict__ depth, int rows, int cols,
                                                         Intr in, const float4 *__restrict__ vmap,
                                                         const float4 *__restrict__ nmap, TrackState *st,
                                                         float2 *__restrict__ partials, int level, float dist2,
                                                         float rmin, float dmax) {
    if (*(volatile int *)&st->converged_level == level) return;
    __shared__ float2 red[8][kTrackSums];
    __shared__ bool last;
    __shared__ float2 tot[kTrackSums];
    float T[12], Pi[12];
#pragma unroll
    for (int k = 0; k < 12; k++) {
        T[k] = st->Tf[k];
        Pi[k] = st->Tprev_inv[k];
    }
    float s[kTrackSums], c[kTrackSums];
#pragma unroll
    for (int k = 0; k < kTrackSums; k++) s[k] = c[k] = 0.f;
    track_accumulate(depth, rows, cols, in, vmap, nmap, T, Pi, level, dist2, rmin, dmax,
                     blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x, s, c);
    track_cta_to_slots(s, c, red, partials);
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = atomicAdd(&st->ticket, 1) == (int)gridDim.x - 1;
    __syncthreads();
    if (!last) return;
    __threadfence();
    // last CTA: reduce the slots, then one warp solves in FP64
    track_slots_to_pairs(partials, tot);
    __syncthreads();
    const float n = pair_value(tot[28]);
    if (threadIdx.x < 32) {
        if (threadIdx.x == 0) st->ticket = 0;
        double x[6];
        if (n >= 60.f && warp_solve6(tot, x)) {  // too few correspondences: keep the pose
            const float step2 = warp_se3_left_update(x, st->T, st->T, st->Tf);
            if (threadIdx.x == 0 && step2 < 1e-14f) st->converged_level = level;
        }
    } else if (threadIdx.x == 32) {
        st->inliers[level] = (int)n;
        st->rmse[level] = n > 0.f ? sqrtf(fmaxf(pair_value(tot[27]), 0.f) / n) : 0.f;
    }
}

#ifdef SS_TRACK_TIMING
// Phase timestamps of CTA 0 (global timer, ns) for tuning builds only.
__device__ unsigned long long g_track_timing[32 * 8];
#define SS_TT(slot, phase)                                                                     \
    do {                                                                                       \
        if (blockIdx.x == 0 && threadIdx.x == 0 && (slot) < 32) {                              \
            unsigned long long t_;                                                             \
            asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t_));                             \
            g_track_timing[(slot) * 8 + (phase)] = t_;                                         \
        }                                                                                      \
    } while (0)
// Every CTA's arrival at (kind 0) and departure from (kind 1) each barrier.
constexpr int kTimingCtas = 512;
__device__ unsigned long long g_track_cta_timing[2 * 32 * kTimingCtas];
#define SS_TC(slot, kind)                                                                                  \
    do {                                                                                                   \
        if (threadIdx.x == 0 && (slot) < 32 && blockIdx.x < kTimingCtas) {                                 \
            unsigned long long t_;                                                                         \
            asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t_));                                         \
            g_track_cta_timing[((kind) * 32 + (slot)) * kTimingCtas + blockIdx.x] = t_;                    \
        }                                                                                                  \
    } while (0)
#else
#define SS_TT(slot, phase) \
    do {                   \
    } while (0)
#define SS_TC(slot, kind) \
    do {                  \
    } while (0)
#endif

// Rigid inverse of T (FP64) as floats by one warp: lanes 0..11 write Ti[lane].
__device__ __forceinline__ void warp_rigid_inverse_f(const double *T, float *Ti) {
    const int lane = threadIdx.x & 31;
    if (lane < 12) {
        const int r = lane >> 2, c = lane & 3;
        Ti[lane] = c < 3 ? (float)T[c * 4 + r] : (float)(-(T[r] * T[3] + T[4 + r] * T[7] + T[8 + r] * T[11]));
    }
}

// All Gauss-Newton iterations of one frame in one cooperative launch, with
// the frame's start (model pose = current pose, its inverse; ICP start = the
// one-shot start pose or the model pose) and end (the FramePose of the result
// for integrate and raycast) folded in. Each CTA adds its sums to the
// counted fixed-point accumulators of the iteration (three buffers in
// rotation); warp 0 of every CTA waits until the iteration's words are
// complete, reads the totals and solves redundantly (bit-identical results
// in every CTA), so no other grid-wide synchronisation is needed. Every CTA
// leaves through the same exit, also after a wait timeout; the last one to
// leave zeroes the accumulators for the next frame.
__global__ void __launch_bounds__(256) track_frame_kernel(const uint16_t *__restrict__ depth, int rows, int cols,
                                                          Intr in, const float4 *__restrict__ vmap,
                                                          const float4 *__restrict__ nmap, TrackState *st,
                                                          unsigned long long *__restrict__ acc, TrackLaunch L) {
    __shared__ float2 red[8][kTrackSums];
    __shared__ int last_out;
    __shared__ double Td[16];
    __shared__ float Tf[12], Pi[12];
    __shared__ int done_level, abort_run;
    __shared__ unsigned long long prevw[kTrackAccBuffers][kTrackAccValues * kTrackAccChunks];
    __shared__ float4 cam[kCamCache][256];
    if (threadIdx.x < 16) Td[threadIdx.x] = st->T[threadIdx.x];
    if (threadIdx.x == 0) {
        done_level = -1;
        abort_run = 0;
    }
    for (int w = threadIdx.x; w < kTrackAccBuffers * kTrackAccValues * kTrackAccChunks; w += blockDim.x)
        (&prevw[0][0])[w] = 0ull;  // the words are zero at the start of a frame
    __syncthreads();
    if (threadIdx.x < 32) {
        // the model maps were raycast at the current pose: Tprev = T
        warp_rigid_inverse_f(Td, Pi);
        if (blockIdx.x == 0) {
            if (threadIdx.x < 16) st->Tprev[threadIdx.x] = Td[threadIdx.x];
            if (threadIdx.x < 12) st->Tprev_inv[threadIdx.x] = Pi[threadIdx.x];
            if (threadIdx.x < kMaxLevels) {
                st->inliers[threadIdx.x] = 0;
                st->rmse[threadIdx.x] = 0.f;
            }
        }
    }
    __syncthreads();
    // ICP start: the one-shot start pose when set (read by every CTA before its
    // first barrier arrival; the last CTA to leave clears it), else the model pose
    if (*(volatile int *)&st->has_start && threadIdx.x < 16) Td[threadIdx.x] = st->Tstart[threadIdx.x];
    __syncthreads();
    if (threadIdx.x < 12) Tf[threadIdx.x] = (float)Td[threadIdx.x];
    __syncthreads();
    unsigned barriers = 0;
    int abuf = 0;  // accumulator buffer of this iteration
    bool alive = true;
    const int tid = blockIdx.x * blockDim.x + threadIdx.x, nthreads = gridDim.x * blockDim.x;
    for (int level = L.levels - 1; level >= 0 && alive; level--) {
        const float dist2 = L.dist[level] * L.dist[level];
        const int npix = ((rows + (1 << level) - 1) >> level) * ((cols + (1 << level) - 1) >> level);
        const int m_count = (npix + nthreads - 1) / nthreads;
        const bool cached = m_count <= kCamCache;  // else the points are recomputed every iteration
        if (cached) track_fill_cam(depth, rows, cols, in, level, L.rmin, L.dmax, tid, nthreads, m_count, cam);
        for (int it = 0; it < L.iters[level]; it++) {
            if (done_level == level) break;  // converged: identical decision in every CTA
            SS_TT(barriers, 0);
            float s[kTrackSums], c[kTrackSums];
#pragma unroll
            for (int k = 0; k < kTrackSums; k++) s[k] = c[k] = 0.f;
            float T[12], P[12];
#pragma unroll
            for (int k = 0; k < 12; k++) {
                T[k] = Tf[k];
                P[k] = Pi[k];
            }
            if (cached)
                if (m_count > kTrackGroup)
                    track_accumulate_cam<kCamCache>(cam, m_count, rows, cols, in, vmap, nmap, T, P, dist2, s, c);
                else
                    track_accumulate_cam<kTrackGroup>(cam, m_count, rows, cols, in, vmap, nmap, T, P, dist2, s, c);
            else
                track_accumulate(depth, rows, cols, in, vmap, nmap, T, P, level, dist2, L.rmin, L.dmax, tid, nthreads,
                                 s, c);
            SS_TT(barriers, 1);
            unsigned long long *buf = acc + (size_t)abuf * kTrackAccBufWords;
            track_cta_to_acc(s, c, red, buf);
            SS_TT(barriers, 2);
            SS_TC(barriers, 0);
            barriers++;
            double v = 0.0;
            if (threadIdx.x < 32 && !track_acc_wait(buf, prevw[abuf], v, L.wait_polls, L.wait_extra)) {
                if (threadIdx.x == 0) {
                    abort_run = 1;
                    atomicOr(&st->status, kStTimeout);
                    if (L.grid_status) atomicOr(L.grid_status, kStTimeout);
                }
            } else if (threadIdx.x < 32) {
                SS_TT(barriers - 1, 3);
                SS_TC(barriers - 1, 1);
                const int lane = threadIdx.x;
                // sums in units of 2^-48: the solve is invariant under that common
                // power-of-two scale, so only the thresholds are scaled
                const double n = __shfl_sync(0xffffffffu, v, kTrackSums - 1);
                const double r2 = __shfl_sync(0xffffffffu, v, kTrackSums - 2);
                const double of = __shfl_sync(0xffffffffu, v, kTrackSums);
                SS_TT(barriers - 1, 4);
                double x[6];
                // too few correspondences, or a sum out of range: keep the pose
                if (above_pos(n, 59.5 * kTrackFixUnit) && __double_as_longlong(of) == 0 &&
                    warp_solve6_lanes(v, x, kPivotMin * kTrackFixUnit)) {
                    SS_TT(barriers - 1, 6);
                    const float step2 = warp_se3_left_update(x, Td, Td, Tf);
                    if (lane == 0 && step2 < 1e-14f) done_level = level;
                    SS_TT(barriers - 1, 7);
                }
                if (blockIdx.x == 0 && lane == 0) {
                    const float nf = (float)n;  // exact: a count below 2^24 times 2^48
                    st->inliers[level] = (int)(nf * (float)(1.0 / kTrackFixUnit));
                    st->rmse[level] = nf > 0.f ? sqrtf(fmaxf((float)r2, 0.f) / nf) : 0.f;
                }
            }
            __syncthreads();
            SS_TT(barriers - 1, 5);
            if (abort_run) {
                alive = false;
                break;
            }
            abuf = abuf == kTrackAccBuffers - 1 ? 0 : abuf + 1;
        }
    }
    pdl_trigger();  // the collection may launch; it waits for this grid before it reads the pose
    if (blockIdx.x == 0 && threadIdx.x < 32) {
        // the result and its FramePose (float pose, float inverse, unit z column)
        const int lane = threadIdx.x;
        if (lane < 16) st->T[lane] = Td[lane];
        if (lane < 12) {
            st->Tf[lane] = Tf[lane];
            st->pose.E.m[lane] = (float)Td[lane];
        }
        warp_rigid_inverse_f(Td, st->pose.Einv.m);
        const float ex = (float)Td[2], ey = (float)Td[6], ez = (float)Td[10];
        const float len = sqrtf(ex * ex + ey * ey + ez * ez);
        if (lane == 0) {
            st->pose.Ez[0] = ex / len;
            st->pose.Ez[1] = ey / len;
            st->pose.Ez[2] = ez / len;
            st->pose.pad = 0.f;
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        last_out = atomicAdd(&st->exits, 1u) == gridDim.x - 1;
        if (last_out) {
            st->barrier = 0u;
            st->exits = 0u;
            st->has_start = 0;
        }
    }
    __syncthreads();
    if (last_out)  // every other CTA has finished its reads
        for (int w = threadIdx.x; w < kTrackAccBuffers * kTrackAccValues * kTrackAccChunks; w += blockDim.x)
            acc[(size_t)w * kTrackAccStride] = 0ull;
}

#ifdef SS_TRACK_TIMING
extern "C" int ss_debug_track_timing(unsigned long long *out) {
    return (int)cudaMemcpyFromSymbol(out, g_track_timing, sizeof(g_track_timing));
}
extern "C" int ss_debug_track_cta_timing(unsigned long long *out) {
    return (int)cudaMemcpyFromSymbol(out, g_track_cta_timing, sizeof(g_track_cta_timing));
}
#endif

int persistent_track_ctas(int num_sms, int want_per_sm) {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, track_frame_kernel, 256, 0) != cudaSuccess) {
        cudaGetLastError();
        per_sm = 1;
    }
    if (per_sm > want_per_sm) per_sm = want_per_sm;
    return num_sms * (per_sm < 1 ? 1 : per_sm);
}

// Host-side launch of one frame's tracking: one cooperative launch, or begin,
// one launch per iteration (levels coarse to fine), then the FramePose of the
// result.
ss_status launch_track(const TrackLaunch &L, cudaStream_t s) {
    if (L.persistent) {
        const uint16_t *depth = L.depth;
        int rows = L.rows, cols = L.cols;
        Intr in = L.in;
        const float4 *vmap = L.vmap, *nmap = L.nmap;
        TrackState *st = L.state;
        unsigned long long *acc = L.acc;
        // cooperative launch (all CTAs co-resident, so the grid barrier cannot wait
        // on a CTA that is not running); the attribute form is stream-capturable
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(L.ctas);
        cfg.blockDim = dim3(256);
        cfg.dynamicSmemBytes = 0;
        cfg.stream = s;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeCooperative;
        attr[0].val.cooperative = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        SS_CUDA_TRY(cudaLaunchKernelEx(&cfg, track_frame_kernel, depth, rows, cols, in, vmap, nmap, st, acc, L));
        return SS_OK;
    }
    track_begin_kernel<<<1, 32, 0, s>>>(L.state);
    SS_LAUNCH_CHECK();
    for (int level = L.levels - 1; level >= 0; level--) {
        for (int it = 0; it < L.iters[level]; it++) {
            track_iter_kernel<<<L.ctas, 256, 0, s>>>(L.depth, L.rows, L.cols, L.in, L.vmap, L.nmap, L.state, L.partials,
                                                     level, L.dist[level] * L.dist[level], L.rmin, L.dmax);
            SS_LAUNCH_CHECK();
        }
    }
    pose_prep_kernel<<<1, 32, 0, s>>>(L.state);
    SS_LAUNCH_CHECK();
    return SS_OK;
}

ss_status launch_pose_prep(TrackState *st, cudaStream_t s) {
    pose_prep_kernel<<<1, 32, 0, s>>>(st);
    SS_LAUNCH_CHECK();
    return SS_OK;
}

// The pose (16 doubles) stored through a device-mapped pointer (pinned host
// memory): a per-frame readback without a copy-engine transfer.
__global__ void pose_out_kernel(const TrackState *st, double *dst) {
    if (threadIdx.x < 16) dst[threadIdx.x] = st->T[threadIdx.x];
}

ss_status launch_pose_out(const TrackState *st, double *dst, cudaStream_t s) {
    pose_out_kernel<<<1, 32, 0, s>>>(st, dst);
    SS_LAUNCH_CHECK();
    return SS_OK;
}

}  // namespace ss
