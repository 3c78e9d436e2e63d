// ss_track_solve.cuh — FP64 solve of the tracker's 6x6 normal equations and
// the SE(3) pose update, by one warp.
//
// On this part an FP64 warp instruction occupies its SM sub-partition's FP64
// pipe for ~64 cycles whether one lane or 32 are active, so a one-thread solve
// costs ~64 cycles per FP64 operation (~140 operations for a Cholesky solve
// with square roots, ~130 more for the SE(3) exponential and pose product).
// Here every lane owns one entry, so each step of the elimination and of the
// pose update is one or two warp instructions, and no square root is taken:
//
// * elimination: Gauss-Jordan elimination without pivoting on the augmented
//   upper triangle [A | b] (27 lanes). The pivots are those of the
//   square-root-free (LDL^T) form of Cholesky (row k of the trailing matrix
//   is updated exactly as in LDL^T, and the trailing matrix stays symmetric,
//   so a_ik = a_ki serves the rows below the pivot); the rows above the pivot
//   are cleared too, so no back substitution is needed. Each step updates
//   every other row in fraction-free form, a_ij <- p' a_ij - a_ik (a_kj 2^-e),
//   rounded as fma(-a_ik, a_kj 2^-e, RN(p' a_ij)),
//   with the pivot p = p' 2^e split exactly into p' in [1, 2) and a power of
//   two by integer operations: each row is scaled by a factor in [1, 2) per
//   step, and no division sits on the elimination's critical path;
// * x_i = c_i / u_ii with the reciprocals of the six pivots computed
//   together: an FP32 seed refined by two Newton-Raphson steps in FP64
//   (r <- r + r (1 - m r); the relative error squares each step, 2^-23 ->
//   2^-46 -> below FP64 rounding);
// * SE(3) exponential by Maclaurin series of sin t / t, (1 - cos t) / t^2,
//   (t - sin t) / t^3 (one series per lane, as many terms as th2 needs), and
//   the pose product R T + V upsilon from one set of lane-parallel dot
//   products (K T, omega^T T, K upsilon, ...), one entry per lane.
#pragma once

#include <cuda_runtime.h>

namespace ss {

constexpr int kAugLanes = 27;  // entries (i, j) of [A | b], 0 <= i <= j <= 6, i < 6
constexpr double kPivotMin = 1e-12;

// lane of entry (i, j) of the augmented upper triangle (rows of 7, 6, ..., 2)
__device__ __forceinline__ int aug_lane(int i, int j) { return 7 * i - ((i * (i - 1)) >> 1) + (j - i); }

// entry (i, j) of lane (lanes >= kAugLanes get j > 6)
__device__ __forceinline__ void aug_entry(int lane, int &i, int &j) {
    i = 0;
#pragma unroll
    for (int r = 1; r < 6; r++)
        if (lane >= aug_lane(r, r)) i = r;
    j = i + (lane - aug_lane(i, i));
}

// x = m 2^e with m in [1, 2) (sign kept), for finite normal x; integer operations only.
__device__ __forceinline__ double split_pow2(double x, int &e) {
    const int hi = __double2hiint(x), lo = __double2loint(x);
    e = ((hi >> 20) & 0x7ff) - 1023;
    return __hiloint2double((hi & 0x800fffff) | 0x3ff00000, lo);
}

// x 2^-e, exact by exponent arithmetic (zero and subnormal inputs, and
// results below the normal range, give zero).
__device__ __forceinline__ double scale_pow2(double x, int e) {
    const int hi = __double2hiint(x), lo = __double2loint(x);
    const int ex = (hi >> 20) & 0x7ff;
    const int nx = ex - e;
    if (ex == 0 || nx <= 0) return 0.0;
    if (nx >= 0x7ff) return __hiloint2double((hi & 0x80000000) | 0x7ff00000, 0);
    return __hiloint2double((hi & 0x800fffff) | (nx << 20), lo);
}

// Conversions by integer operations, off the FP64 pipe (whose conversion
// instructions cost as much latency as an FMA): m in [1, 2) to the float of
// its leading 23 mantissa bits (truncated), and a normal float to its exact
// double.
__device__ __forceinline__ float f32_of_unit_mantissa(double m) {
    const unsigned hi = (unsigned)__double2hiint(m), lo = (unsigned)__double2loint(m);
    return __uint_as_float(0x3f800000u | ((hi & 0xfffffu) << 3) | (lo >> 29));
}
__device__ __forceinline__ double f64_of_normal_f32(float f) {
    const unsigned u = __float_as_uint(f);
    const unsigned hi = (u & 0x80000000u) | ((((u >> 23) & 0xffu) + 896u) << 20) | ((u & 0x7fffffu) >> 3);
    return __hiloint2double((int)hi, (int)(u << 29));
}

// (float)d, rounded to nearest even, by integer operations where the result
// is a normal float (other values: the conversion instruction).
__device__ __forceinline__ float f32_rn_of_f64(double d) {
    const unsigned hi = (unsigned)__double2hiint(d), lo = (unsigned)__double2loint(d);
    const int e = (int)((hi >> 20) & 0x7ffu) - 1023;
    if (e < -126 || e > 127) return (float)d;
    const unsigned top = ((hi & 0xfffffu) << 3) | (lo >> 29), rest = lo & 0x1fffffffu;
    unsigned bits = ((unsigned)(e + 127) << 23) | top;
    if (rest > 0x10000000u || (rest == 0x10000000u && (top & 1u))) bits += 1u;  // a carry moves into the exponent
    return __uint_as_float(bits | (hi & 0x80000000u));
}

// 1 / x for finite normal x > 0: FP32 seed on the mantissa, two Newton-Raphson steps in FP64.
__device__ __forceinline__ double rcp_pos(double x) {
    int e;
    const double m = split_pow2(x, e);
    float sf;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(sf) : "f"(f32_of_unit_mantissa(m)));
    double r = f64_of_normal_f32(sf);  // sf in [0.5, 1]
    double t = fma(-m, r, 1.0);
    r = fma(r, t, r);
    t = fma(-m, r, 1.0);
    r = fma(r, t, r);
    return scale_pow2(r, e);
}

// Index q of the normal-equation sum behind this lane's entry (i, j) of
// [A | b]: 0..20 the upper triangle of A row-major, 21..26 J^T r.
__device__ __forceinline__ int aug_sum_index(int i, int j) {
    return (j < 6) ? 6 * i - ((i * (i - 1)) >> 1) + (j - i) : 21 + i;
}

// Gauss-Jordan core: lane (i, j) < kAugLanes holds entry (i, j) of [A | b]
// in a (b = -J^T r), other lanes 0. A pivot must exceed pivot_min.
__device__ __forceinline__ bool warp_solve6_aug(double a, double x[6], double pivot_min = kPivotMin);

// x > y for y >= 0 finite, x not NaN or +inf (false for those), by integer
// comparison of the bit patterns (which order like the values for x, y >= 0;
// negative x has the sign bit and compares below): no FP64 instruction.
__device__ __forceinline__ bool above_pos(double x, double y) {
    const long long bx = __double_as_longlong(x);
    return bx > __double_as_longlong(y) && bx < 0x7ff0000000000000ll;
}

// Solves A x = b in FP64 with the calling warp (all 32 lanes, converged).
// pairs[0..20]: the upper triangle of A row-major, pairs[21..26]: J^T r (b = -J^T r),
// each an FP32 (sum, compensation) pair with value sum - compensation.
// Every lane returns the same x and the same verdict (false: a pivot <= kPivotMin).
__device__ __forceinline__ bool warp_solve6(const float2 *pairs, double x[6]) {
    const int lane = threadIdx.x & 31;
    int i, j;
    aug_entry(lane, i, j);
    double a = 0.0;
    if (lane < kAugLanes) {
        const float2 p = pairs[aug_sum_index(i, j)];
        a = (double)p.x - (double)p.y;
        if (j == 6) a = -a;
    }
    return warp_solve6_aug(a, x);
}

// The same with the sums already in FP64, lane q < 27 of the warp holding sum
// q, all of them scaled by one power of two 2^s: the elimination's pivot
// splits, row scalings and reciprocals are exact under such a scaling, so x
// comes out bit for bit as for the unscaled sums when pivot_min is scaled too.
__device__ __forceinline__ bool warp_solve6_lanes(double sum, double x[6], double pivot_min = kPivotMin) {
    const int lane = threadIdx.x & 31;
    int i, j;
    aug_entry(lane, i, j);
    const bool live = lane < kAugLanes;
    double a = __shfl_sync(0xffffffffu, sum, live ? aug_sum_index(i, j) : 0);
    if (!live) a = 0.0;
    if (j == 6) a = -a;
    return warp_solve6_aug(a, x, pivot_min);
}

__device__ __forceinline__ bool warp_solve6_aug(double a, double x[6], double pivot_min) {
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    int i, j;
    aug_entry(lane, i, j);
    const bool live = lane < kAugLanes;
    bool ok = true;
#pragma unroll
    for (int k = 0; k < 6; k++) {
        const double p = __shfl_sync(full, a, aug_lane(k, k));
        ok = ok && above_pos(p, pivot_min);
        int e;
        const double ph = split_pow2(p, e);
        const bool upd = live && i != k;
        const double ahat = (live && i == k) ? scale_pow2(a, e) : a;  // row k times 2^-e
        // a_ik of this lane's row (upper triangle: (i, k) above the pivot, (k, i) below)
        const double aik = __shfl_sync(full, a, !upd ? 0 : (i < k ? aug_lane(i, k) : aug_lane(k, i)));
        // a_kj 2^-e of this lane's column (columns left of the pivot are cleared: 0)
        const double akj = __shfl_sync(full, ahat, (upd && j >= k) ? aug_lane(k, j) : 0);
        // ph a needs only the pivot, so it overlaps the shuffles of a_kj
        if (upd) a = fma(-aik, j >= k ? akj : 0.0, ph * a);
    }
    // row i is now u_ii x_i = c_i: reciprocals on the diagonal lanes, x_i on lanes (i, 6)
    const bool diag = live && i == j;
    const double r = rcp_pos(diag && above_pos(a, pivot_min) ? a : 1.0);
    const bool rhs = live && j == 6;
    const double rii = __shfl_sync(full, r, rhs ? aug_lane(i, i) : 0);
    const double xl = a * rii;
#pragma unroll
    for (int k = 0; k < 6; k++) x[k] = __shfl_sync(full, xl, aug_lane(k, 6));
    return ok;
}

// Series coefficient s of the SE(3) exponential at th2 = |omega|^2:
// s = 0: A = sin t / t, 1: B = (1 - cos t) / t^2, 2: C = (t - sin t) / t^3.
// Maclaurin series cut where the first omitted term of A (the largest of
// the three) is below 1e-17: 2 terms for th2 < 3.4e-8, 3 below 3.7e-5, 4
// below 1.38e-3, 5 below 2.5e-3; sin and cos beyond. Each branch also
// evaluates the caller's independent product k2 = fma(p, q, -(th2 y)) so that
// its FP64 instructions overlap the series' dependent chain.
__device__ __forceinline__ double se3_series(int s, double th2, double p, double q, double y, double &k2) {
    const double c4 = s == 0 ? 1.0 / 362880 : (s == 1 ? 1.0 / 3628800 : 1.0 / 39916800);
    const double c3 = s == 0 ? -1.0 / 5040 : (s == 1 ? -1.0 / 40320 : -1.0 / 362880);
    const double c2 = s == 0 ? 1.0 / 120 : (s == 1 ? 1.0 / 720 : 1.0 / 5040);
    const double c1 = s == 0 ? -1.0 / 6 : (s == 1 ? -1.0 / 24 : -1.0 / 120);
    const double c0 = s == 0 ? 1.0 : (s == 1 ? 0.5 : 1.0 / 6);
    if (!above_pos(th2, 3.4e-8)) {
        k2 = fma(p, q, -(th2 * y));
        return fma(c1, th2, c0);
    }
    if (!above_pos(th2, 3.7e-5)) {
        k2 = fma(p, q, -(th2 * y));
        return fma(fma(c2, th2, c1), th2, c0);
    }
    if (!above_pos(th2, 1.38e-3)) {
        k2 = fma(p, q, -(th2 * y));
        return fma(fma(fma(c3, th2, c2), th2, c1), th2, c0);
    }
    k2 = fma(p, q, -(th2 * y));
    if (!above_pos(th2, 0.0025)) return fma(fma(fma(fma(c4, th2, c3), th2, c2), th2, c1), th2, c0);
    const double th = sqrt(th2), sn = sin(th), cs = cos(th);
    return s == 0 ? sn / th : (s == 1 ? (1.0 - cs) / th2 : (th - sn) / (th2 * th));
}

// T <- exp(xi) T (left increment, xi = (omega, upsilon)) in FP64 with the calling
// warp. Tin: 12 doubles (rows of [R | t]); Tout (12 doubles) and Tfout (12 floats)
// are written by lanes 0..11 and may alias Tin only if the caller syncs the warp
// before reading them. Returns |xi|^2 (FP32, every lane).
//
// With K = [omega]x, K^2 = omega omega^T - th2 I and exp(xi) = [R | V upsilon],
// R = I + A K + B K^2, V = I + B K + C K^2:
//   R T = T + A (K T) + B (omega (omega^T T) - th2 T),
//   V upsilon = upsilon + B (K upsilon) + C (omega (omega . upsilon) - th2 upsilon),
// so one set of three-term dot products (K T, omega^T T, K upsilon,
// omega . upsilon and th2 in different lanes) feeds everything, and the
// dependent FP64 chain is: dot products (3), the series overlapped with the
// K^2 terms (1 to 4), two FMAs, one add.
__device__ __forceinline__ float warp_se3_left_update(const double xi[6], const double *Tin, double *Tout,
                                                      float *Tfout) {
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const double wx = xi[0], wy = xi[1], wz = xi[2], ux = xi[3], uy = xi[4], uz = xi[5];
    // lanes 0..11: (r, c) = (lane / 4, lane % 4) of K T; 12..15: column c of omega^T T;
    // 16..18: row r of K upsilon; 19: omega . upsilon; 20: th2
    const bool nl = lane < 12, ul = lane >= 16 && lane < 19;
    const int r = nl ? (lane >> 2) : (ul ? lane - 16 : 0), c = lane & 3;
    // row r of K: (0, -wz, wy), (wz, 0, -wx), (-wy, wx, 0)
    const bool krow = nl || ul;
    const double a0 = krow ? (r == 0 ? 0.0 : (r == 1 ? wz : -wy)) : wx;
    const double a1 = krow ? (r == 0 ? -wz : (r == 1 ? 0.0 : wx)) : wy;
    const double a2 = krow ? (r == 0 ? wy : (r == 1 ? -wx : 0.0)) : wz;
    const bool tcol = lane < 16;
    const double b0 = tcol ? Tin[c] : (lane == 20 ? wx : ux);
    const double b1 = tcol ? Tin[4 + c] : (lane == 20 ? wy : uy);
    const double b2 = tcol ? Tin[8 + c] : (lane == 20 ? wz : uz);
    const double d = fma(a2, b2, fma(a1, b1, a0 * b0));
    const double th2 = __shfl_sync(full, d, 20);
    const double wu = __shfl_sync(full, d, 19);
    const double wtt = __shfl_sync(full, d, 12 + c);
    // K^2 term of this lane: omega_r X - th2 Y, with (X, Y) = ((omega^T T)_c, T_rc) or (omega . upsilon, upsilon_r)
    const double wr = r == 0 ? wx : (r == 1 ? wy : wz);
    const double Y = nl ? Tin[4 * r + c] : (r == 0 ? ux : (r == 1 ? uy : uz));
    const double X = nl ? wtt : wu;
    double k2;
    const double coef = se3_series(lane % 3, th2, wr, X, Y, k2);
    const double A = __shfl_sync(full, coef, 0), B = __shfl_sync(full, coef, 1), C = __shfl_sync(full, coef, 2);
    // lanes 0..11: (R T)_rc = T_rc + A (K T)_rc + B (K^2 T)_rc; lanes 16..18: (V upsilon)_r
    double nv = fma(nl ? B : C, k2, fma(nl ? A : B, d, Y));
    const double tr = __shfl_sync(full, nv, 16 + (nl ? r : 0));
    if (nl && c == 3) nv += tr;
    if (nl) {
        Tout[lane] = nv;
        Tfout[lane] = f32_rn_of_f64(nv);
    }
    // |xi|^2 in FP32: lane k < 6 converts xi[k], then a sum over 8 lanes
    const int k6 = lane & 7;
    const double xk = k6 == 0 ? wx : k6 == 1 ? wy : k6 == 2 ? wz : k6 == 3 ? ux : k6 == 4 ? uy : uz;
    const float xf = k6 < 6 ? (float)xk : 0.f;
    float n2 = xf * xf;
    n2 += __shfl_xor_sync(full, n2, 1);
    n2 += __shfl_xor_sync(full, n2, 2);
    n2 += __shfl_xor_sync(full, n2, 4);
    return n2;
}

}  // namespace ss
