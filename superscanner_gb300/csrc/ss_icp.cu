// ss_icp.cu — CreatePcdFromDepthView, CalculateNormalsFromPCDView and
// kokkosICP (src/utils/imageutil.cpp:89-157, src/postprocessing/kokkosICP.cpp:25-210).
//
// The reference runs the 10x10-window correspondence search on the GPU and
// then copies both point clouds and the correspondences to the host every
// iteration for centroids, RMSE, H and an Eigen JacobiSVD. Here one kernel
// per iteration does the search, reduces the 18 sums per CTA as float pairs
// (warp shuffles), adds the CTA's totals exactly in fixed point with integer
// atomics, and the last CTA to finish takes the totals, the rotation as the polar factor of
// H^T (the SVD's V U^T for a full-rank H; a one-sided Jacobi SVD otherwise)
// and writes the next Txy, so the 10 iterations run without a host round trip.
#include <climits>
#include <mutex>

#include "ss_grid_impl.cuh"

namespace ss {

// ------------------------------------------------------------- pcd/normals
__global__ void depth_to_pcd_kernel(const uint16_t *__restrict__ depth, int rows, int cols, Intr in,
                                    float *__restrict__ pcd) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y;
    if (j >= cols || i >= rows) return;
    const size_t p = (size_t)i * cols + j;
    const F3 v = get_point(in, i, j, depth_m(__ldg(depth + p)));
    pcd[p * 3 + 0] = v.x;
    pcd[p * 3 + 1] = v.y;
    pcd[p * 3 + 2] = v.z;
}

__device__ __forceinline__ F3 ld3(const float *__restrict__ a, size_t p) {
    return {__ldg(a + p * 3), __ldg(a + p * 3 + 1), __ldg(a + p * 3 + 2)};
}

// Both reference launches in one: default (0,0,1) (imageutil.cpp:123-126),
// interior pixels with five valid depths get the normalized sum of the four
// neighbour cross products (:128-154).
__global__ void normals_kernel(const float *__restrict__ pcd, int rows, int cols, float *__restrict__ out) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y;
    if (j >= cols || i >= rows) return;
    const size_t p = (size_t)i * cols + j;
    F3 n{0.f, 0.f, 1.f};
    if (i >= 1 && i < rows - 1 && j >= 1 && j < cols - 1) {
        const F3 c = ld3(pcd, p), up = ld3(pcd, p + cols), dn = ld3(pcd, p - cols), rt = ld3(pcd, p + 1),
                 lf = ld3(pcd, p - 1);
        if (c.z != 0 && up.z != 0 && dn.z != 0 && rt.z != 0 && lf.z != 0) {
            // pcd(i+1,j) = up, pcd(i-1,j) = dn, pcd(i,j+1) = rt, pcd(i,j-1) = lf
            const F3 n1 = f3cross(f3sub(up, c), f3sub(rt, c));
            const F3 n2 = f3cross(f3sub(lf, c), f3sub(up, c));
            const F3 n3 = f3cross(f3sub(rt, c), f3sub(dn, c));
            const F3 n4 = f3cross(f3sub(dn, c), f3sub(lf, c));
            n = f3normalized(f3add(f3add(f3add(n1, n2), n3), n4));
        }
    }
    out[p * 3 + 0] = n.x;
    out[p * 3 + 1] = n.y;
    out[p * 3 + 2] = n.z;
}

// 16- and 8-byte asynchronous copies from global to shared memory (no
// registers held while they are in flight).
__device__ __forceinline__ void cp_async16(unsigned dst, const void *src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async8(unsigned dst, const void *src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(dst), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// ----------------------------------------------------------------- kokkosICP
constexpr int kIcpSums = 18;  // n_cors, sum x (3), sum y (3), sum x y^T (9), sum tmp^2, n_x
constexpr int kIcpIters = 10; // n_it (kokkosICP.cpp:54)

// Cross-CTA sums of an iteration in fixed point: a CTA's pair (hi, lo) of
// value v is converted exactly, to a resolution of 2^-kIcpFix, into a signed
// integer below 2^95 in magnitude (values below 2^47: every sum of a 640 x 480
// image is far below), split into three 32-bit chunks (two unsigned, the top
// one signed) and each chunk added with a 64-bit integer atomic into its own
// word: fewer than 2^10 CTAs add less than 2^42 to a word, so no carry leaves
// it. The totals are exact and do not depend on the order in which the CTAs
// arrive; the last CTA (by ticket) recombines each into a 128-bit integer and
// takes it as a float pair.
constexpr int kIcpFix = kFix48;
constexpr int kIcpAccWords = 3 * kIcpSums;

struct IcpState {
    float Txy[16];      // float copy used by the search (EigentoKmat4f(Txy.cast<float>()))
    float2 best[16];    // bestTxy_eigen, each entry a float pair (hi + lo)
    float lowest;       // lowestRSME
    float best_fitness;
    int ticket;         // CTAs done with the iteration
    int iteration;
    int overflow;       // a CTA value out of the fixed-point range (or NaN) this iteration
    float stats[kIcpIters * 4];  // per iteration: correspondences, RMSE, fitness, became best
    unsigned long long acc[kIcpAccWords];  // value v: chunk words 3 v, 3 v + 1, 3 v + 2
};

// The starting transform of a call (Txy as floats), passed by value to the
// prep kernel, which initialises the state with it.
struct IcpInit {
    float Txy[16];
};

// A call's result as the final iteration's last CTA writes it (into host
// memory mapped into the device's address space, where the caller has some).
struct IcpOut {
    float2 best[16];  // bestTxy_eigen as float pairs
    float lowest;     // lowestRSME
};

// t 2^-kIcpFix rounded to the nearest float (ties to even), |t| < 2^127, by
// integer operations (every such value is a normal float).
__device__ __forceinline__ float icp_float_of_fixed(__int128 t) {
    if (t == 0) return 0.f;
    const bool neg = t < 0;
    unsigned __int128 m = neg ? (unsigned __int128)(-t) : (unsigned __int128)t;
    const unsigned long long mh = (unsigned long long)(m >> 64), ml = (unsigned long long)m;
    const int lz = mh ? __clzll((long long)mh) : 64 + __clzll((long long)ml);
    m <<= lz;  // the leading one at bit 127
    const unsigned long long th = (unsigned long long)(m >> 64), tl = (unsigned long long)m;
    unsigned mant = (unsigned)(th >> 40);  // 24 bits
    int ex = 127 - lz - kIcpFix;           // value in [2^ex, 2^(ex + 1))
    if (((th >> 39) & 1ull) && ((th & ((1ull << 39) - 1ull)) || tl || (mant & 1u))) {
        if (++mant >> 24) {
            mant >>= 1;
            ex++;
        }
    }
    return __uint_as_float((neg ? 0x80000000u : 0u) | ((unsigned)(ex + 127) << 23) | (mant & 0x7fffffu));
}

// depth_to_pcd_kernel for both of kokkosICP's depth images and normals_kernel
// for the second, in one launch: a pixel's column and row quotients of
// getPoint are shared by its points, and its neighbours' points are
// recomputed from their depths with the same roundings, so the three images
// equal those of the three separate launches bit for bit. The source points
// go out as float triples; the target point and normal of a pixel as one
// 16-byte (x, y, z, nx) and one 8-byte (ny, nz) entry, the layout the
// iteration kernel stages in shared memory, x holding NaN where the
// reference's search skips the tap (py.z == 0, or n.x == 0 point-to-plane:
// kokkosICP.cpp:89,100) so that its distance fails every comparison.
__global__ void icp_prep_kernel(const uint16_t *__restrict__ d1, const uint16_t *__restrict__ d2, int rows, int cols,
                                Intr in, int type, float *__restrict__ xp, float4 *__restrict__ ya,
                                float2 *__restrict__ yb, IcpInit ini, IcpState *__restrict__ st) {
    if (blockIdx.x == 0 && blockIdx.y == 0) {  // the call's state: Txy, identity best, counters cleared
        const int t = threadIdx.x;
        if (t < 16) {
            st->Txy[t] = ini.Txy[t];
            st->best[t] = make_float2(t % 5 == 0 ? 1.f : 0.f, 0.f);
        }
        for (int k = t; k < kIcpAccWords; k += blockDim.x) st->acc[k] = 0ull;
        for (int k = t; k < kIcpIters * 4; k += blockDim.x) st->stats[k] = 0.f;
        if (t == 0) {
            st->lowest = 1e6f;  // lowestRSME (kokkosICP.cpp:59)
            st->best_fitness = 0.f;
            st->ticket = 0;
            st->iteration = 0;
            st->overflow = 0;
        }
    }
    const int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y;
    if (j >= cols || i >= rows) return;
    const size_t p = (size_t)i * cols + j;
    const float qx = __fdiv_rn(__fsub_rn((float)j, in.cj), in.fx), qy = __fdiv_rn(__fsub_rn((float)i, in.ci), in.fy);
    auto pt = [](float ux, float uy, float d) { return F3{__fmul_rn(ux, d), __fmul_rn(uy, d), d}; };
    const F3 x = pt(qx, qy, depth_m(__ldg(d1 + p)));
    const F3 c = pt(qx, qy, depth_m(__ldg(d2 + p)));
    xp[p * 3 + 0] = x.x;
    xp[p * 3 + 1] = x.y;
    xp[p * 3 + 2] = x.z;
    F3 n{0.f, 0.f, 1.f};
    if (i >= 1 && i < rows - 1 && j >= 1 && j < cols - 1) {
        const float qxl = __fdiv_rn(__fsub_rn((float)(j - 1), in.cj), in.fx);
        const float qxr = __fdiv_rn(__fsub_rn((float)(j + 1), in.cj), in.fx);
        const float qyd = __fdiv_rn(__fsub_rn((float)(i - 1), in.ci), in.fy);
        const float qyu = __fdiv_rn(__fsub_rn((float)(i + 1), in.ci), in.fy);
        const F3 up = pt(qx, qyu, depth_m(__ldg(d2 + p + cols))), dn = pt(qx, qyd, depth_m(__ldg(d2 + p - cols)));
        const F3 rt = pt(qxr, qy, depth_m(__ldg(d2 + p + 1))), lf = pt(qxl, qy, depth_m(__ldg(d2 + p - 1)));
        if (c.z != 0 && up.z != 0 && dn.z != 0 && rt.z != 0 && lf.z != 0) {  // as normals_kernel
            const F3 n1 = f3cross(f3sub(up, c), f3sub(rt, c));
            const F3 n2 = f3cross(f3sub(lf, c), f3sub(up, c));
            const F3 n3 = f3cross(f3sub(rt, c), f3sub(dn, c));
            const F3 n4 = f3cross(f3sub(dn, c), f3sub(lf, c));
            n = f3normalized(f3add(f3add(f3add(n1, n2), n3), n4));
        }
    }
    const bool tap = c.z != 0 && (type == SS_ICP_POINT_TO_POINT || n.x != 0);
    ya[p] = make_float4(tap ? c.x : __int_as_float(0x7fc00000), c.y, c.z, n.x);
    yb[p] = make_float2(n.y, n.z);
}


__device__ void svd3_jacobi(const double *H, double *U, double *S, double *V) {
    double A[9];
    for (int k = 0; k < 9; k++) A[k] = H[k];
    for (int k = 0; k < 9; k++) V[k] = (k % 4 == 0) ? 1.0 : 0.0;
    for (int sweep = 0; sweep < 60; sweep++) {
        bool rotated = false;
        for (int p = 0; p < 2; p++)
            for (int q = p + 1; q < 3; q++) {
                double alpha = 0, beta = 0, gamma = 0;
                for (int i = 0; i < 3; i++) {
                    alpha += A[i * 3 + p] * A[i * 3 + p];
                    beta += A[i * 3 + q] * A[i * 3 + q];
                    gamma += A[i * 3 + p] * A[i * 3 + q];
                }
                if (gamma == 0.0 || fabs(gamma) <= 1e-15 * sqrt(alpha * beta)) continue;
                rotated = true;
                const double zeta = (beta - alpha) / (2.0 * gamma);
                const double t = (zeta >= 0 ? 1.0 : -1.0) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
                const double c = 1.0 / sqrt(1.0 + t * t), s = c * t;
                for (int i = 0; i < 3; i++) {
                    const double ap = A[i * 3 + p], aq = A[i * 3 + q];
                    A[i * 3 + p] = c * ap - s * aq;
                    A[i * 3 + q] = s * ap + c * aq;
                    const double vp = V[i * 3 + p], vq = V[i * 3 + q];
                    V[i * 3 + p] = c * vp - s * vq;
                    V[i * 3 + q] = s * vp + c * vq;
                }
            }
        if (!rotated) break;
    }
    int zero_col = -1;
    for (int j = 0; j < 3; j++) {
        const double n = sqrt(A[j] * A[j] + A[3 + j] * A[3 + j] + A[6 + j] * A[6 + j]);
        S[j] = n;
        if (n > 1e-300) {
            for (int i = 0; i < 3; i++) U[i * 3 + j] = A[i * 3 + j] / n;
        } else {
            zero_col = j;
            for (int i = 0; i < 3; i++) U[i * 3 + j] = 0;
        }
    }
    if (zero_col >= 0) {
        const int a = (zero_col + 1) % 3, b = (zero_col + 2) % 3;
        const double ua[3] = {U[a], U[3 + a], U[6 + a]}, ub[3] = {U[b], U[3 + b], U[6 + b]};
        U[zero_col] = ua[1] * ub[2] - ua[2] * ub[1];
        U[3 + zero_col] = ua[2] * ub[0] - ua[0] * ub[2];
        U[6 + zero_col] = ua[0] * ub[1] - ua[1] * ub[0];
    }
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// Orthogonal polar factor R of A = H^T (A = R P, P symmetric positive
// semidefinite), by one warp: the scaled Newton iteration X <- (g X + (g X)^-T) / 2
// (Higham, "Computing the polar decomposition with applications", SIAM J. Sci.
// Stat. Comput. 7, 1986), lane r*3+c holding X[r][c] in FP64, X^-T from the
// cofactors, g = (|X^-1|_F / |X|_F)^(1/2) in FP32 (the scaling only sets the
// speed, not the fixed point). For a full-rank H = U S V^T, R = V U^T: the
// rotation kokkosICP takes from its SVD (kokkosICP.cpp:173-176), without its
// sign and order conventions. Returns false for a (nearly) rank-deficient H;
// R is then left unset. Every lane of the warp calls it.
__device__ bool polar3_warp(const double *H, double *R) {
    const int lane = threadIdx.x & 31;
    const bool mine = lane < 9;
    const int r = mine ? lane / 3 : 0, c = mine ? lane % 3 : 0;
    double x = mine ? H[c * 3 + r] : 0.0;  // A = H^T
    // exact power-of-two normalisation (the polar factor does not depend on scale)
    double mx = fabs(x);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if (!(mx > 0.0) || !isfinite(mx)) return false;
    x = ldexp(x, -ilogb(mx));
    const int r1 = (r + 1) % 3, r2 = (r + 2) % 3, c1 = (c + 1) % 3, c2 = (c + 2) % 3;
    bool ok = true;
    for (int it = 0; it < 24; it++) {
        // signed cofactor of (r, c) by the cyclic rule
        const double a11 = __shfl_sync(0xffffffffu, x, r1 * 3 + c1), a22 = __shfl_sync(0xffffffffu, x, r2 * 3 + c2);
        const double a12 = __shfl_sync(0xffffffffu, x, r1 * 3 + c2), a21 = __shfl_sync(0xffffffffu, x, r2 * 3 + c1);
        const double cof = mine ? fma(a11, a22, -a12 * a21) : 0.0;
        // det = sum_c X[0][c] C[0][c] (lanes 0..2)
        double dterm = lane < 3 ? x * cof : 0.0;
        dterm += __shfl_down_sync(0xffffffffu, dterm, 1);
        dterm += __shfl_down_sync(0xffffffffu, dterm, 2);
        const double det = __shfl_sync(0xffffffffu, dterm, 0);
        double fx = x * x, fc = cof * cof;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            fx += __shfl_xor_sync(0xffffffffu, fx, o);
            fc += __shfl_xor_sync(0xffffffffu, fc, o);
        }
        // |det| well below |X|^3: rank-deficient (relative 1e-10)
        if (!(fabs(det) > 1e-10 * fx * sqrt(fx))) {
            ok = false;
            break;
        }
        const float q = (float)fc / ((float)(det * det) * (float)fx);
        const double g = (double)sqrtf(sqrtf(q));
        // 1 / (g det) in FP64: FP32 seed, two Newton steps
        const double a = g * det;
        double y = (double)(1.0f / (float)a);
        y = fma(y, fma(-a, y, 1.0), y);
        y = fma(y, fma(-a, y, 1.0), y);
        const double xn = 0.5 * fma(g, x, cof * y);
        double dlt = fabs(xn - x);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) dlt = fmax(dlt, __shfl_xor_sync(0xffffffffu, dlt, o));
        x = xn;
        if (dlt <= 4e-16) break;
    }
    if (!ok) return false;
    if (mine) R[lane] = x;
    __syncwarp();
    return true;
}

// The same polar factor in FP32, by every lane of the warp at once:
// the scaled Newton iteration on A = H^T normalised by a power of two, until
// an update changes no entry by more than 1e-4, then one more (the error
// squares each step), R written as doubles. It is used where
// |det X| > 1e-4 |X|_F^3 at every step: then the two smaller singular values
// of H sum to more than 0.02 times the largest, and the FP32 roundings move
// R by at most a few 1e-6 rad (the polar factor's sensitivity to a
// perturbation of A is below 2 / (s_i + s_j) for the singular values
// s_i, s_j of the rotation's plane). Returns false otherwise (R unset): the
// FP64 iteration then decides. Every lane of the warp calls it.
__device__ bool polar3_warp_f32(const float *Hf, float *R) {
    // every lane iterates the whole 3 x 3 in its registers (no shuffles on
    // the dependent chain); the lanes compute identical values. Hf: H as
    // floats (each lane of the caller converted one entry).
    float X[9];
#pragma unroll
    for (int r = 0; r < 3; r++)
#pragma unroll
        for (int c = 0; c < 3; c++) X[r * 3 + c] = Hf[c * 3 + r];  // A = H^T
    float mx = 0.f;
#pragma unroll
    for (int k = 0; k < 9; k++) mx = fmaxf(mx, fabsf(X[k]));
    if (!(mx > 0.f) || !isfinite(mx)) return false;
    const int ex = ilogbf(mx);
#pragma unroll
    for (int k = 0; k < 9; k++) X[k] = ldexpf(X[k], -ex);
    bool last = false;
    for (int it = 0; it < 24; it++) {
        float cof[9];
#pragma unroll
        for (int r = 0; r < 3; r++)
#pragma unroll
            for (int c = 0; c < 3; c++) {
                const int r1 = (r + 1) % 3, r2 = (r + 2) % 3, c1 = (c + 1) % 3, c2 = (c + 2) % 3;
                cof[r * 3 + c] = fmaf(X[r1 * 3 + c1], X[r2 * 3 + c2], -X[r1 * 3 + c2] * X[r2 * 3 + c1]);
            }
        const float det = fmaf(X[0], cof[0], fmaf(X[1], cof[1], X[2] * cof[2]));
        float fx = 0.f, fc = 0.f;
#pragma unroll
        for (int k = 0; k < 9; k++) {
            fx = fmaf(X[k], X[k], fx);
            fc = fmaf(cof[k], cof[k], fc);
        }
        if (!(fabsf(det) > 1e-4f * fx * sqrtf(fx))) return false;
        // the scale g only sets the speed (approximate instructions suffice);
        // y is the reciprocal of the g det that scales X
        const float g = rsqrtf(rsqrtf(__fdividef(fc, det * det * fx)));
        const float y = __frcp_rn(g * det);
        float dlt = 0.f;
#pragma unroll
        for (int k = 0; k < 9; k++) {
            const float xn = 0.5f * fmaf(g, X[k], cof[k] * y);
            dlt = fmaxf(dlt, fabsf(xn - X[k]));
            X[k] = xn;
        }
        if (last) break;
        last = dlt <= 1e-4f;
    }
    if (!last) return false;
    const int lane = threadIdx.x & 31;
    float mine = 0.f;  // X[lane] without dynamic register indexing
#pragma unroll
    for (int k = 0; k < 9; k++)
        if (lane == k) mine = X[k];
    if (lane < 9) R[lane] = mine;
    __syncwarp();
    return true;
}

// Float pairs (hi, lo) holding hi + lo: the per-pixel terms of kokkosICP's
// double sums are exact in this form (x and y coordinates are floats; a
// product of two floats is hi = RN(a b), lo = the exact rounding error), and
// pairs add with an error-free TwoSum, so the CTA sums keep double-like
// accuracy without FP64 instructions (one FP64 warp instruction occupies an
// SM sub-partition's FP64 pipe for tens of cycles on this part).
__device__ __forceinline__ void fp2_add(float &h, float &l, float h2, float l2) {
    const float s = __fadd_rn(h, h2);
    const float bb = __fsub_rn(s, h);
    const float e = __fadd_rn(__fsub_rn(h, __fsub_rn(s, bb)), __fsub_rn(h2, bb));
    const float t = __fadd_rn(__fadd_rn(l, l2), e);
    h = __fadd_rn(s, t);
    l = __fsub_rn(t, __fsub_rn(h, s));
}

// fp2_add of two independent pairs at once (packed: value 0 in the low
// halves), the same operations in the same order on each half.
__device__ __forceinline__ void fp2_add2(f32x2 &h, f32x2 &l, f32x2 h2, f32x2 l2) {
    const f32x2 s = f2_add(h, h2);
    const f32x2 bb = f2_sub(s, h);
    const f32x2 e = f2_add(f2_sub(h, f2_sub(s, bb)), f2_sub(h2, bb));
    const f32x2 t = f2_add(f2_add(l, l2), e);
    h = f2_add(s, t);
    l = f2_sub(t, f2_sub(h, s));
}

// The CTA's 18 sums: each lane's pairs, a warp transpose-reduce (at offset o a
// lane keeps the half of its values selected by lane bit o and adds the other
// lane's; after offsets 16..1 lane v holds the warp's pair of value v), then
// the warps' pairs by a fixed tree; thread v < kIcpSums returns the CTA's
// pair of value v.
__device__ __forceinline__ float2 icp_cta_sum(float *vh, float *vl, float2 (*red)[kIcpSums]) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) {
        const bool upper = (lane & o) != 0;
        if (o >= 2) {  // two values per step in paired instructions (the same roundings)
#pragma unroll
            for (int k = 0; k < o; k += 2) {
                float kh[2], kl[2], rh[2], rl[2];
#pragma unroll
                for (int u = 0; u < 2; u++) {
                    const float sh = upper ? vh[k + u] : vh[k + u + o], sl = upper ? vl[k + u] : vl[k + u + o];
                    kh[u] = upper ? vh[k + u + o] : vh[k + u];
                    kl[u] = upper ? vl[k + u + o] : vl[k + u];
                    rh[u] = __shfl_xor_sync(0xffffffffu, sh, o);
                    rl[u] = __shfl_xor_sync(0xffffffffu, sl, o);
                }
                f32x2 ph = f2_pack(kh[0], kh[1]), pl = f2_pack(kl[0], kl[1]);
                fp2_add2(ph, pl, f2_pack(rh[0], rh[1]), f2_pack(rl[0], rl[1]));
                f2_unpack(ph, vh[k], vh[k + 1]);
                f2_unpack(pl, vl[k], vl[k + 1]);
            }
        } else {
            const float sh = upper ? vh[0] : vh[1], sl = upper ? vl[0] : vl[1];
            float kh = upper ? vh[1] : vh[0], kl = upper ? vl[1] : vl[0];
            const float rh = __shfl_xor_sync(0xffffffffu, sh, 1), rl = __shfl_xor_sync(0xffffffffu, sl, 1);
            fp2_add(kh, kl, rh, rl);
            vh[0] = kh;
            vl[0] = kl;
        }
    }
    if (lane < kIcpSums) red[wid][lane] = make_float2(vh[0], vl[0]);
    __syncthreads();
    float h = 0.f, l = 0.f;
    if (threadIdx.x < kIcpSums) {  // the eight warps' pairs by a tree, three additions deep
        float2 p[8];
#pragma unroll
        for (int w = 0; w < 8; w++) p[w] = red[w][threadIdx.x];
#pragma unroll
        for (int st = 1; st < 8; st <<= 1)
#pragma unroll
            for (int w = 0; w < 8; w += 2 * st) fp2_add(p[w].x, p[w].y, p[w + st].x, p[w + st].y);
        h = p[0].x;
        l = p[0].y;
    }
    return make_float2(h, l);
}

// Target pixels staged per CTA: a tile's 10 x 10 windows (kokkosICP.cpp:81-83)
// usually fall inside a region of some 42 x 26 pixels; up to this many are
// staged, larger regions are read from global memory.
constexpr int kIcpStage = 1536;
constexpr int kIcpSearch = 5;         // n_search (kokkosICP.cpp:53)
constexpr float kIcpMaxDist = 0.075f; // max_dist (kokkosICP.cpp:55)

// The transformed source point px = Txy x and its window centre
// (kokkosICP.cpp:72-76); true when the reference searches (x.z != 0 and the
// window inside the image, :79).
__device__ __forceinline__ bool icp_center(const Mat34 &T, F3 x, Intr in, int rows, int cols, F3 &px, int &ci,
                                           int &cj) {
    px = F3{0.f, 0.f, 0.f};
    ci = cj = 0;
    if (x.z == 0) return false;
    px = xform(T, x);
    const float c0 = __fadd_rn(__fdiv_rn(__fmul_rn(px.y, in.fy), px.z), in.ci);
    const float c1 = __fadd_rn(__fdiv_rn(__fmul_rn(px.x, in.fx), px.z), in.cj);
    ci = __float2int_rz(c0);
    cj = __float2int_rz(c1);
    return ci > kIcpSearch && ci < rows - kIcpSearch && cj > kIcpSearch && cj < cols - kIcpSearch;
}

// A tap's distance (kokkosICP.cpp:91,101-102) from its (x, y, z, nx) and
// (ny, nz) entries; NaN for a tap the reference skips.
template <int kType>
__device__ __forceinline__ float icp_tap_dist(const float4 a, const float2 b, F3 px) {
    const F3 py{a.x, a.y, a.z};
    return kType == SS_ICP_POINT_TO_POINT ? f3len(f3sub(py, px)) : fabsf(f3dot(f3sub(py, px), F3{a.w, b.x, b.y}));
}

// The search state of one window: the even and the odd columns keep separate
// minima (two independent compare chains) with their taps' indices (staged
// or image indices, increasing in the window's scan order); the first tap of
// the scan with the smallest distance is then the one of the smaller
// minimum, on a tie the earlier tap. Starting from max_dist, the accepted
// taps of `dist < smallest && dist < max_dist` are exactly those of
// `dist < min(smallest, max_dist)`.
struct IcpBest {
    float s0 = kIcpMaxDist, s1 = kIcpMaxDist;
    int b0 = -1, b1 = -1;
    __device__ __forceinline__ void take(bool odd, float dist, int idx) {
        if (odd) {
            if (dist < s1) {
                s1 = dist;
                b1 = idx;
            }
        } else if (dist < s0) {
            s0 = dist;
            b0 = idx;
        }
    }
    __device__ __forceinline__ int best() const { return (s1 < s0 || (s1 == s0 && b1 < b0)) ? b1 : b0; }
};

// The distances of one tap to two transformed source points (packed x, y and
// z of both): icp_tap_dist for each, the same roundings in the same order.
template <int kType>
__device__ __forceinline__ void icp_tap_dist2(const float4 a, const float2 b, f32x2 px, f32x2 py, f32x2 pz, float &da,
                                              float &db) {
    const f32x2 dx = f2_sub(f2_pack(a.x, a.x), px), dy = f2_sub(f2_pack(a.y, a.y), py),
                dz = f2_sub(f2_pack(a.z, a.z), pz);
    if (kType == SS_ICP_POINT_TO_POINT) {
        f2_unpack(f2_add(f2_add(f2_mul(dx, dx), f2_mul(dy, dy)), f2_mul(dz, dz)), da, db);
        da = __fsqrt_rn(da);
        db = __fsqrt_rn(db);
    } else {
        f2_unpack(f2_add(f2_add(f2_mul(dx, f2_pack(a.w, a.w)), f2_mul(dy, f2_pack(b.x, b.x))), f2_mul(dz, f2_pack(b.y, b.y))),
                  da, db);
        da = fabsf(da);
        db = fabsf(db);
    }
}

// One window row of staged taps [row, row + 10) for up to two windows that
// contain it (a vertical pixel pair's windows share nine of their rows): a
// half row's taps are loaded once, before their comparisons, and each tap's
// distances to both source points are evaluated together (packed pairs pa, pb
// of the two points' coordinates: x, y, z).
template <int kType>
__device__ __forceinline__ void icp_scan_row(const float4 *sA, const float2 *sB, int row, f32x2 px, f32x2 py,
                                             f32x2 pz, bool ua, IcpBest &ba, bool ub, IcpBest &bb) {
#pragma unroll
    for (int half = 0; half < 2; half++) {
        float4 a[kIcpSearch];
        float2 b[kIcpSearch];
#pragma unroll
        for (int dl = 0; dl < kIcpSearch; dl++) {
            a[dl] = sA[row + half * kIcpSearch + dl];
            b[dl] = kType == SS_ICP_POINT_TO_PLANE ? sB[row + half * kIcpSearch + dl] : make_float2(0.f, 0.f);
        }
#pragma unroll
        for (int dl = 0; dl < kIcpSearch; dl++) {
            const bool odd = ((dl + half * kIcpSearch) & 1) != 0;
            const int idx = row + half * kIcpSearch + dl;
            float da, db;
            icp_tap_dist2<kType>(a[dl], b[dl], px, py, pz, da, db);
            if (ua) ba.take(odd, da, idx);
            if (ub) bb.take(odd, db, idx);
        }
    }
}

// A window read from global memory (a tile whose window region does not fit
// the stage): image indices, the reference's loops.
template <int kType>
__device__ __forceinline__ int icp_search_global(const float4 *__restrict__ ya, const float2 *__restrict__ yb, int cols,
                                                 int ci, int cj, F3 px) {
    IcpBest bt;
    for (int k = ci - kIcpSearch; k < ci + kIcpSearch; k++)
        for (int l = cj - kIcpSearch; l < cj + kIcpSearch; l++) {
            const int tag = k * cols + l;
            const float2 b = kType == SS_ICP_POINT_TO_PLANE ? __ldg(yb + tag) : make_float2(0.f, 0.f);
            bt.take(false, icp_tap_dist<kType>(__ldg(ya + tag), b, px), tag);
        }
    return bt.best();
}

// Adds one source pixel's terms of the host sums (kokkosICP.cpp:121-171) to
// the lane's float pairs: for a correspondence (x_nearest.z != 0) the count,
// x, x_nearest, x x_nearest^T (each product exact as a pair) and the RMSE
// term. best indexes the staged region (staged) or the image.
template <int kType>
__device__ __forceinline__ void icp_add_terms(F3 x, const Mat34 &T, int best, bool staged, const float4 *sA,
                                              const float2 *sB, const float4 *__restrict__ ya,
                                              const float2 *__restrict__ yb, float *vh, float *vl) {
    if (best < 0) return;
    const F3 px = xform(T, x);
    const float4 a = staged ? sA[best] : __ldg(ya + best);
    const float2 b = kType == SS_ICP_POINT_TO_PLANE ? (staged ? sB[best] : __ldg(yb + best)) : make_float2(0.f, 0.f);
    const F3 py{a.x, a.y, a.z}, nn{a.w, b.x, b.y};
    const F3 bpt = kType == SS_ICP_POINT_TO_POINT ? py : f3add(px, f3smul(f3dot(f3sub(py, px), nn), nn));
    if (bpt.z == 0) return;  // x_nearest(i, j).z == 0: no correspondence (kokkosICP.cpp:131)
    const float xa[3] = {x.x, x.y, x.z}, xb[3] = {bpt.x, bpt.y, bpt.z};
    fp2_add(vh[0], vl[0], 1.f, 0.f);
#pragma unroll
    for (int r = 0; r < 3; r++) {
        fp2_add(vh[1 + r], vl[1 + r], xa[r], 0.f);
        fp2_add(vh[4 + r], vl[4 + r], xb[r], 0.f);
#pragma unroll
        for (int c = 0; c < 3; c++) {  // x y^T, each product exact as a pair
            const float q = __fmul_rn(xa[r], xb[c]);
            fp2_add(vh[7 + 3 * r + c], vl[7 + 3 * r + c], q, fmaf(xa[r], xb[c], -q));
        }
    }
    // RMSE term || x_nearest - Txy x || squared in float (kokkosICP.cpp:137-138; the
    // reference evaluates the norm in double, this in FP32 with the float Txy)
    const float e0 = xb[0] - fmaf(T.m[0], xa[0], fmaf(T.m[1], xa[1], fmaf(T.m[2], xa[2], T.m[3])));
    const float e1 = xb[1] - fmaf(T.m[4], xa[0], fmaf(T.m[5], xa[1], fmaf(T.m[6], xa[2], T.m[7])));
    const float e2 = xb[2] - fmaf(T.m[8], xa[0], fmaf(T.m[9], xa[1], fmaf(T.m[10], xa[2], T.m[11])));
    const float tmp = sqrtf(fmaf(e0, e0, fmaf(e1, e1, e2 * e2)));
    fp2_add(vh[16], vl[16], tmp * tmp, 0.f);
}

// Copies the target entries of rows [r0, r0 + h) x columns [q0, q0 + w) of
// the image into the stage (row pitch w) with asynchronous copies: warp k
// copies rows k, k + 8, ..., its lanes the columns, the entries in the layout
// icp_prep_kernel wrote them in. The caller waits for them.
template <int kType>
__device__ __forceinline__ void icp_stage(float4 *sA, float2 *sB, const float4 *__restrict__ ya,
                                          const float2 *__restrict__ yb, int cols, int r0, int q0, int w, int h) {
    const unsigned sa_s = (unsigned)__cvta_generic_to_shared(sA), sb_s = (unsigned)__cvta_generic_to_shared(sB);
    const int ln = threadIdx.x & 31;
    for (int r = threadIdx.x >> 5; r < h; r += 8) {
        const size_t q = (size_t)(r0 + r) * cols + q0;
        for (int c = ln; c < w; c += 32) {
            const int t = r * w + c;
            cp_async16(sa_s + 16u * t, ya + q + c);
            if (kType == SS_ICP_POINT_TO_PLANE) cp_async8(sb_s + 8u * t, yb + q + c);
        }
    }
}

// Pixels by which an iteration widens the region its CTA needed in the
// iteration before when it stages that region ahead of its wait.
constexpr int kIcpMargin = 2;

// One kokkosICP iteration: Closest Point Kernel (kokkosICP.cpp:69-115) fused
// with the host sums (:121-171) and, in the last CTA, the rotation update
// (:173-185). A CTA covers a 32 x 16 tile of source pixels, each thread a
// vertical pair (rows 2w and 2w + 1 of warp w's lane column). The target
// points and normals under the tile's windows are staged in shared memory
// first by asynchronous copies of icp_prep_kernel's entries (a tap that the
// reference skips holding NaN, so that its distance fails every comparison).
// The search keeps the reference's scan order and strict comparisons for
// each window, remembers the best tap and forms the correspondence from it
// afterwards. Every iteration after the first stages, before it waits for
// the previous one, the region its CTA needed there widened by kIcpMargin
// (regions[cta]: rows r0.., columns q0.., width, height), and keeps it when
// it holds every window of this iteration (the centres move little between
// iterations); the images are constant, so any staged region is valid and
// only its bounds matter. When the two windows lie in the same columns at most two rows
// apart (the usual case: neighbouring pixels project to neighbouring centres,
// one row apart), the thread scans their union, loading each tap once for
// both; otherwise it scans the lower window on its own after the upper one.
// 64 registers (four CTAs per SM; only the rank-deficient fallback of the
// last CTA spills).
template <int kType>
__global__ void __launch_bounds__(256, 4) icp_ref_iter_kernel(const float *__restrict__ xp,
                                                           const float4 *__restrict__ ya,
                                                           const float2 *__restrict__ yb, int rows, int cols, Intr in,
                                                           IcpState *st,
                                                           int4 *__restrict__ regions, int prestage, IcpOut *out) {
    __shared__ float4 sA[kIcpStage];  // target (x, y, z, nx)
    __shared__ float2 sB[kIcpStage];  // target (ny, nz)
    __shared__ float2 red[8][kIcpSums];
    __shared__ int box[4];
    __shared__ int4 pre;
    __shared__ bool last;
    const unsigned nctas = gridDim.x * gridDim.y, cta = blockIdx.y * gridDim.x + blockIdx.x;
    const int j = blockIdx.x * 32 + (threadIdx.x & 31), i0 = blockIdx.y * 16 + 2 * (threadIdx.x >> 5);
    const size_t p0 = (size_t)i0 * cols + j, p1 = p0 + cols;
    // the source points do not change between iterations (written before the
    // first one): loaded before this launch waits for the previous iteration,
    // whose last CTA is still forming Txy from the totals
    const F3 x0 = j < cols && i0 < rows ? ld3(xp, p0) : F3{0.f, 0.f, 0.f};
    const F3 x1 = j < cols && i0 + 1 < rows ? ld3(xp, p1) : F3{0.f, 0.f, 0.f};
    int4 P = make_int4(0, 0, 0, 0);  // the region staged before the wait: r0, q0, width, height
    if (prestage) {
        if (threadIdx.x == 0) {
            // the region written by this CTA's previous iteration (a stale
            // read only costs the restaging: it is checked to lie in the image)
            const int4 R = __ldcg(regions + cta);
            int4 q = make_int4(0, 0, 0, 0);
            if (R.z > 0 && R.w > 0 && R.x >= 0 && R.y >= 0 && R.w <= rows - R.x && R.z <= cols - R.y)
                for (int m = kIcpMargin; m >= 0; m--) {
                    const int a0 = max(R.x - m, 0), b0 = max(R.y - m, 0);
                    const int a1 = min(R.x + R.w + m, rows), b1 = min(R.y + R.z + m, cols);
                    if ((a1 - a0) * (b1 - b0) <= kIcpStage) {
                        q = make_int4(a0, b0, b1 - b0, a1 - a0);
                        break;
                    }
                }
            pre = q;
        }
        __syncthreads();
        P = pre;
        if (P.w > 0) icp_stage<kType>(sA, sB, ya, yb, cols, P.x, P.y, P.z, P.w);
    }
    pdl_wait();
    Mat34 T;
#pragma unroll
    for (int k = 0; k < 12; k++) T.m[k] = st->Txy[k];
    F3 pa, pb;
    int ca_i, ca_j, cb_i, cb_j;
    const bool sa = icp_center(T, x0, in, rows, cols, pa, ca_i, ca_j);
    const bool sb = icp_center(T, x1, in, rows, cols, pb, cb_i, cb_j);
    // the tile's window region [r0, r1) x [q0, q1)
    if (threadIdx.x == 0) {
        box[0] = INT_MAX;
        box[1] = INT_MIN;
        box[2] = INT_MAX;
        box[3] = INT_MIN;
    }
    __syncthreads();
    {
        int lo_i = sa ? ca_i : INT_MAX, hi_i = sa ? ca_i : INT_MIN;
        int lo_j = sa ? ca_j : INT_MAX, hi_j = sa ? ca_j : INT_MIN;
        if (sb) {
            lo_i = min(lo_i, cb_i);
            hi_i = max(hi_i, cb_i);
            lo_j = min(lo_j, cb_j);
            hi_j = max(hi_j, cb_j);
        }
        lo_i = __reduce_min_sync(0xffffffffu, lo_i);
        hi_i = __reduce_max_sync(0xffffffffu, hi_i);
        lo_j = __reduce_min_sync(0xffffffffu, lo_j);
        hi_j = __reduce_max_sync(0xffffffffu, hi_j);
        if ((threadIdx.x & 31) == 0 && lo_i != INT_MAX) {
            atomicMin(&box[0], lo_i);
            atomicMax(&box[1], hi_i);
            atomicMin(&box[2], lo_j);
            atomicMax(&box[3], hi_j);
        }
    }
    __syncthreads();
    const bool any = box[0] != INT_MAX;
    const int r0 = box[0] - kIcpSearch, q0 = box[2] - kIcpSearch;
    const int W = any ? box[3] + kIcpSearch - q0 : 0, H = any ? box[1] + kIcpSearch - r0 : 0;
    // the staged region: the one staged before the wait when it holds every
    // window (its origin and row pitch sr0, sq0, sw), else this one
    const bool reuse =
        any && P.w > 0 && r0 >= P.x && q0 >= P.y && r0 + H <= P.x + P.w && q0 + W <= P.y + P.z;
    bool staged = reuse || (any && W * H <= kIcpStage);
    const int sr0 = reuse ? P.x : r0, sq0 = reuse ? P.y : q0, sw = reuse ? P.z : W;
    if (!reuse && staged) {
        if (P.w > 0) {  // the early copies land before their entries are overwritten
            cp_async_wait_all();
            __syncthreads();
        }
        // inside the image: the border test keeps every window within rows x cols
        icp_stage<kType>(sA, sB, ya, yb, cols, r0, q0, W, H);
    }
    cp_async_wait_all();
    if (threadIdx.x == 0) regions[cta] = any ? make_int4(r0, q0, W, H) : make_int4(0, 0, 0, 0);
    __syncthreads();

    int best0 = -1, best1 = -1;
    if (staged) {
        // the thread's windows: the upper one leads, and the other joins it
        // when it lies dr = 0..2 rows below in the same columns (its rows are
        // then the lead's rows dr..dr + 9); a lower window that does not join
        // is scanned on its own afterwards
        int dr = 0;
        bool joined = false, swap = !sa && sb;  // swap: the lower pixel leads
        if (sa && sb && ca_j == cb_j && abs(cb_i - ca_i) <= 2) {
            joined = true;
            dr = abs(cb_i - ca_i);
            swap = cb_i < ca_i;
        }
        const F3 pl = swap ? pb : pa, pm = swap ? pa : pb;
        const f32x2 qx = f2_pack(pl.x, pm.x), qy = f2_pack(pl.y, pm.y), qz = f2_pack(pl.z, pm.z);
        IcpBest bl, bm;
        if (sa || sb) {
            const int li = swap ? cb_i : ca_i, lj = swap ? cb_j : ca_j;
            const int base = (li - kIcpSearch - sr0) * sw + (lj - kIcpSearch - sq0);
            const int nr = 2 * kIcpSearch + dr;
#pragma unroll 1
            for (int dk = 0; dk < nr; dk++)
                icp_scan_row<kType>(sA, sB, base + dk * sw, qx, qy, qz, dk < 2 * kIcpSearch, bl, joined && dk >= dr, bm);
        }
        if (sa && sb && !joined) {  // the lower window on its own (the upper one led)
            const int base = (cb_i - kIcpSearch - sr0) * sw + (cb_j - kIcpSearch - sq0);
            const f32x2 ux = f2_pack(pb.x, pb.x), uy = f2_pack(pb.y, pb.y), uz = f2_pack(pb.z, pb.z);
#pragma unroll 1
            for (int dk = 0; dk < 2 * kIcpSearch; dk++)
                icp_scan_row<kType>(sA, sB, base + dk * sw, ux, uy, uz, true, bm, false, bl);
        }
        best0 = swap ? bm.best() : bl.best();
        best1 = swap ? bl.best() : bm.best();
    } else {
        if (sa) best0 = icp_search_global<kType>(ya, yb, cols, ca_i, ca_j, pa);
        if (sb) best1 = icp_search_global<kType>(ya, yb, cols, cb_i, cb_j, pb);
    }

    // this thread's terms as float pairs, padded to 32 for the transpose-reduce
    float vh[32], vl[32];
#pragma unroll
    for (int k = 0; k < 32; k++) vh[k] = vl[k] = 0.f;
    vh[17] = (float)((x0.z != 0) + (x1.z != 0));  // n_pointsinX
    icp_add_terms<kType>(x0, T, best0, staged, sA, sB, ya, yb, vh, vl);
    icp_add_terms<kType>(x1, T, best1, staged, sA, sB, ya, yb, vh, vl);
    const int lane = threadIdx.x & 31;
    const float2 csum = icp_cta_sum(vh, vl, red);
    // the CTA's sums into the fixed-point words (thread v < kIcpSums: value v)
    if (threadIdx.x < kIcpSums) {
        __int128 qh, ql;
        const bool ok = fixed48_of_float(csum.x, qh) & fixed48_of_float(csum.y, ql);
        if (!ok) atomicOr(&st->overflow, 1);
        const __int128 q = ok ? qh + ql : (__int128)0;
        fixed48_add(st->acc + 3 * threadIdx.x, q);
    }
    // the additions, ordered by the barrier, are released by thread 0's fence
    // before its ticket; the last CTA acquires everyone's by a fence after its
    // ticket and reads the words from L2
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        const bool l = atomicAdd(&st->ticket, 1) == (int)nctas - 1;
        if (l) __threadfence();
        last = l;
    }
    __syncthreads();
    if (!last) return;  // (a CTA's exit lets the next iteration launch)
    pdl_trigger();      // the next iteration may launch (it waits for this grid before reading anything it writes)
    if (threadIdx.x >= 32) return;
    // last CTA, warp 0: lane v < kIcpSums takes total v as a float pair and
    // clears its words for the next iteration
    const float lowest = *(volatile float *)&st->lowest;  // the best RMSE so far
    __shared__ float2 tot[kIcpSums];
    __shared__ double Hs[9], Rs[9];
    __shared__ float Hf[9], Rf[9];
    if (lane < kIcpSums) {
        unsigned long long *w = st->acc + 3 * lane;
        const unsigned long long s0 = __ldcg(w), s1 = __ldcg(w + 1), s2 = __ldcg(w + 2);
        w[0] = 0ull;
        w[1] = 0ull;
        w[2] = 0ull;
        const __int128 t = fixed48_total(s0, s1, s2);
        const float h = icp_float_of_fixed(t);
        __int128 hq;
        fixed48_of_float(h, hq);
        float2 v = make_float2(h, icp_float_of_fixed(t - hq));
        if (*(volatile int *)&st->overflow) v = make_float2(__int_as_float(0x7fc00000), 0.f);  // as the reference's NaNs
        tot[lane] = v;
    }
    __syncwarp();
    // the update in float pairs (no FP64 instruction on this serial path; the
    // reference forms it in double, kokkosICP.cpp:121-185): n is an exact count
    const unsigned FULL = 0xffffffffu;
    const float n = tot[0].x;
    float ch = 0.f, cl = 0.f;  // lane k < 6: centerx (k < 3), centery (k >= 3) = sum / n
    if (lane < 6) {
        const float2 t = tot[1 + lane];
        ch = __fdiv_rn(t.x, n);
        cl = __fdiv_rn(fmaf(-ch, n, t.x) + t.y, n);  // the remainder t.x - ch n is exact
        const float q = ch + cl;
        cl -= q - ch;
        ch = q;
    }
    // H = sum (x - cx)(y - cy)^T = sum x y^T - n cx cy^T, lane 3 r + c: entry (r, c)
    {
        const int hr = min(lane / 3, 2), hc = lane % 3;
        const float xh = __shfl_sync(FULL, ch, hr), xl = __shfl_sync(FULL, cl, hr);
        const float yh = __shfl_sync(FULL, ch, 3 + hc), yl = __shfl_sync(FULL, cl, 3 + hc);
        const float ph = xh * yh, pl = fmaf(xh, yh, -ph) + fmaf(xh, yl, xl * yh);
        const float qh = n * ph, ql = fmaf(n, ph, -qh) + n * pl;
        if (lane < 9) {
            float hh = tot[7 + lane].x, hl = tot[7 + lane].y;
            fp2_add(hh, hl, -qh, -ql);
            Hf[lane] = hh;
            Hs[lane] = (double)hh + (double)hl;  // for the rank-deficient fallback
        }
    }
    __syncwarp();
    if (!polar3_warp_f32(Hf, Rf)) {  // the same outcome in every lane
        if (!polar3_warp(Hs, Rs) && lane == 0) {
            // rank-deficient H: the SVD's own completion of U
            double U[9], S[3], V[9];
            svd3_jacobi(Hs, U, S, V);
            for (int r = 0; r < 3; r++)
                for (int c = 0; c < 3; c++)
                    Rs[r * 3 + c] = V[r * 3] * U[c * 3] + V[r * 3 + 1] * U[c * 3 + 1] + V[r * 3 + 2] * U[c * 3 + 2];
        }
        __syncwarp();
        if (lane < 9) Rf[lane] = (float)Rs[lane];
        __syncwarp();
    }
    // the new Txy_eigen, one entry per lane: [R | centery - R centerx] (kokkosICP.cpp:177-179)
    float2 tn = make_float2((lane % 5 == 0) ? 1.f : 0.f, 0.f);
    {
        const int r = min(lane >> 2, 2);
        float cxh[3], cxl[3];
#pragma unroll
        for (int k = 0; k < 3; k++) {
            cxh[k] = __shfl_sync(FULL, ch, k);
            cxl[k] = __shfl_sync(FULL, cl, k);
        }
        const float cyh = __shfl_sync(FULL, ch, 3 + r), cyl = __shfl_sync(FULL, cl, 3 + r);
        if (lane < 12) {
            if ((lane & 3) < 3) {
                tn = make_float2(Rf[r * 3 + (lane & 3)], 0.f);
            } else {
                float sh = 0.f, sl = 0.f;  // R centerx as a pair
#pragma unroll
                for (int k = 0; k < 3; k++) {
                    const float a = Rf[r * 3 + k], p = a * cxh[k];
                    fp2_add(sh, sl, p, fmaf(a, cxh[k], -p) + a * cxl[k]);
                }
                float th = cyh, tl = cyl;
                fp2_add(th, tl, -sh, -sl);
                tn = make_float2(th, tl);
            }
        }
    }
    if (lane < 16) st->Txy[lane] = tn.x;
    float rsme = tot[16].x;
    rsme /= n;
    rsme = sqrtf(rsme);
    const float fitness = n / tot[17].x;
    const bool became_best = rsme < lowest;  // kokkosICP.cpp:181-185
    if (became_best && lane < 16) st->best[lane] = tn;
    if (out) {  // the final iteration, with a host-mapped result
        if (lane < 16) out->best[lane] = became_best ? tn : st->best[lane];
        if (lane == 0) out->lowest = became_best ? rsme : lowest;
    }
    if (lane != 0) return;
    if (became_best) st->lowest = rsme;
    const int it = st->iteration;
    if (fitness > st->best_fitness) st->best_fitness = fitness;
    if (it < kIcpIters) {
        st->stats[it * 4 + 0] = n;
        st->stats[it * 4 + 1] = rsme;
        st->stats[it * 4 + 2] = fitness;
        st->stats[it * 4 + 3] = became_best ? 1.f : 0.f;
    }
    st->iteration = it + 1;
    st->ticket = 0;
    st->overflow = 0;
}

// The iteration kernel's grid: one CTA per 32 x 16 tile of source pixels.
static inline int icp_tiles_x(int cols) { return (cols + 31) / 32; }
static inline int icp_tiles_y(int rows) { return (rows + 15) / 16; }

// Scratch of ss_kokkos_icp, one per device, grown on demand.
struct IcpWorkspace {
    float *xp = nullptr;
    float4 *ya = nullptr;
    float2 *yb = nullptr;
    int4 *regions = nullptr;
    IcpState *state = nullptr;
    IcpOut *out_host = nullptr, *out_dev = nullptr;  // pinned, mapped
    size_t npix = 0;
    int ctas = 0;
};
static std::mutex g_icp_mutex;
static IcpWorkspace g_icp_ws[64];

static ss_status icp_workspace(int dev, size_t npix, int ctas, IcpWorkspace **out) {
    if (dev < 0 || dev >= 64) return SS_ERR_ARG;
    IcpWorkspace &w = g_icp_ws[dev];
    if (w.npix < npix) {
        cudaFree(w.xp);
        cudaFree(w.ya);
        cudaFree(w.yb);
        w.xp = nullptr;
        w.ya = nullptr;
        w.yb = nullptr;
        w.npix = 0;
        if (cudaMalloc(&w.xp, npix * 12) != cudaSuccess || cudaMalloc(&w.ya, npix * 16) != cudaSuccess ||
            cudaMalloc(&w.yb, npix * 8) != cudaSuccess) {
            cudaGetLastError();
            return SS_ERR_NOMEM;
        }
        w.npix = npix;
    }
    if (w.ctas < ctas || !w.state) {
        cudaFree(w.regions);
        cudaFree(w.state);
        w.regions = nullptr;
        w.state = nullptr;
        w.ctas = 0;
        if (cudaMalloc(&w.regions, (size_t)ctas * sizeof(int4)) != cudaSuccess ||
            cudaMalloc(&w.state, sizeof(IcpState)) != cudaSuccess) {
            cudaGetLastError();
            return SS_ERR_NOMEM;
        }
        w.ctas = ctas;
    }
    if (!w.out_host) {
        if (cudaHostAlloc(&w.out_host, sizeof(IcpOut), cudaHostAllocMapped) != cudaSuccess ||
            cudaHostGetDevicePointer(&w.out_dev, w.out_host, 0) != cudaSuccess) {
            cudaGetLastError();
            if (w.out_host) cudaFreeHost(w.out_host);
            w.out_host = w.out_dev = nullptr;
            return SS_ERR_NOMEM;
        }
    }
    *out = &w;
    return SS_OK;
}

static void inverse4d(const double *m, double *out) {
    double a[4][8];
    for (int r = 0; r < 4; r++)
        for (int c = 0; c < 8; c++) a[r][c] = c < 4 ? m[r * 4 + c] : (c - 4 == r ? 1.0 : 0.0);
    for (int col = 0; col < 4; col++) {
        int piv = col;
        for (int r = col + 1; r < 4; r++)
            if (std::fabs(a[r][col]) > std::fabs(a[piv][col])) piv = r;
        if (piv != col)
            for (int c = 0; c < 8; c++) {
                double t = a[col][c];
                a[col][c] = a[piv][c];
                a[piv][c] = t;
            }
        const double d = a[col][col];
        for (int c = 0; c < 8; c++) a[col][c] /= d;
        for (int r = 0; r < 4; r++) {
            if (r == col) continue;
            const double f = a[r][col];
            for (int c = 0; c < 8; c++) a[r][c] -= f * a[col][c];
        }
    }
    for (int r = 0; r < 4; r++)
        for (int c = 0; c < 4; c++) out[r * 4 + c] = a[r][c + 4];
}

// The rotation block of a 4x4 pose (row-major) made orthogonal to double
// precision: Newton's iteration X <- (X + X^-T) / 2 (X^-T = cofactors / det)
// from the device's polar factor, which the FP32 iteration leaves orthogonal
// to about 1e-7; each step squares the deviation, three are plenty.
static void orthonormalize_rotation(double *T) {
    double X[9];
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) X[r * 3 + c] = T[r * 4 + c];
    for (int it = 0; it < 3; it++) {
        double C[9];
        for (int r = 0; r < 3; r++)
            for (int c = 0; c < 3; c++) {
                const int r1 = (r + 1) % 3, r2 = (r + 2) % 3, c1 = (c + 1) % 3, c2 = (c + 2) % 3;
                C[r * 3 + c] = X[r1 * 3 + c1] * X[r2 * 3 + c2] - X[r1 * 3 + c2] * X[r2 * 3 + c1];
            }
        const double det = X[0] * C[0] + X[1] * C[1] + X[2] * C[2];
        if (!(std::fabs(det) > 0.5)) return;  // not near a rotation: leave it
        for (int k = 0; k < 9; k++) X[k] = 0.5 * (X[k] + C[k] / det);
    }
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) T[r * 4 + c] = X[r * 3 + c];
}

// Runs the 10 iterations on prepared point clouds; shared by the entry points.
// With a host-mapped result (out_host, out_dev) the final iteration writes
// it there and the call ends with a stream synchronisation; without, the
// state is copied back.
ss_status icp_ref_run(const uint16_t *d1, const uint16_t *d2, int rows, int cols, Intr in, const double tx[16],
                      const double ty[16], int type, float *xp, float4 *ya, float2 *yb, int ctas,
                      int4 *regions, IcpState *state, IcpOut *out_host, IcpOut *out_dev, double txy_out[16],
                      float *rmse_out, cudaStream_t s) {
    // Txy = ty^-1 * tx (kokkosICP.cpp:57), float copy for the search
    double tyi[16], T[16];
    inverse4d(ty, tyi);
    for (int r = 0; r < 4; r++)
        for (int c = 0; c < 4; c++) {
            double acc = 0;
            for (int k = 0; k < 4; k++) acc += tyi[r * 4 + k] * tx[k * 4 + c];
            T[r * 4 + c] = acc;
        }
    IcpInit ini;
    for (int k = 0; k < 16; k++) ini.Txy[k] = (float)T[k];
    const dim3 blk(128), grid((cols + 127) / 128, rows);
    icp_prep_kernel<<<grid, blk, 0, s>>>(d1, d2, rows, cols, in, type, xp, ya, yb, ini, state);
    SS_LAUNCH_CHECK();
    const dim3 tiles(icp_tiles_x(cols), icp_tiles_y(rows));  // ctas == tiles.x * tiles.y
    // four CTAs per SM (64 registers, 38 KB of shared memory each) need the
    // largest shared-memory carveout; a hint, so its status is not fatal
    if (type == SS_ICP_POINT_TO_POINT)
        cudaFuncSetAttribute(icp_ref_iter_kernel<SS_ICP_POINT_TO_POINT>, cudaFuncAttributePreferredSharedMemoryCarveout,
                             (int)cudaSharedmemCarveoutMaxShared);
    else
        cudaFuncSetAttribute(icp_ref_iter_kernel<SS_ICP_POINT_TO_PLANE>, cudaFuncAttributePreferredSharedMemoryCarveout,
                             (int)cudaSharedmemCarveoutMaxShared);
    cudaGetLastError();
    // programmatic dependent launches: an iteration's CTAs start while the
    // previous one's last CTA forms the transform (not the first: it loads the
    // source points that the launch before it writes before it waits)
    for (int it = 0; it < kIcpIters; it++) {
        IcpOut *o = it == kIcpIters - 1 ? out_dev : nullptr;
        if (type == SS_ICP_POINT_TO_POINT)
            SS_CUDA_TRY(launch_kernel(icp_ref_iter_kernel<SS_ICP_POINT_TO_POINT>, tiles, dim3(256), 0, s, it > 0, xp, ya,
                                      yb, rows, cols, in, state, regions, (int)(it > 0), o));
        else
            SS_CUDA_TRY(launch_kernel(icp_ref_iter_kernel<SS_ICP_POINT_TO_PLANE>, tiles, dim3(256), 0, s, it > 0, xp, ya,
                                      yb, rows, cols, in, state, regions, (int)(it > 0), o));
    }
    float2 best[16];
    float lowest;
    if (out_host) {
        SS_CUDA_TRY(cudaStreamSynchronize(s));
        const volatile IcpOut *o = out_host;
        for (int k = 0; k < 16; k++) best[k] = make_float2(o->best[k].x, o->best[k].y);
        lowest = o->lowest;
    } else {
        IcpState h;
        SS_CUDA_TRY(cudaMemcpyAsync(&h, state, sizeof(h), cudaMemcpyDeviceToHost, s));
        SS_CUDA_TRY(cudaStreamSynchronize(s));
        for (int k = 0; k < 16; k++) best[k] = h.best[k];
        lowest = h.lowest;
    }
    for (int k = 0; k < 16; k++) txy_out[k] = (double)best[k].x + (double)best[k].y;
    orthonormalize_rotation(txy_out);
    if (rmse_out) *rmse_out = lowest;
    return SS_OK;
}

static ss_status icp_check_args(const uint16_t *d1, const uint16_t *d2, int rows, int cols, float fx, float fy,
                                const double *tx, const double *ty, int type, double *out) {
    if (!d1 || !d2 || !tx || !ty || !out) return SS_ERR_ARG;
    if (rows <= 2 * 5 + 1 || cols <= 2 * 5 + 1) return SS_ERR_DIMS;
    if (type != SS_ICP_POINT_TO_POINT && type != SS_ICP_POINT_TO_PLANE) return SS_ERR_ARG;
    if (!(fx != 0.f) || !(fy != 0.f)) return SS_ERR_ARG;
    return SS_OK;
}

// ------------------------------------------------- allocation-free variant
// Scratch of ss_kokkos_icp_noalloc: the same three point / normal images, staged
// regions and solver state that ss_kokkos_icp takes from its lazily allocated
// workspace, but in one statically sized device array that exists as soon as
// the library is loaded, so the entry point never calls cudaMalloc. Every GPU
// that loads the library holds these bytes until the process exits.
constexpr size_t kNoAllocMaxPixels = 640 * 480;  // largest rows * cols accepted
constexpr int kNoAllocCtas = 4096;  // iteration-grid CTAs (32 x 16 tiles): any rows x cols <= 640 x 480 needs <= 1600
constexpr size_t kAlign256(size_t n) { return (n + 255) / 256 * 256; }
constexpr size_t kNoAllocSource = kAlign256(kNoAllocMaxPixels * 12);  // source points
constexpr size_t kNoAllocTargetA = kAlign256(kNoAllocMaxPixels * 16);  // target (x, y, z, nx)
constexpr size_t kNoAllocTargetB = kAlign256(kNoAllocMaxPixels * 8);   // target (ny, nz)
constexpr size_t kNoAllocImages = kNoAllocSource + kNoAllocTargetA + kNoAllocTargetB;
constexpr size_t kNoAllocRegions = kAlign256((size_t)kNoAllocCtas * sizeof(int4));  // staged region per CTA
constexpr size_t kNoAllocBytes = kNoAllocImages + kNoAllocRegions + kAlign256(sizeof(IcpState));

static __device__ __align__(256) unsigned char g_icp_noalloc_scratch[kNoAllocBytes];

// Device address of the array on each device (the host-side symbol is only a
// stand-in and must never be handed to a kernel). Filled on the first call
// made with that device current and kept for the life of the process: a
// cudaDeviceReset would leave a stale address here, so callers do not reset a
// device they call this entry point on.
static std::mutex g_noalloc_mutex;
static unsigned char *g_noalloc_addr[64] = {};

static ss_status noalloc_scratch(int dev, unsigned char **out) {
    if (dev < 0 || dev >= 64) return SS_ERR_ARG;
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_addr[dev]) {
        void *ptr = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&ptr, g_icp_noalloc_scratch);
        if (e != cudaSuccess || !ptr) {
            set_last_error("cudaGetSymbolAddress(g_icp_noalloc_scratch)", e);
            return SS_ERR_CUDA;
        }
        g_noalloc_addr[dev] = (unsigned char *)ptr;
    }
    *out = g_noalloc_addr[dev];
    return SS_OK;
}

// Test hook kernel: every thread adds its values into the three words; the
// last CTA (by ticket) forms the total like the kokkosICP and differentiable
// raycast last CTAs do.
__global__ void fixed48_sum_kernel(const float *__restrict__ values, int n, unsigned long long *acc, int *ticket,
                                   double *out) {
    __shared__ bool last;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        __int128 q;
        if (fixed48_of_float(values[k], q)) fixed48_add(acc, q);
        else atomicAdd(acc + 3, 1ull);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        const bool l = atomicAdd(ticket, 1) == (int)gridDim.x - 1;
        if (l) __threadfence();
        last = l;
    }
    __syncthreads();
    if (!last || threadIdx.x != 0) return;
    const __int128 t = fixed48_total(__ldcg(acc), __ldcg(acc + 1), __ldcg(acc + 2));
    const float h = icp_float_of_fixed(t);
    __int128 hq;
    fixed48_of_float(h, hq);
    out[0] = f64_of_fixed48(t);
    out[1] = h;
    out[2] = icp_float_of_fixed(t - hq);
    out[3] = (double)__ldcg(acc + 3);
}

}  // namespace ss

using namespace ss;

extern "C" {

ss_status ss_test_fixed48_sum(const float *values, int32_t n, double out[3], ss_stream_t stream) {
    if (n < 0 || !out || (n > 0 && !values)) return SS_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    unsigned char *scratch = nullptr;  // 4 words (the chunks, out-of-range count), a ticket, 4 doubles
    SS_CUDA_TRY(cudaMallocAsync((void **)&scratch, 96, s));
    SS_CUDA_TRY(cudaMemsetAsync(scratch, 0, 96, s));
    fixed48_sum_kernel<<<64, 256, 0, s>>>(values, n, (unsigned long long *)scratch, (int *)(scratch + 32),
                                          (double *)(scratch + 64));
    SS_LAUNCH_CHECK();
    double h[4];
    SS_CUDA_TRY(cudaMemcpyAsync(h, scratch + 64, 4 * sizeof(double), cudaMemcpyDeviceToHost, s));
    SS_CUDA_TRY(cudaFreeAsync(scratch, s));
    SS_CUDA_TRY(cudaStreamSynchronize(s));
    if (h[3] != 0.0) return SS_ERR_ARG;
    out[0] = h[0];
    out[1] = h[1];
    out[2] = h[2];
    return SS_OK;
}

// Same computation and arguments as ss_kokkos_icp, for callers that cannot
// allocate device memory while they run: a tracking thread with a real-time
// budget (cudaMalloc may synchronise the device and take milliseconds), or a
// process whose device memory is handed out by its own pool allocator that
// must stay the only allocator. Images larger than 640 x 480 pixels are
// rejected with SS_ERR_DIMS. The first call on each device looks up the
// scratch array's device address (cudaGetSymbolAddress); make that first call
// before any stream capture. All calls share the one array and it keeps the
// last call's contents: the per-call state is re-initialised by every call,
// and two calls whose work overlaps on the GPU (different streams, or
// different host threads) race on it, so serialise them.
ss_status ss_kokkos_icp_noalloc(const uint16_t *d1, const uint16_t *d2, int32_t rows, int32_t cols, float fx,
                                float fy, float cx, float cy, const double tx[16], const double ty[16],
                                int32_t icp_type, double txy_out[16], float *rmse_out, ss_stream_t stream) {
    ss_status st = icp_check_args(d1, d2, rows, cols, fx, fy, tx, ty, icp_type, txy_out);
    if (st != SS_OK) return st;
    if ((size_t)rows * (size_t)cols > kNoAllocMaxPixels) {
        set_last_error_text("ss_kokkos_icp_noalloc: rows * cols exceeds the 640 x 480 scratch");
        return SS_ERR_DIMS;
    }
    int dev = 0;
    SS_CUDA_TRY(cudaGetDevice(&dev));
    const int ctas = icp_tiles_x(cols) * icp_tiles_y(rows);  // <= 1600 for any image of at most 640 x 480 pixels
    if (ctas > kNoAllocCtas) {
        set_last_error_text("ss_kokkos_icp_noalloc: more 32 x 16 tiles than the scratch holds");
        return SS_ERR_DIMS;
    }
    unsigned char *base = nullptr;
    st = noalloc_scratch(dev, &base);
    if (st != SS_OK) return st;
    float *xp = (float *)base;
    float4 *ya = (float4 *)(base + kNoAllocSource);
    float2 *yb = (float2 *)(base + kNoAllocSource + kNoAllocTargetA);
    int4 *regions = (int4 *)(base + kNoAllocImages);
    IcpState *state = (IcpState *)(base + kNoAllocImages + kNoAllocRegions);
    const Intr in{fx, fy, (float)rows - cy, cx};
    return icp_ref_run(d1, d2, rows, cols, in, tx, ty, icp_type, xp, ya, yb, ctas, regions, state, nullptr,
                       nullptr, txy_out,
                       rmse_out, (cudaStream_t)stream);
}


ss_status ss_depth_to_pcd(const uint16_t *depth, int32_t rows, int32_t cols, float fx, float fy, float cx, float cy,
                          float *pcd, ss_stream_t stream) {
    if (!depth || !pcd || rows <= 0 || cols <= 0) return SS_ERR_ARG;
    const Intr in{fx, fy, (float)rows - cy, cx};
    depth_to_pcd_kernel<<<dim3((cols + 127) / 128, rows), 128, 0, (cudaStream_t)stream>>>(depth, rows, cols, in, pcd);
    SS_LAUNCH_CHECK();
    return SS_OK;
}

ss_status ss_normals_from_pcd(const float *pcd, int32_t rows, int32_t cols, float *normals, ss_stream_t stream) {
    if (!pcd || !normals || rows <= 0 || cols <= 0) return SS_ERR_ARG;
    normals_kernel<<<dim3((cols + 127) / 128, rows), 128, 0, (cudaStream_t)stream>>>(pcd, rows, cols, normals);
    SS_LAUNCH_CHECK();
    return SS_OK;
}

ss_status ss_kokkos_icp(const uint16_t *d1, const uint16_t *d2, int32_t rows, int32_t cols, float fx, float fy,
                        float cx, float cy, const double tx[16], const double ty[16], int32_t icp_type,
                        double txy_out[16], float *rmse_out, ss_stream_t stream) {
    ss_status st = icp_check_args(d1, d2, rows, cols, fx, fy, tx, ty, icp_type, txy_out);
    if (st != SS_OK) return st;
    int dev = 0;
    SS_CUDA_TRY(cudaGetDevice(&dev));
    const int ctas = icp_tiles_x(cols) * icp_tiles_y(rows);
    std::lock_guard<std::mutex> lock(g_icp_mutex);
    IcpWorkspace *w = nullptr;
    st = icp_workspace(dev, (size_t)rows * cols, ctas, &w);
    if (st != SS_OK) return st;
    const Intr in{fx, fy, (float)rows - cy, cx};  // ci = resi - cy, cj = cx (kokkosICP.cpp:48-49)
    return icp_ref_run(d1, d2, rows, cols, in, tx, ty, icp_type, w->xp, w->ya, w->yb, ctas, w->regions,
                       w->state, w->out_host, w->out_dev,
                       txy_out, rmse_out, (cudaStream_t)stream);
}

}  // extern "C"
