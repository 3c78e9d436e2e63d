// ss_internal.cuh — device-side building blocks shared by the kernels.
//
// Reference-order arithmetic: the parity kernels evaluate every expression of
// the reference (src/VoxelGrid/GPUVoxelGrid.{h,cpp}) with explicit
// round-to-nearest intrinsics (__fmul_rn, __fadd_rn, __fdiv_rn ...), so nvcc
// cannot contract them into FMAs and the results are those of the C++
// expressions evaluated in IEEE single precision, operand by operand.
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/ss_abi.h"

namespace ss {

constexpr int kEdge = 8;          // voxelPerEdge (GPUVoxelGrid.h:6)
constexpr int kBlockVoxels = 512; // voxelPerBlock (GPUVoxelGrid.h:8)

// Hash-table key domain: the reference's key is an int32 sign-extended to
// u64, so the upper 32 bits are all-zero or all-one. These two words have
// upper bits zero and bit 31 set, which no key can have.
constexpr uint64_t kEmptyKey = 0x00000000FFFFFFFFull;
constexpr uint64_t kTombKey = 0x00000000FFFFFFFEull;

// Block stamp word: [63:42] epoch of the last call that touched the block,
// [41:28] x+8192, [27:14] y+8192, [13:0] z+8192.
constexpr int kCoordBias = 8192;
constexpr int kEpochShift = 42;
constexpr uint32_t kEpochMax = (1u << 22) - 1;

// Device status word bits (ORed; mapped to the first ss_status by the host).
enum : int {
    kStTableFull = 1 << 0,
    kStListOverflow = 1 << 1,
    kStRange = 1 << 2,
    kStTimeout = 1 << 3,
};

// Device-resident counters of one grid (one 128-byte line).
struct Counters {
    int list_count;                   // touched blocks of the current call
    int status;                       // kSt* bits
    uint32_t epoch;                   // current call epoch (1 .. kEpochMax)
    int work;                         // dynamic work index for persistent kernels
    int live_blocks;                  // allocated blocks (maintained by insert / clean)
    int last_touched;                 // list_count of the previous call
    unsigned long long touched_total; // sum of list_count over all calls
    unsigned long long calls;         // integrate/deintegrate calls finalized
    unsigned long long ray_finds;     // hash finds of the reference-semantics raycast (all calls)
    unsigned long long ray_voxels;    // voxel (sdf, w) reads of the reference-semantics raycast (all calls)
    int sb_lo[3], sb_hi[3];           // bounding box of the marked super-blocks (empty: lo > hi)
    int pad[12];
};
static_assert(sizeof(Counters) == 128, "Counters is one 128-byte line");

struct Intr {
    float fx, fy, ci, cj;  // ci = resi - cy, cj = cx (GPUVoxelGrid.cpp:257-262)
};

struct Mat34 {
    float m[12];  // row-major 3x4 affine part of a 4x4 float matrix
};

// Pose of one integrate/raycast call as the kernels consume it. Host-side
// calls pass it by value; the per-frame pipeline keeps it in device memory
// (written by the tracker) and passes a pointer, so no host round trip is
// needed between tracking and fusion.
struct __align__(16) FramePose {  // 16-byte aligned: a kernel loads E or Einv as three float4
    Mat34 E;     // camera -> world, float (the reference's E view)
    Mat34 Einv;  // world -> camera, float (E_inv)
    float Ez[3]; // normalized third column of E
    float pad;
};

__device__ __forceinline__ void load_pose(const FramePose *p, Mat34 &E, Mat34 &Einv, float &ezx, float &ezy,
                                          float &ezz) {
#pragma unroll
    for (int k = 0; k < 12; k++) {
        E.m[k] = __ldg(&p->E.m[k]);
        Einv.m[k] = __ldg(&p->Einv.m[k]);
    }
    ezx = __ldg(&p->Ez[0]);
    ezy = __ldg(&p->Ez[1]);
    ezz = __ldg(&p->Ez[2]);
}

// View of one grid passed by value to kernels.
struct GridView {
    unsigned long long *keys;   // [buckets] u64 prime-hash keys
    unsigned long long *stamp;  // [buckets] epoch | packed block coords
    float2 *vox32;              // [buckets][512] (sdf, w)     SS_STORAGE_F32
    uint32_t *vox16;            // [buckets][512] half(sdf/trunc) | u16 w << 16   SS_STORAGE_F16
    float *rgb;                 // [buckets][3][512] or null
    int *list;                  // [buckets] touched bucket indices
    Counters *ctr;
    unsigned long long *sbkeys; // [sb_buckets] occupied super-blocks (8^3 blocks) for empty-space skipping
    uint32_t sbmask;            // sb_buckets - 1
    uint32_t mask;              // buckets - 1
    float vl, vbl, trunc, rmin, d_max, max_weight;
    float rvbl;  // RN(1 / vbl), computed on the host
    float rvl;   // RN(1 / vl), computed on the host
    int resi, resj;
    Intr in;
    // getPoint's per-column and per-row quotients (j - cj) / fx and
    // (i - ci) / fy in IEEE float, computed on the host when the intrinsics
    // are set (the same roundings as the device expression)
    const float *ray_u, *ray_v;  // [resj], [resi]
};

// ------------------------------------------------------------------ math
struct F3 {
    float x, y, z;
};

__device__ __forceinline__ F3 f3sub(F3 a, F3 b) {
    return {__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y), __fsub_rn(a.z, b.z)};
}
__device__ __forceinline__ F3 f3add(F3 a, F3 b) {
    return {__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y), __fadd_rn(a.z, b.z)};
}
__device__ __forceinline__ F3 f3smul(float a, F3 b) {
    return {__fmul_rn(a, b.x), __fmul_rn(a, b.y), __fmul_rn(a, b.z)};
}
// Kvec3f scalar product x*a.x + y*a.y + z*a.z (kokkosFunctions.h:211-214)
__device__ __forceinline__ float f3dot(F3 a, F3 b) {
    return __fadd_rn(__fadd_rn(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)), __fmul_rn(a.z, b.z));
}
__device__ __forceinline__ F3 f3cross(F3 a, F3 b) {
    return {__fsub_rn(__fmul_rn(a.y, b.z), __fmul_rn(a.z, b.y)),
            __fsub_rn(__fmul_rn(a.z, b.x), __fmul_rn(a.x, b.z)),
            __fsub_rn(__fmul_rn(a.x, b.y), __fmul_rn(a.y, b.x))};
}
__device__ __forceinline__ float f3len(F3 a) { return __fsqrt_rn(f3dot(a, a)); }
__device__ __forceinline__ F3 f3normalized(F3 a) {
    float t = f3len(a);
    return {__fdiv_rn(a.x, t), __fdiv_rn(a.y, t), __fdiv_rn(a.z, t)};
}

// transformPoint (GPUVoxelGrid.h:240-247): ((p.x*E0 + p.y*E1) + p.z*E2) + E3
__device__ __forceinline__ F3 xform(const Mat34 &E, F3 p) {
    F3 o;
    o.x = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(p.x, E.m[0]), __fmul_rn(p.y, E.m[1])), __fmul_rn(p.z, E.m[2])), E.m[3]);
    o.y = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(p.x, E.m[4]), __fmul_rn(p.y, E.m[5])), __fmul_rn(p.z, E.m[6])), E.m[7]);
    o.z = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(p.x, E.m[8]), __fmul_rn(p.y, E.m[9])), __fmul_rn(p.z, E.m[10])), E.m[11]);
    return o;
}

// getPoint from the grid's quotient tables: bit-identical to get_point.
__device__ __forceinline__ F3 get_point_t(const GridView &g, int i, int j, float d) {
    return {__fmul_rn(__ldg(g.ray_u + j), d), __fmul_rn(__ldg(g.ray_v + i), d), d};
}

// getPoint (GPUVoxelGrid.h:229-232): ((j - cj)/fx*d, (i - ci)/fy*d, d)
__device__ __forceinline__ F3 get_point(const Intr &in, int i, int j, float d) {
    return {__fmul_rn(__fdiv_rn(__fsub_rn((float)j, in.cj), in.fx), d),
            __fmul_rn(__fdiv_rn(__fsub_rn((float)i, in.ci), in.fy), d), d};
}

// (float)(depth) / 1000 (GPUVoxelGrid.h:306), the IEEE quotient, as
// q0 = RN(d y) with y = RN(1/1000), then one residual correction
// q = RN(q0 + RN(d - q0 1000) y) (the remainder d - q0 1000 is exact in one
// fma). Equal to the correctly rounded quotient for every u16 d: the whole
// input range is checked in exact arithmetic (tests/test_device_arith.py).
__device__ __forceinline__ float depth_m(uint16_t d) {
    const float a = (float)d, y = 1.0e-3f;
    const float q0 = __fmul_rn(a, y);
    return __fmaf_rn(__fmaf_rn(-q0, 1000.f, a), y, q0);
}

// Index rule of getIndeces / getVBIndeces / getVinVBIndeces
// (GPUVoxelGrid.h:131-221): a >= 0 ? (int)(a/len) : (int)(a/len - 1).
// __float2int_rz is the (int) cast of the reference's device build. Not
// inlined: the hot paths take it only where the multiplication form
// (idx_fast) is not decisive, and its IEEE division inlined at every call site
// made the reference raycast's loops larger than the instruction cache likes
// (0.354 -> 0.336 ms per ss_raycast call as a called function).
static __device__ __noinline__ int idx_rule(float a, float len) {
    float q = __fdiv_rn(a, len);
    return a >= 0.f ? __float2int_rz(q) : __float2int_rz(__fsub_rn(q, 1.f));
}

// idx_rule with the quotient taken as q1 = a * rlen, rlen = RN(1 / len), where
// that gives the same result: q1 is within 3.02 u |q1| of the IEEE quotient
// q = RN(a / len) (u = 2^-24: three roundings), and RN(q - 1) within a
// further u (|q1| + 1) of q - 1, so when q1 lies more than 5 u (|q1| + 1)
// from every integer, no integer separates q from q1 or RN(q - 1) from
// RN(q1 - 1), and the truncations agree; both are then floor(q1) (a >= 0:
// q1 >= 0 is no integer; a < 0: neither is RN(q1 - 1), which truncates to
// floor(q1)). idx_fast returns false where q1 is too close to an integer (and
// for zero, huge or non-finite values): there the IEEE division decides.
__device__ __forceinline__ bool idx_fast(float a, float rlen, int &out) {
    const float q1 = __fmul_rn(a, rlen);
    out = __float2int_rd(q1);
    return fabsf(__fsub_rn(q1, rintf(q1))) > __fmaf_rn(fabsf(q1), 3.0e-7f, 3.0e-7f);  // > 5 u (|q1| + 1)
}

// idx_rule(a, len) through idx_fast where that is decisive (rlen = RN(1 / len)).
__device__ __forceinline__ int idx_rule_fast(float a, float len, float rlen) {
    int o;
    return idx_fast(a, rlen, o) ? o : idx_rule(a, len);
}

// The block range of a point's truncation band: idx_rule of its corners lo
// and hi, six multiplications and one check for all six; the six IEEE
// divisions only when some quotient is too close to an integer (a few
// pixels per million).
__device__ __forceinline__ void block_range(F3 lo, F3 hi, float len, float rlen, int &lx, int &ly, int &lz, int &hx,
                                            int &hy, int &hz) {
    const bool ok = idx_fast(lo.x, rlen, lx) & idx_fast(lo.y, rlen, ly) & idx_fast(lo.z, rlen, lz) &
                    idx_fast(hi.x, rlen, hx) & idx_fast(hi.y, rlen, hy) & idx_fast(hi.z, rlen, hz);
    if (!ok) {
        lx = idx_rule(lo.x, len);
        ly = idx_rule(lo.y, len);
        lz = idx_rule(lo.z, len);
        hx = idx_rule(hi.x, len);
        hy = idx_rule(hi.y, len);
        hz = idx_rule(hi.z, len);
    }
}

// getPrimeHash (GPUVoxelGrid.h:124-128), int wrap, sign-extended to u64.
__device__ __forceinline__ unsigned long long prime_hash(int x, int y, int z) {
    uint32_t h = 73856093u * (uint32_t)x + 19349669u * (uint32_t)y + 83492791u * (uint32_t)z;
    return (unsigned long long)(long long)(int32_t)h;
}

__device__ __forceinline__ bool packable(int x, int y, int z) {
    return x >= -kCoordBias && x < kCoordBias && y >= -kCoordBias && y < kCoordBias && z >= -kCoordBias &&
           z < kCoordBias;
}
__device__ __forceinline__ unsigned long long pack_coords(int x, int y, int z) {
    return ((unsigned long long)(uint32_t)(x + kCoordBias) << 28) |
           ((unsigned long long)(uint32_t)(y + kCoordBias) << 14) | (unsigned long long)(uint32_t)(z + kCoordBias);
}
__device__ __forceinline__ void unpack_coords(unsigned long long p, int &x, int &y, int &z) {
    x = (int)((p >> 28) & 0x3fff) - kCoordBias;
    y = (int)((p >> 14) & 0x3fff) - kCoordBias;
    z = (int)(p & 0x3fff) - kCoordBias;
}

// Home bucket: murmur3 finalizer of the low key word (the prime hash is
// linear in the coordinates, so neighbouring blocks need mixing).
__device__ __forceinline__ uint32_t home_bucket(unsigned long long key, uint32_t mask) {
    uint32_t h = (uint32_t)key;
    h ^= h >> 16;
    h *= 0x85ebca6bu;
    h ^= h >> 13;
    h *= 0xc2b2ae35u;
    h ^= h >> 16;
    return h & mask;
}

__device__ __forceinline__ unsigned long long ld_relaxed(const unsigned long long *p) {
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ uint32_t ld_relaxed_u32(const uint32_t *p) {
    uint32_t v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Lookup only (UnorderedMap::find): bucket index or -1. Tombstones continue
// the probe, an empty bucket ends it. Read-only kernels see a table that no
// other kernel is modifying, so plain loads suffice.
__device__ __forceinline__ int table_find(const GridView &g, unsigned long long key) {
    uint32_t b = home_bucket(key, g.mask);
    for (uint32_t probe = 0; probe <= g.mask; probe++) {
        unsigned long long k = __ldg(g.keys + b);
        if (k == key) return (int)b;
        if (k == kEmptyKey) return -1;
        b = (b + 1) & g.mask;
    }
    return -1;
}

// Lock-free find-or-insert (UnorderedMap::find + insert,
// GPUVoxelGrid.cpp:493-499). Returns the bucket, or -1 with kStTableFull set.
// Inserts claim the first tombstone or the terminating empty bucket of the
// probe sequence with one 64-bit CAS and re-scan when the CAS loses. The
// payload of a free bucket is always zero (create/reset/clean keep it so), so
// a claimed bucket is a default-constructed Voxelblock.
__device__ __forceinline__ int table_find_or_insert(const GridView &g, unsigned long long key,
                                                    bool *inserted = nullptr) {
    const uint32_t home = home_bucket(key, g.mask);
    for (int attempt = 0; attempt < 64; attempt++) {
        int free_b = -1;
        unsigned long long free_expect = 0;
        uint32_t b = home;
        uint32_t probe = 0;
        for (; probe <= g.mask; probe++) {
            unsigned long long k = ld_relaxed(g.keys + b);
            if (k == key) return (int)b;
            if (k == kTombKey && free_b < 0) {
                free_b = (int)b;
                free_expect = kTombKey;
            }
            if (k == kEmptyKey) {
                if (free_b < 0) {
                    free_b = (int)b;
                    free_expect = kEmptyKey;
                }
                break;
            }
            b = (b + 1) & g.mask;
        }
        if (free_b < 0) break;
        unsigned long long old = atomicCAS(g.keys + free_b, free_expect, key);
        if (old == free_expect) {
            atomicAdd(&g.ctr->live_blocks, 1);
            if (inserted) *inserted = true;
            return free_b;
        }
        if (old == key) return free_b;
    }
    atomicOr(&g.ctr->status, kStTableFull);
    return -1;
}

// ---------------------------------------------------------- super-blocks
// A super-block is 8x8x8 blocks (coordinates b >> 3); the set of super-blocks
// holding at least one allocated block lets a ray skip 8 blocks at a time
// through empty space. Kept as a small open-addressing set of packed
// coordinates; inserts are idempotent, entries are only removed by a rebuild.
constexpr int kSuperShift = 3;
constexpr unsigned long long kSuperEmpty = ~0ull;

__device__ __forceinline__ unsigned long long super_key(int sx, int sy, int sz) {
    return ((unsigned long long)(uint32_t)(sx + 1024) << 22) | ((unsigned long long)(uint32_t)(sy + 1024) << 11) |
           (unsigned long long)(uint32_t)(sz + 1024);
}
__device__ __forceinline__ uint32_t super_home(unsigned long long key, uint32_t mask) {
    uint32_t h = (uint32_t)(key ^ (key >> 29)) * 0x9E3779B1u;
    h ^= h >> 15;
    return h & mask;
}
__device__ __forceinline__ void super_insert(const GridView &g, int bx, int by, int bz) {
    const unsigned long long key = super_key(bx >> kSuperShift, by >> kSuperShift, bz >> kSuperShift);
    uint32_t b = super_home(key, g.sbmask);
    for (uint32_t probe = 0; probe <= g.sbmask; probe++) {
        const unsigned long long k = ld_relaxed(g.sbkeys + b);
        if (k == key) return;
        if (k == kSuperEmpty) {
            const unsigned long long old = atomicCAS(g.sbkeys + b, kSuperEmpty, key);
            if (old == kSuperEmpty) {  // a new super-block: grow the bounding box
                const int sx = bx >> kSuperShift, sy = by >> kSuperShift, sz = bz >> kSuperShift;
                atomicMin(&g.ctr->sb_lo[0], sx);
                atomicMin(&g.ctr->sb_lo[1], sy);
                atomicMin(&g.ctr->sb_lo[2], sz);
                atomicMax(&g.ctr->sb_hi[0], sx);
                atomicMax(&g.ctr->sb_hi[1], sy);
                atomicMax(&g.ctr->sb_hi[2], sz);
                return;
            }
            if (old == key) return;
        }
        b = (b + 1) & g.sbmask;
    }
    atomicOr(&g.ctr->status, kStTableFull);
}
__device__ __forceinline__ bool super_occupied(const GridView &g, int sx, int sy, int sz) {
    const unsigned long long key = super_key(sx, sy, sz);
    uint32_t b = super_home(key, g.sbmask);
    for (uint32_t probe = 0; probe <= g.sbmask; probe++) {
        const unsigned long long k = __ldg(g.sbkeys + b);
        if (k == key) return true;
        if (k == kSuperEmpty) return false;
        b = (b + 1) & g.sbmask;
    }
    return false;
}

__device__ __forceinline__ int lane_id() { return threadIdx.x & 31; }

// Programmatic dependent launch. A kernel launched with the programmatic
// stream-serialization attribute may start while the kernel before it in the
// stream is still running; pdl_wait() then blocks until that kernel has
// completed and its memory is visible, so a kernel calls it before it reads
// (or writes) anything the previous kernel writes (or reads). pdl_trigger()
// lets the next kernel launch once every CTA of this one has called it or
// exited. Both are no-ops for an ordinary launch.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// Packed pairs of floats (a 64-bit register pair: lane 0 in the low half)
// and the paired FP32 instructions of this architecture: each half rounded to
// nearest as the scalar instruction would, so one instruction does the arithmetic of two
// independent values.
typedef unsigned long long f32x2;
__device__ __forceinline__ f32x2 f2_pack(float lo, float hi) {
    f32x2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}
__device__ __forceinline__ void f2_unpack(f32x2 v, float &lo, float &hi) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}
__device__ __forceinline__ f32x2 f2_sub(f32x2 a, f32x2 b) {
    f32x2 r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f32x2 f2_mul(f32x2 a, f32x2 b) {
    f32x2 r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f32x2 f2_add(f32x2 a, f32x2 b) {
    f32x2 r;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}

// Exact cross-CTA sums in fixed point (resolution 2^-48): a CTA's float
// value becomes a signed integer below 2^95 in magnitude, added as three
// 32-bit chunks (two unsigned, the top one signed) into three 64-bit words
// with integer atomics, so the total does not depend on the order in which
// the CTAs arrive (fewer than 2^10 CTAs add less than 2^42 to a word: no
// carry leaves it). All by integer operations: this part's FP64 pipe takes
// conversions at FMA latency.
constexpr int kFix48 = 48;

// f 2^48 truncated toward zero, for |f| < 2^47 (false otherwise, NaN included).
__device__ __forceinline__ bool fixed48_of_float(float f, __int128 &q) {
    q = 0;
    if (!(fabsf(f) < 0x1p47f)) return false;
    const unsigned u = __float_as_uint(f);
    const int ex = (int)((u >> 23) & 0xffu);
    if (ex == 0) return true;  // zero or subnormal: below the resolution
    const unsigned long long m = (u & 0x7fffffu) | 0x800000u;  // f = m 2^(ex - 150)
    const int sh = ex - 150 + kFix48;                          // < 71: m 2^sh < 2^95
    __int128 mag = 0;
    if (sh >= 0)
        mag = (__int128)m << sh;
    else if (sh > -24)
        mag = (__int128)(m >> -sh);
    q = (u >> 31) ? -mag : mag;
    return true;
}

// Adds the fixed-point value q into its three words w[0..2].
__device__ __forceinline__ void fixed48_add(unsigned long long *w, __int128 q) {
    atomicAdd(w, (unsigned long long)q & 0xffffffffull);
    atomicAdd(w + 1, (unsigned long long)(q >> 32) & 0xffffffffull);
    atomicAdd(w + 2, (unsigned long long)(long long)(q >> 64));
}

// The total held by three words (their sums of chunks) as a 128-bit integer.
__device__ __forceinline__ __int128 fixed48_total(unsigned long long s0, unsigned long long s1,
                                                  unsigned long long s2) {
    const unsigned __int128 u = ((unsigned __int128)(__int128)(long long)s2 << 64) + ((unsigned __int128)s1 << 32) + s0;
    return (__int128)u;  // two's complement: the top word's sign
}

// t 2^-48 rounded to the nearest double (ties to even), |t| < 2^127.
__device__ __forceinline__ double f64_of_fixed48(__int128 t) {
    if (t == 0) return 0.0;
    const bool neg = t < 0;
    unsigned __int128 m = neg ? (unsigned __int128)(-t) : (unsigned __int128)t;
    const unsigned long long mh = (unsigned long long)(m >> 64), ml = (unsigned long long)m;
    const int lz = mh ? __clzll((long long)mh) : 64 + __clzll((long long)ml);
    m <<= lz;  // the leading one at bit 127
    const unsigned long long th = (unsigned long long)(m >> 64), tl = (unsigned long long)m;
    unsigned long long mant = th >> 11;  // 53 bits
    int ex = 127 - lz - kFix48 + 1023;
    if (((th >> 10) & 1ull) && ((th & 0x3ffull) || tl || (mant & 1ull))) {
        if (++mant >> 53) {
            mant >>= 1;
            ex++;
        }
    }
    return __longlong_as_double((long long)((neg ? 0x8000000000000000ull : 0ull) | ((unsigned long long)ex << 52) |
                                            (mant & 0xfffffffffffffull)));
}

}  // namespace ss
