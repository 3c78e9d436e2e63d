// ss_ref_math.h — reference-rounding helpers shared by the oracle files.
// TEST INFRASTRUCTURE ONLY (see ss_oracle.cpp's header).
#pragma once

#include <cmath>
#include <cstdint>

namespace orc {

constexpr int kEdge = 8;
constexpr int kVox = 512;
constexpr int kCoordBias = 8192;  // packable block coordinate range [-8192, 8191]

struct V3 {
    float x, y, z;
};
struct I3 {
    int x, y, z;
};

// Kvec3f operators (src/VoxelGrid/kokkosFunctions.h:187-247, 265-268)
inline V3 sub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 add(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 smul(float a, V3 b) { return {a * b.x, a * b.y, a * b.z}; }
inline float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(V3 a, V3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
inline float length(V3 a) { return std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
inline V3 normalized(V3 a) {
    float t = length(a);
    return {a.x / t, a.y / t, a.z / t};
}

// (int) cast as executed by the reference's CUDA build (cvt.rzi.s32.f32).
inline int f2i(float f) {
    if (std::isnan(f)) return 0;
    if (f >= 2147483648.0f) return 2147483647;
    if (f < -2147483648.0f) return (-2147483647 - 1);
    return (int)f;
}

// transformPoint (GPUVoxelGrid.h:240-247) / Kmat4f * Kvec3f (kokkosFunctions.h:713-722)
inline V3 xform(const float *E, V3 p) {
    V3 o;
    o.x = p.x * E[0] + p.y * E[1] + p.z * E[2] + E[3];
    o.y = p.x * E[4] + p.y * E[5] + p.z * E[6] + E[7];
    o.z = p.x * E[8] + p.y * E[9] + p.z * E[10] + E[11];
    return o;
}

// getPrimeHash (GPUVoxelGrid.h:124-128): int arithmetic, wrapped, then
// converted to unsigned long long (sign extension).
inline uint64_t prime_hash(int x, int y, int z) {
    uint32_t h = 73856093u * (uint32_t)x + 19349669u * (uint32_t)y + 83492791u * (uint32_t)z;
    return (uint64_t)(int64_t)(int32_t)h;
}

// Index rule of getIndeces / getVBIndeces / getVinVBIndeces (GPUVoxelGrid.h:131-221).
inline int idx_rule(float a, float len) {
    if (a >= 0) return f2i(a / len);
    return f2i(a / len - 1);
}

inline uint64_t pack_coords(int x, int y, int z) {
    return ((uint64_t)(uint32_t)(x + kCoordBias) << 28) |
           ((uint64_t)(uint32_t)(y + kCoordBias) << 14) | (uint64_t)(uint32_t)(z + kCoordBias);
}
inline I3 unpack_coords(uint64_t p) {
    return {(int)((p >> 28) & 0x3fff) - kCoordBias, (int)((p >> 14) & 0x3fff) - kCoordBias,
            (int)(p & 0x3fff) - kCoordBias};
}
inline bool packable(int x, int y, int z) {
    return x >= -kCoordBias && x < kCoordBias && y >= -kCoordBias && y < kCoordBias &&
           z >= -kCoordBias && z < kCoordBias;
}

}  // namespace orc
