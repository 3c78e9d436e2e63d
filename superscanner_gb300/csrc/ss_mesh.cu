// ss_mesh.cu — triangle mesh of the TSDF's zero level set on the GPU.
//
// The reference meshes the volume on the host: marchingCubesHost
// (GPUVoxelGrid.cpp:200-251) copies every block to the host into an Open3D
// ScalableTSDFVolume and runs its marching cubes. Here the mesh is extracted
// where the volume lives, by marching tetrahedra (a published method: each
// cell of 8 voxel centres is split into the 6 tetrahedra of the Freudenthal
// subdivision along the diagonal from corner 0 to corner 7; the split is the
// same in every cell, so neighbouring cells agree on their shared faces and
// the surface has no cracks; each tetrahedron has 16 sign cases, handled in
// code). A cell counts only where all 8 voxels are observed (weight > 0).
// Vertices lie on tetrahedron edges whose ends change sign (sdf < 0 is
// inside), linearly interpolated; triangles face from negative to positive
// sdf (out of the surface). Output: a triangle soup in world coordinates.
//
// One CTA per bucket of the hash table (grid-stride; empty buckets are
// skipped by the whole CTA), 256 threads x 2 cells per block; the up to 7
// neighbouring blocks a block's last row of cells reaches into are looked up
// once per CTA. Each triangle is appended with one atomic on the counter.
#include "ss_grid_impl.cuh"
#include "ss_mc_table.h"
#include "ss_trilinear.cuh"

namespace ss {

// The 6 tetrahedra (corner indices n = dx + 2 dy + 4 dz): 0 -> e_a -> e_a + e_b -> 7 for each axis order.
__constant__ int kTet[6][4] = {{0, 1, 3, 7}, {0, 1, 5, 7}, {0, 2, 3, 7}, {0, 2, 6, 7}, {0, 4, 5, 7}, {0, 4, 6, 7}};

struct MeshOut {
    float *tris;                // [cap][9]
    unsigned long long *count;  // total triangles (may exceed cap)
    unsigned long long cap;
};

__device__ __forceinline__ F3 edge_point(const F3 &p, float sp, const F3 &q, float sq) {
    const float t = sp / (sp - sq);
    return F3{fmaf(t, q.x - p.x, p.x), fmaf(t, q.y - p.y, p.y), fmaf(t, q.z - p.z, p.z)};
}

// Appends triangle (a, b, c), flipped if needed so that its normal points
// along dir (from the tetrahedron's inside corners to its outside corners).
__device__ __forceinline__ void emit(const MeshOut &o, F3 a, F3 b, F3 c, const F3 &dir) {
    const float ux = b.x - a.x, uy = b.y - a.y, uz = b.z - a.z, vx = c.x - a.x, vy = c.y - a.y, vz = c.z - a.z;
    const float nx = uy * vz - uz * vy, ny = uz * vx - ux * vz, nz = ux * vy - uy * vx;
    if (nx * dir.x + ny * dir.y + nz * dir.z < 0.f) {
        const F3 t = b;
        b = c;
        c = t;
    }
    const unsigned long long at = atomicAdd(o.count, 1ull);
    if (at >= o.cap) return;
    float *d = o.tris + at * 9;
    d[0] = a.x, d[1] = a.y, d[2] = a.z, d[3] = b.x, d[4] = b.y, d[5] = b.z, d[6] = c.x, d[7] = c.y, d[8] = c.z;
}

__device__ void tetra(const MeshOut &o, const F3 *p, const float *s, const int *t) {
    int in[4], out[4], ni = 0, no = 0;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        if (s[t[k]] < 0.f) in[ni++] = t[k];
        else out[no++] = t[k];
    }
    if (ni == 0 || ni == 4) return;
    F3 ci{0.f, 0.f, 0.f}, co{0.f, 0.f, 0.f};
    for (int k = 0; k < ni; k++) ci = F3{ci.x + p[in[k]].x, ci.y + p[in[k]].y, ci.z + p[in[k]].z};
    for (int k = 0; k < no; k++) co = F3{co.x + p[out[k]].x, co.y + p[out[k]].y, co.z + p[out[k]].z};
    const F3 dir{co.x / no - ci.x / ni, co.y / no - ci.y / ni, co.z / no - ci.z / ni};
    if (ni == 1 || ni == 3) {
        const int a = ni == 1 ? in[0] : out[0];
        const int *r = ni == 1 ? out : in;  // the three other corners
        emit(o, edge_point(p[a], s[a], p[r[0]], s[r[0]]), edge_point(p[a], s[a], p[r[1]], s[r[1]]),
             edge_point(p[a], s[a], p[r[2]], s[r[2]]), dir);
    } else {  // two inside (a, b), two outside (c, d): the quad ac, ad, bd, bc
        const int a = in[0], b = in[1], c = out[0], d = out[1];
        const F3 ac = edge_point(p[a], s[a], p[c], s[c]), ad = edge_point(p[a], s[a], p[d], s[d]);
        const F3 bd = edge_point(p[b], s[b], p[d], s[d]), bc = edge_point(p[b], s[b], p[c], s[c]);
        emit(o, ac, ad, bd, dir);
        emit(o, ac, bd, bc, dir);
    }
}

template <int kStorage>
__global__ void __launch_bounds__(256) mesh_kernel(GridView g, MeshOut o) {
    __shared__ int nb[8];  // bucket of block (bx + (n & 1), by + (n >> 1 & 1), bz + (n >> 2)); -1 missing
    __shared__ int bc[3];
    for (uint32_t bucket = blockIdx.x; bucket <= g.mask; bucket += gridDim.x) {
        const unsigned long long key = g.keys[bucket];
        if (key == kEmptyKey || key == kTombKey) continue;  // uniform over the CTA
        __syncthreads();  // the previous block's cells are done with nb
        if (threadIdx.x == 0) {
            int x, y, z;
            unpack_coords(g.stamp[bucket] & ((1ull << kEpochShift) - 1ull), x, y, z);
            bc[0] = x, bc[1] = y, bc[2] = z;
            nb[0] = (int)bucket;
        }
        __syncthreads();
        if (threadIdx.x >= 1 && threadIdx.x < 8) {
            const int n = threadIdx.x, x = bc[0] + (n & 1), y = bc[1] + ((n >> 1) & 1), z = bc[2] + (n >> 2);
            nb[n] = packable(x, y, z) ? table_find(g, prime_hash(x, y, z)) : -1;
        }
        __syncthreads();
        for (int c = threadIdx.x; c < kBlockVoxels; c += blockDim.x) {
            const int i = c & 7, j = (c >> 3) & 7, k = c >> 6;
            F3 p[8];
            float s[8];
            bool ok = true;
#pragma unroll
            for (int n = 0; n < 8; n++) {
                const int vi = i + (n & 1), vj = j + ((n >> 1) & 1), vk = k + (n >> 2);
                const int b = nb[(vi >> 3) + 2 * (vj >> 3) + 4 * (vk >> 3)];
                if (b < 0) {
                    ok = false;
                    break;
                }
                const float2 sw = voxel_sw<kStorage>(g, b, (vi & 7) + 8 * (vj & 7) + 64 * (vk & 7));
                if (!(sw.y > 0.f)) {
                    ok = false;
                    break;
                }
                s[n] = sw.x;
                // voxel centre (pzero + (index + 0.5) vl, GPUVoxelGrid.cpp:521)
                p[n] = F3{((float)(bc[0] * 8 + vi) + 0.5f) * g.vl, ((float)(bc[1] * 8 + vj) + 0.5f) * g.vl,
                          ((float)(bc[2] * 8 + vk) + 0.5f) * g.vl};
            }
            if (!ok) continue;
#pragma unroll 1
            for (int t = 0; t < 6; t++) tetra(o, p, s, kTet[t]);
        }
    }
}

// ---------------------------------------------------------- marching cubes
// The case table (ss_mc_table.h) in global memory, read through the
// read-only cache (the lanes of a warp hold different cases).
__device__ const McTable g_mc_table = kMcTable;

// Marching cubes over the same cells as mesh_kernel: corner m of the table
// (x + y, ... order of ss_mc_table.h) is cell corner n = dx + 2 dy + 4 dz.
__constant__ int kMcCornerCell[8] = {0, 1, 3, 2, 4, 5, 7, 6};
// The end of each table edge with the lower coordinate: a vertex is
// interpolated from that end, so the cubes sharing an edge compute it alike.
__constant__ int kMcEdgeLo[12] = {0, 1, 3, 0, 4, 5, 7, 4, 0, 1, 2, 3};
__constant__ int kMcEdgeHi[12] = {1, 2, 2, 3, 5, 6, 6, 7, 4, 5, 6, 7};

template <int kStorage>
__global__ void __launch_bounds__(256) mesh_mc_kernel(GridView g, MeshOut o) {
    __shared__ int nb[8];
    __shared__ int bc[3];
    for (uint32_t bucket = blockIdx.x; bucket <= g.mask; bucket += gridDim.x) {
        const unsigned long long key = g.keys[bucket];
        if (key == kEmptyKey || key == kTombKey) continue;  // uniform over the CTA
        __syncthreads();
        if (threadIdx.x == 0) {
            int x, y, z;
            unpack_coords(g.stamp[bucket] & ((1ull << kEpochShift) - 1ull), x, y, z);
            bc[0] = x, bc[1] = y, bc[2] = z;
            nb[0] = (int)bucket;
        }
        __syncthreads();
        if (threadIdx.x >= 1 && threadIdx.x < 8) {
            const int n = threadIdx.x, x = bc[0] + (n & 1), y = bc[1] + ((n >> 1) & 1), z = bc[2] + (n >> 2);
            nb[n] = packable(x, y, z) ? table_find(g, prime_hash(x, y, z)) : -1;
        }
        __syncthreads();
        for (int c = threadIdx.x; c < kBlockVoxels; c += blockDim.x) {
            const int i = c & 7, j = (c >> 3) & 7, k = c >> 6;
            F3 p[8];
            float s[8];
            bool ok = true;
            int cs = 0;
#pragma unroll
            for (int m = 0; m < 8; m++) {
                const int n = kMcCornerCell[m];
                const int vi = i + (n & 1), vj = j + ((n >> 1) & 1), vk = k + (n >> 2);
                const int b = nb[(vi >> 3) + 2 * (vj >> 3) + 4 * (vk >> 3)];
                if (b < 0) {
                    ok = false;
                    break;
                }
                const float2 sw = voxel_sw<kStorage>(g, b, (vi & 7) + 8 * (vj & 7) + 64 * (vk & 7));
                if (!(sw.y > 0.f)) {  // a corner without observations: no cube (weight 0)
                    ok = false;
                    break;
                }
                s[m] = sw.x;
                if (sw.x < 0.f) cs |= 1 << m;
                p[m] = F3{((float)(bc[0] * 8 + vi) + 0.5f) * g.vl, ((float)(bc[1] * 8 + vj) + 0.5f) * g.vl,
                          ((float)(bc[2] * 8 + vk) + 0.5f) * g.vl};
            }
            if (!ok || cs == 0 || cs == 255) continue;
            const signed char *tri = g_mc_table.tri[cs];
            for (int q = 0; q < kMcMaxTris * 3; q += 3) {
                const int e0 = __ldg(tri + q);
                if (e0 < 0) break;
                const int es[3] = {e0, __ldg(tri + q + 1), __ldg(tri + q + 2)};
                F3 v[3];
#pragma unroll
                for (int u = 0; u < 3; u++) {
                    const int a = kMcEdgeLo[es[u]], b = kMcEdgeHi[es[u]];
                    v[u] = edge_point(p[a], s[a], p[b], s[b]);
                }
                const unsigned long long at = atomicAdd(o.count, 1ull);
                if (at >= o.cap) continue;
                float *d = o.tris + at * 9;
                d[0] = v[0].x, d[1] = v[0].y, d[2] = v[0].z, d[3] = v[1].x, d[4] = v[1].y, d[5] = v[1].z;
                d[6] = v[2].x, d[7] = v[2].y, d[8] = v[2].z;
            }
        }
    }
}

}  // namespace ss

using namespace ss;

extern "C" ss_status ss_grid_extract_mesh_cubes(ss_grid *g, int64_t max_triangles, float *triangles, int64_t *count,
                                                ss_stream_t stream) {
    if (!g || !count || max_triangles < 0 || (max_triangles > 0 && !triangles)) return SS_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    if (!g->mesh_count) SS_CUDA_TRY(cudaMalloc(&g->mesh_count, sizeof(unsigned long long)));
    SS_CUDA_TRY(cudaMemsetAsync(g->mesh_count, 0, sizeof(unsigned long long), s));
    MeshOut o{triangles, g->mesh_count, (unsigned long long)max_triangles};
    const int ctas = g->num_sms * 8;
    if (g->p.storage == SS_STORAGE_F32)
        mesh_mc_kernel<SS_STORAGE_F32><<<ctas, 256, 0, s>>>(g->v, o);
    else
        mesh_mc_kernel<SS_STORAGE_F16><<<ctas, 256, 0, s>>>(g->v, o);
    SS_LAUNCH_CHECK();
    unsigned long long n = 0;
    SS_CUDA_TRY(cudaMemcpyAsync(&n, g->mesh_count, sizeof(n), cudaMemcpyDeviceToHost, s));
    SS_CUDA_TRY(cudaStreamSynchronize(s));
    *count = (int64_t)n;
    return SS_OK;
}

extern "C" ss_status ss_grid_extract_mesh(ss_grid *g, int64_t max_triangles, float *triangles, int64_t *count,
                                          ss_stream_t stream) {
    if (!g || !count || max_triangles < 0 || (max_triangles > 0 && !triangles)) return SS_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    if (!g->mesh_count) SS_CUDA_TRY(cudaMalloc(&g->mesh_count, sizeof(unsigned long long)));
    SS_CUDA_TRY(cudaMemsetAsync(g->mesh_count, 0, sizeof(unsigned long long), s));
    MeshOut o{triangles, g->mesh_count, (unsigned long long)max_triangles};
    const int ctas = g->num_sms * 8;
    if (g->p.storage == SS_STORAGE_F32)
        mesh_kernel<SS_STORAGE_F32><<<ctas, 256, 0, s>>>(g->v, o);
    else
        mesh_kernel<SS_STORAGE_F16><<<ctas, 256, 0, s>>>(g->v, o);
    SS_LAUNCH_CHECK();
    unsigned long long n = 0;
    SS_CUDA_TRY(cudaMemcpyAsync(&n, g->mesh_count, sizeof(n), cudaMemcpyDeviceToHost, s));
    SS_CUDA_TRY(cudaStreamSynchronize(s));
    *count = (int64_t)n;
    return SS_OK;
}
