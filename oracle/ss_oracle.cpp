// ss_oracle.cpp — CPU restatement of SuperScanner's reconstruction hot path.
//
// TEST INFRASTRUCTURE ONLY. This file is the parity checker: only tests/,
// __graft_entry__.smoke() and bench.py's cpu_baseline / reference legs load it.
// The product path (superscanner_gb300/) never links or calls it.
//
// Parity status: PINNED by the reference's own code. The reference's
// hot-path sources (GPUVoxelGrid.cpp, kokkosICP.cpp, imageutil.cpp,
// kokkosUtil.cpp, kokkosFunctions.cpp) compile unchanged on the host against
// the stand-ins of ref_stub/ (Kokkos, Eigen, Open3D and OpenCV are absent):
// `make ref` builds them into _ref/libss_ref.so, tests/golden/ref_*.npz hold
// their outputs on the config-1 and config-2 sequences of tests/refcases.py,
// and tests/test_ref_pinned.py checks that this restatement reproduces every
// block, voxel, raycast row and kokkosICP pose of those fixtures bit for bit
// (and equals the live reference build on further cases). What the pin does
// not reach: the third-party arithmetic the stand-ins restate (Eigen's 4x4
// inverse and JacobiSVD, Kokkos' hash-map slot layout) and the reference
// binary's FMA contraction (ref_stub/ss_ref_stub.h, oracle/Makefile).
//
// Semantics follow the reference source statement by statement, in IEEE
// single precision with no floating-point contraction (build with
// -ffp-contract=off): operand types and evaluation order are those of the
// C++ expressions in the cited lines, including the places where the
// reference promotes to double. Float->int casts follow the CUDA device
// conversion the reference actually ran (truncate toward zero, saturate,
// NaN -> 0), see f2i() below.
//
// Three behaviours of the reference are data races or undefined; the oracle
// and the CUDA path share one canonical resolution for each:
//  * Blocks whose prime hashes collide alias one map entry and the entry's
//    pzero/vbInd are written by every visitor (GPUVoxelGrid.cpp:500-502, last
//    writer wins). Canonical rule: the entry takes the coordinates of the
//    visitor with the largest packed coordinate word of the current call.
//  * The raycast's step back can land in a block that is not in the map, where
//    the reference calls value_at(find(..)) on an invalid index
//    (GPUVoxelGrid.cpp:669-672). Canonical rule: that voxel reads as empty
//    (w = 0, sdf = 0, colour 0).
//  * kokkosICP's correspondence view is never zeroed before the first
//    iteration (kokkosICP.cpp:43; Kvec3f's default constructor,
//    kokkosFunctions.h:149, writes nothing), so pixels without a
//    correspondence hold whatever the device memory held. Canonical rule: it
//    starts at zero, as freshly allocated device memory reads.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <unordered_map>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "ss_ref_math.h"

namespace {

using namespace orc;

struct Block {
    I3 vb;
    V3 pzero;
    float sdf[kVox];
    float w[kVox];  // reference: short (GPUVoxelGrid.h:14); FP32 holds the same integers
    float r[kVox], g[kVox], b[kVox];
};

struct Grid {
    float vl, vbl, trunc;
    int resi, resj;
    float fx = 0, fy = 0, cx = 0, cy = 0, ci = 0, cj = 0;
    bool intr = false;
    float rmin = 0.2f;   // GPUVoxelGrid.h:56
    float d_max = 10.0f; // GPUVoxelGrid.h:55
    float max_weight = 0.f;
    std::unordered_map<uint64_t, int> map;
    std::vector<Block *> blocks;  // index -> block (nullptr after erase)
    std::vector<int> free_list;
    int status = 0;
};

// getPoint (GPUVoxelGrid.h:229-232)
inline V3 get_point(const Grid &g, int i, int j, float d) {
    return {(j - g.cj) / g.fx * d, (i - g.ci) / g.fy * d, d};
}

int find_or_insert(Grid &g, uint64_t key) {
    auto it = g.map.find(key);
    if (it != g.map.end()) return it->second;
    int idx;
    if (!g.free_list.empty()) {
        idx = g.free_list.back();
        g.free_list.pop_back();
    } else {
        idx = (int)g.blocks.size();
        g.blocks.push_back(nullptr);
    }
    Block *b = new Block;
    std::memset(b, 0, sizeof(Block));  // default-constructed Voxelblock (GPUVoxelGrid.h:20-26)
    g.blocks[idx] = b;
    g.map.emplace(key, idx);
    return idx;
}

const Block *find_block(const Grid &g, uint64_t key) {
    auto it = g.map.find(key);
    return it == g.map.end() ? nullptr : g.blocks[it->second];
}

struct Cand {
    uint64_t key;
    uint64_t packed;
};

// vbCollectionTag (GPUVoxelGrid.cpp:471-514) after depthToPcdTag (GPUVoxelGrid.h:303-307).
// Returns the touched entries of this call, each once.
std::vector<int> collect(Grid &g, const uint16_t *depth, const float *E) {
    const int rows = g.resi, cols = g.resj;
    std::vector<std::vector<Cand>> per_row(rows);
#pragma omp parallel for schedule(dynamic, 4)
    for (int i = 0; i < rows; i++) {
        std::vector<Cand> &out = per_row[i];
        uint64_t last[8];
        int nlast = 0;
        for (int j = 0; j < cols; j++) {
            V3 p = get_point(g, i, j, (float)(depth[i * cols + j]) / 1000);
            if (!(p.z > g.rmin)) continue;
            V3 pt = xform(E, p);
            V3 lo = sub(pt, V3{g.trunc, g.trunc, g.trunc});
            V3 hi = add(pt, V3{g.trunc, g.trunc, g.trunc});
            I3 mn{idx_rule(lo.x, g.vbl), idx_rule(lo.y, g.vbl), idx_rule(lo.z, g.vbl)};
            I3 mx{idx_rule(hi.x, g.vbl), idx_rule(hi.y, g.vbl), idx_rule(hi.z, g.vbl)};
            for (int x = mn.x; x <= mx.x; x++)
                for (int y = mn.y; y <= mx.y; y++)
                    for (int z = mn.z; z <= mx.z; z++) {
                        if (!packable(x, y, z)) continue;  // reported as SS_ERR_RANGE
                        uint64_t pk = pack_coords(x, y, z);
                        bool seen = false;
                        for (int q = 0; q < nlast; q++) seen |= (last[q] == pk);
                        if (seen) continue;
                        if (nlast < 8) last[nlast++] = pk;
                        else { std::memmove(last, last + 1, 7 * sizeof(uint64_t)); last[7] = pk; }
                        out.push_back({prime_hash(x, y, z), pk});
                    }
        }
    }
    // Sequential merge: find / insert, canonical coordinates, per-call dedupe
    // (alreadyIntegrated, GPUVoxelGrid.cpp:504-509).
    std::vector<int> touched;
    std::unordered_map<int, uint64_t> frame_coords;
    frame_coords.reserve(1 << 16);
    for (int i = 0; i < rows; i++) {
        for (const Cand &c : per_row[i]) {
            int idx = find_or_insert(g, c.key);
            auto it = frame_coords.find(idx);
            if (it == frame_coords.end()) {
                frame_coords.emplace(idx, c.packed);
                touched.push_back(idx);
            } else if (c.packed > it->second) {
                it->second = c.packed;
            }
        }
    }
    for (int idx : touched) {
        I3 v = unpack_coords(frame_coords[idx]);
        Block *b = g.blocks[idx];
        b->vb = v;
        b->pzero = smul(g.vbl, V3{(float)v.x, (float)v.y, (float)v.z});  // GPUVoxelGrid.cpp:501
    }
    return touched;
}

// updateSingleVoxel[Color] / deUpdateSingleVoxel[Color] (GPUVoxelGrid.cpp:345-469)
inline void update_voxel(const Grid &g, Block &b, int v, V3 vm, const uint16_t *depth,
                         const uint8_t *rgb, const float *E, const float *Einv, V3 Ez,
                         bool color, bool deint) {
    V3 q = xform(Einv, vm);
    // getCoordinate (GPUVoxelGrid.h:234-237)
    float cxf = q.y * g.fy / q.z + g.ci;
    float cyf = q.x * g.fx / q.z + g.cj;
    int cori = f2i(cxf);
    int corj = f2i(cyf);
    if (!(cori < g.resi && corj < g.resj && cori >= 0 && corj >= 0)) return;
    V3 vpt = get_point(g, cori, corj, (float)(depth[cori * g.resj + corj]) / 1000);
    if (!(vpt.z > g.rmin)) return;
    vpt = xform(E, vpt);
    float sdf = dot(sub(vpt, vm), Ez);
    if (!(std::fabs(sdf) < g.trunc)) return;
    float w = b.w[v];
    if (!deint) {
        b.sdf[v] = (b.sdf[v] * w + sdf) / (w + 1);
        if (color) {
            const uint8_t *c = rgb + ((size_t)cori * g.resj + corj) * 3;
            b.r[v] = (b.r[v] * w + c[0]) / (w + 1);
            b.g[v] = (b.g[v] * w + c[1]) / (w + 1);
            b.b[v] = (b.b[v] * w + c[2]) / (w + 1);
        }
        float nw = w + 1;
        if (g.max_weight > 0 && nw > g.max_weight) nw = g.max_weight;
        b.w[v] = nw;
    } else {
        if (w != 1) {
            b.sdf[v] = (b.sdf[v] * w - sdf) / (w - 1);
            if (color) {
                const uint8_t *c = rgb + ((size_t)cori * g.resj + corj) * 3;
                b.r[v] = (b.r[v] * w - c[0]) / (w - 1);
                b.g[v] = (b.g[v] * w - c[1]) / (w - 1);
                b.b[v] = (b.b[v] * w - c[2]) / (w - 1);
            }
            b.w[v] = w - 1;
        } else {
            b.w[v] = 0;
            b.sdf[v] = 0;
            if (color) b.r[v] = b.g[v] = b.b[v] = 0;
        }
    }
}

// 4x4 inverse (row-major) by the adjugate in double, each cofactor a 3x3
// minor expanded along its first row, rounded to float once. Stands in for
// Eigen::Matrix4f::inverse() at GPUVoxelGrid.cpp:55 (Eigen is absent); the
// library's host code and the stand-in of oracle/ref_stub use the same form.
double det3_rowmajor(const double a[9]) {
    return a[0] * (a[4] * a[8] - a[5] * a[7]) - a[1] * (a[3] * a[8] - a[5] * a[6]) +
           a[2] * (a[3] * a[7] - a[4] * a[6]);
}

void inverse4(const float *Ef, float *out) {
    double m[16], cof[16];
    for (int k = 0; k < 16; k++) m[k] = Ef[k];
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) {
            double sub[9];
            int n = 0;
            for (int r = 0; r < 4; r++)
                if (r != i)
                    for (int c = 0; c < 4; c++)
                        if (c != j) sub[n++] = m[4 * r + c];
            const double d = det3_rowmajor(sub);
            cof[4 * i + j] = ((i + j) & 1) ? -d : d;
        }
    const double det = m[0] * cof[0] + m[1] * cof[1] + m[2] * cof[2] + m[3] * cof[3];
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) out[4 * j + i] = (float)(cof[4 * i + j] / det);
}

// ---------------------------------------------------------------- Jacobi SVD
// One-sided (Hestenes) Jacobi SVD of a 3x3 double matrix, H = U diag(S) V^T.
// Stands in for Eigen::JacobiSVD at kokkosICP.cpp:173-175; R = V U^T does not
// depend on the SVD's sign or ordering conventions when H has full rank.
void svd3(const double *H, double *U, double *S, double *V) {
    double A[9];
    std::memcpy(A, H, sizeof(A));
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
                if (gamma == 0.0 || std::fabs(gamma) <= 1e-15 * std::sqrt(alpha * beta)) continue;
                rotated = true;
                double zeta = (beta - alpha) / (2.0 * gamma);
                double t = (zeta >= 0 ? 1.0 : -1.0) / (std::fabs(zeta) + std::sqrt(1.0 + zeta * zeta));
                double c = 1.0 / std::sqrt(1.0 + t * t), s = c * t;
                for (int i = 0; i < 3; i++) {
                    double ap = A[i * 3 + p], aq = A[i * 3 + q];
                    A[i * 3 + p] = c * ap - s * aq;
                    A[i * 3 + q] = s * ap + c * aq;
                    double vp = V[i * 3 + p], vq = V[i * 3 + q];
                    V[i * 3 + p] = c * vp - s * vq;
                    V[i * 3 + q] = s * vp + c * vq;
                }
            }
        if (!rotated) break;
    }
    int zero_col = -1;
    for (int j = 0; j < 3; j++) {
        double n = std::sqrt(A[j] * A[j] + A[3 + j] * A[3 + j] + A[6 + j] * A[6 + j]);
        S[j] = n;
        if (n > 1e-300) {
            for (int i = 0; i < 3; i++) U[i * 3 + j] = A[i * 3 + j] / n;
        } else {
            zero_col = j;
            for (int i = 0; i < 3; i++) U[i * 3 + j] = 0;
        }
    }
    if (zero_col >= 0) {  // complete U to a right-handed orthonormal basis
        int a = (zero_col + 1) % 3, b = (zero_col + 2) % 3;
        double ua[3] = {U[a], U[3 + a], U[6 + a]}, ub[3] = {U[b], U[3 + b], U[6 + b]};
        U[zero_col] = ua[1] * ub[2] - ua[2] * ub[1];
        U[3 + zero_col] = ua[2] * ub[0] - ua[0] * ub[2];
        U[6 + zero_col] = ua[0] * ub[1] - ua[1] * ub[0];
    }
}

void matmul4d(const double *A, const double *B, double *C) {
    for (int r = 0; r < 4; r++)
        for (int c = 0; c < 4; c++) {
            double s = 0;
            for (int k = 0; k < 4; k++) s += A[r * 4 + k] * B[k * 4 + c];
            C[r * 4 + c] = s;
        }
}

void inverse4d(const double *m, double *out) {
    float f[16], fi[16];
    (void)f;
    (void)fi;
    // Rigid-or-general inverse by Gauss-Jordan with partial pivoting (double).
    double a[4][8];
    for (int r = 0; r < 4; r++)
        for (int c = 0; c < 8; c++) a[r][c] = c < 4 ? m[r * 4 + c] : (c - 4 == r ? 1.0 : 0.0);
    for (int col = 0; col < 4; col++) {
        int piv = col;
        for (int r = col + 1; r < 4; r++)
            if (std::fabs(a[r][col]) > std::fabs(a[piv][col])) piv = r;
        if (piv != col)
            for (int c = 0; c < 8; c++) std::swap(a[col][c], a[piv][c]);
        double d = a[col][col];
        for (int c = 0; c < 8; c++) a[col][c] /= d;
        for (int r = 0; r < 4; r++) {
            if (r == col) continue;
            double f2 = a[r][col];
            for (int c = 0; c < 8; c++) a[r][c] -= f2 * a[col][c];
        }
    }
    for (int r = 0; r < 4; r++)
        for (int c = 0; c < 4; c++) out[r * 4 + c] = a[r][c + 4];
}

}  // namespace

extern "C" {

void *orc_grid_new(float vl, float trunc, int resi, int resj, float max_weight) {
    Grid *g = new Grid;
    g->vl = vl;
    g->vbl = kEdge * vl;  // GPUVoxelGrid.cpp:15
    g->trunc = trunc;
    g->resi = resi;
    g->resj = resj;
    g->max_weight = max_weight;
    g->map.reserve(1 << 18);
    return g;
}

void orc_grid_free(void *h) {
    Grid *g = (Grid *)h;
    for (Block *b : g->blocks) delete b;
    delete g;
}

// setIntrinsic (GPUVoxelGrid.cpp:253-266)
void orc_grid_set_intrinsic(void *h, float fx, float fy, float cx, float cy) {
    Grid *g = (Grid *)h;
    g->cx = cx;
    g->cy = cy;
    g->ci = g->resi - cy;
    g->cj = cx;
    g->fx = fx;
    g->fy = fy;
    g->intr = true;
}

void orc_inverse4f(const float *E, float *out) { inverse4(E, out); }

// integrate / deIntegrate (GPUVoxelGrid.cpp:41-136). Returns the number of
// touched entries.
int orc_grid_fuse(void *h, const uint16_t *depth, const uint8_t *rgb, const float *E,
                  int with_color, int deint) {
    Grid *g = (Grid *)h;
    // Ez: normalized third column of extr (GPUVoxelGrid.cpp:52-53)
    V3 Ez = normalized(V3{E[2], E[6], E[10]});
    float Einv[16];
    inverse4(E, Einv);
    std::vector<int> touched = collect(*g, depth, E);
    const float vl = g->vl;
    const bool color = with_color != 0 && rgb != nullptr;
#pragma omp parallel for schedule(dynamic, 8)
    for (size_t t = 0; t < touched.size(); t++) {
        Block &b = *g->blocks[touched[t]];
        // integrationCoreTag: voxel centre in double, stored as float
        // (GPUVoxelGrid.cpp:521: pzero.x + (k + 0.5) * vl)
        for (int m = 0; m < kEdge; m++)
            for (int l = 0; l < kEdge; l++)
                for (int k = 0; k < kEdge; k++) {
                    V3 vm{(float)(b.pzero.x + (k + 0.5) * vl), (float)(b.pzero.y + (l + 0.5) * vl),
                          (float)(b.pzero.z + (m + 0.5) * vl)};
                    int v = k + l * kEdge + m * kEdge * kEdge;
                    update_voxel(*g, b, v, vm, depth, rgb, E, Einv, Ez, color, deint != 0);
                }
    }
    return (int)touched.size();
}

int orc_grid_count(void *h) { return (int)((Grid *)h)->map.size(); }

// Canonical dump sorted by key.
int orc_grid_export(void *h, int max_blocks, uint64_t *keys, int32_t *coords, float *sdf,
                    float *w, float *rgb) {
    Grid *g = (Grid *)h;
    std::vector<std::pair<uint64_t, int>> items(g->map.begin(), g->map.end());
    std::sort(items.begin(), items.end());
    int n = 0;
    for (auto &it : items) {
        if (n >= max_blocks) break;
        const Block &b = *g->blocks[it.second];
        if (keys) keys[n] = it.first;
        if (coords) {
            coords[n * 3 + 0] = b.vb.x;
            coords[n * 3 + 1] = b.vb.y;
            coords[n * 3 + 2] = b.vb.z;
        }
        if (sdf) std::memcpy(sdf + (size_t)n * kVox, b.sdf, sizeof(b.sdf));
        if (w) std::memcpy(w + (size_t)n * kVox, b.w, sizeof(b.w));
        if (rgb) {
            std::memcpy(rgb + (size_t)n * 3 * kVox, b.r, sizeof(b.r));
            std::memcpy(rgb + (size_t)n * 3 * kVox + kVox, b.g, sizeof(b.g));
            std::memcpy(rgb + (size_t)n * 3 * kVox + 2 * kVox, b.b, sizeof(b.b));
        }
        n++;
    }
    return n;
}

// Loads a canonical dump (keys recomputed from coordinates).
void orc_grid_import(void *h, int n, const int32_t *coords, const float *sdf, const float *w,
                     const float *rgb) {
    Grid *g = (Grid *)h;
    for (int t = 0; t < n; t++) {
        int x = coords[t * 3], y = coords[t * 3 + 1], z = coords[t * 3 + 2];
        int idx = find_or_insert(*g, prime_hash(x, y, z));
        Block &b = *g->blocks[idx];
        b.vb = {x, y, z};
        b.pzero = smul(g->vbl, V3{(float)x, (float)y, (float)z});
        std::memcpy(b.sdf, sdf + (size_t)t * kVox, sizeof(b.sdf));
        std::memcpy(b.w, w + (size_t)t * kVox, sizeof(b.w));
        if (rgb) {
            std::memcpy(b.r, rgb + (size_t)t * 3 * kVox, sizeof(b.r));
            std::memcpy(b.g, rgb + (size_t)t * 3 * kVox + kVox, sizeof(b.g));
            std::memcpy(b.b, rgb + (size_t)t * 3 * kVox + 2 * kVox, sizeof(b.b));
        }
    }
}

// cleanMemory / cleanTag (GPUVoxelGrid.cpp:185-196, 785-805)
int orc_grid_clean(void *h) {
    Grid *g = (Grid *)h;
    int erased = 0;
    for (auto it = g->map.begin(); it != g->map.end();) {
        Block *b = g->blocks[it->second];
        bool empty = true;
        for (int v = 0; v < kVox; v++)
            if (b->w[v] != 0) empty = false;
        if (empty) {
            delete b;
            g->blocks[it->second] = nullptr;
            g->free_list.push_back(it->second);
            it = g->map.erase(it);
            erased++;
        } else {
            ++it;
        }
    }
    return erased;
}

// raycastingTag (GPUVoxelGrid.cpp:561-715) with normPcd from createNormPcdTag (:717-722).
void orc_grid_raycast(void *h, const float *Er, float *ray_pcd, float *ray_color) {
    Grid &g = *(Grid *)h;
    const float vl = g.vl, vbl = g.vbl, d_trunc = g.trunc, d_max = g.d_max;
#pragma omp parallel for schedule(dynamic, 4)
    for (int i = 0; i < g.resi; i++) {
        for (int j = 0; j < g.resj; j++) {
            auto vb_of = [&](V3 p) {
                return I3{idx_rule(p.x, vbl), idx_rule(p.y, vbl), idx_rule(p.z, vbl)};
            };
            auto vin_of = [&](V3 p, I3 b) {
                V3 q = sub(p, V3{vbl * b.x, vbl * b.y, vbl * b.z});
                return I3{idx_rule(q.x, vl), idx_rule(q.y, vl), idx_rule(q.z, vl)};
            };
            auto mid = [&](I3 v, I3 b) {  // getVoxelMidPoint (GPUVoxelGrid.h:274-278)
                return V3{(float)(b.x * vbl + (v.x + 0.5) * vl), (float)(b.y * vbl + (v.y + 0.5) * vl),
                          (float)(b.z * vbl + (v.z + 0.5) * vl)};
            };
            auto same = [](I3 a, I3 b) { return a.x == b.x && a.y == b.y && a.z == b.z; };

            V3 np = normalized(get_point(g, i, j, 1.0f));
            V3 rv = xform(Er, np);
            V3 dir = sub(rv, V3{Er[3], Er[7], Er[11]});
            float l = 0.1f;
            {
                V3 st = smul(1 - l, dir);
                rv = sub(rv, st);
            }
            bool done = false, Fn = false, Lp = false;
            I3 oldvb{0, 0, 0};
            size_t pix = (size_t)i * g.resj + j;
            while (!done && !Fn && l < d_max) {
                I3 vbInd = vb_of(rv);
                const Block *blk = find_block(g, prime_hash(vbInd.x, vbInd.y, vbInd.z));
                int count = 0;
                while (!blk && l < d_max) {
                    rv = add(rv, smul(vbl, dir));
                    l += vbl;
                    vbInd = vb_of(rv);
                    blk = find_block(g, prime_hash(vbInd.x, vbInd.y, vbInd.z));
                    count++;
                }
                if (l >= d_max) break;
                if (count > 0) {
                    rv = sub(rv, smul(vbl - d_trunc, dir));
                    l -= (vbl - d_trunc);
                    vbInd = vb_of(rv);
                    blk = find_block(g, prime_hash(vbInd.x, vbInd.y, vbInd.z));
                    while (!blk && l < d_max) {
                        rv = add(rv, smul(d_trunc, dir));
                        l += d_trunc;
                        vbInd = vb_of(rv);
                        blk = find_block(g, prime_hash(vbInd.x, vbInd.y, vbInd.z));
                    }
                }
                if (l >= d_max) break;
                const Block &vb = *blk;
                I3 vInd = vin_of(rv, vbInd);
                oldvb = vbInd;
                while (!done && l < d_max && same(oldvb, vbInd) && !Fn) {
                    int ci_ = vInd.x + vInd.y * kEdge + vInd.z * kEdge * kEdge;
                    float cw = vb.w[ci_], cs = vb.sdf[ci_];
                    if (cw > 0) {
                        if (cs > 0) {
                            Lp = true;
                            rv = add(rv, smul(vl, dir));
                            l += vl;
                            oldvb = vbInd;
                            vbInd = vb_of(rv);
                            vInd = vin_of(rv, vbInd);
                        } else {
                            if (Lp) {
                                done = true;
                                V3 vm_in = mid(vInd, vbInd);
                                rv = sub(rv, smul(vl, dir));
                                l -= vl;
                                vbInd = vb_of(rv);
                                vInd = vin_of(rv, vbInd);
                                V3 vm_out = mid(vInd, vbInd);
                                int oi = vInd.x + vInd.y * kEdge + vInd.z * kEdge * kEdge;
                                float ow = 0, os = 0, orr = 0, og = 0, ob = 0;
                                const Block *ob_ = same(vbInd, oldvb)
                                                       ? &vb
                                                       : find_block(g, prime_hash(vbInd.x, vbInd.y, vbInd.z));
                                if (ob_) {
                                    ow = ob_->w[oi];
                                    os = ob_->sdf[oi];
                                    orr = ob_->r[oi];
                                    og = ob_->g[oi];
                                    ob = ob_->b[oi];
                                }
                                float x = (ow * os / vl + cw * (1 - cs / vl)) / (cw + ow);
                                V3 p = add(vm_out, smul(x, sub(vm_in, vm_out)));
                                float s = dot(p, dir) - dot(rv, dir);
                                V3 out = add(rv, smul(s, dir));
                                ray_pcd[pix * 3 + 0] = out.x;
                                ray_pcd[pix * 3 + 1] = out.y;
                                ray_pcd[pix * 3 + 2] = out.z;
                                if (ray_color) {
                                    ray_color[pix * 3 + 0] = (float)((0.5 * orr + 0.5 * vb.r[ci_]) / 255);
                                    ray_color[pix * 3 + 1] = (float)((0.5 * og + 0.5 * vb.g[ci_]) / 255);
                                    ray_color[pix * 3 + 2] = (float)((0.5 * ob + 0.5 * vb.b[ci_]) / 255);
                                }
                            } else {
                                Fn = true;
                            }
                        }
                    } else {
                        Lp = false;
                        rv = add(rv, smul(vl, dir));
                        l += vl;
                        oldvb = vbInd;
                        vbInd = vb_of(rv);
                        vInd = vin_of(rv, vbInd);
                    }
                }
            }
            if (!done) {
                ray_pcd[pix * 3 + 0] = ray_pcd[pix * 3 + 1] = ray_pcd[pix * 3 + 2] = 0.f;
                if (ray_color) ray_color[pix * 3 + 0] = ray_color[pix * 3 + 1] = ray_color[pix * 3 + 2] = 0.f;
            }
        }
    }
}

// CreatePcdFromDepthView (imageutil.cpp:89-111)
void orc_depth_to_pcd(const uint16_t *depth, int rows, int cols, float fx, float fy, float cx,
                      float cy, float *pcd) {
    float ci = rows - cy, cj = cx;
    for (int i = 0; i < rows; i++)
        for (int j = 0; j < cols; j++) {
            float d = (float)(depth[i * cols + j]) / 1000;
            size_t p = ((size_t)i * cols + j) * 3;
            pcd[p + 0] = (j - cj) / fx * d;
            pcd[p + 1] = (i - ci) / fy * d;
            pcd[p + 2] = d;
        }
}

// CalculateNormalsFromPCDView (imageutil.cpp:117-157)
void orc_normals(const float *pcd, int rows, int cols, float *out) {
    auto P = [&](int i, int j) {
        size_t p = ((size_t)i * cols + j) * 3;
        return V3{pcd[p], pcd[p + 1], pcd[p + 2]};
    };
    for (int i = 0; i < rows; i++)
        for (int j = 0; j < cols; j++) {
            size_t p = ((size_t)i * cols + j) * 3;
            out[p] = 0.f;
            out[p + 1] = 0.f;
            out[p + 2] = 1.f;
        }
    for (int i = 1; i < rows - 1; i++)
        for (int j = 1; j < cols - 1; j++) {
            if (P(i, j).z != 0 && P(i + 1, j).z != 0 && P(i - 1, j).z != 0 && P(i, j + 1).z != 0 &&
                P(i, j - 1).z != 0) {
                V3 c = P(i, j);
                V3 n1 = cross(sub(P(i + 1, j), c), sub(P(i, j + 1), c));
                V3 n2 = cross(sub(P(i, j - 1), c), sub(P(i + 1, j), c));
                V3 n3 = cross(sub(P(i, j + 1), c), sub(P(i - 1, j), c));
                V3 n4 = cross(sub(P(i - 1, j), c), sub(P(i, j - 1), c));
                V3 n = normalized(add(add(add(n1, n2), n3), n4));
                size_t p = ((size_t)i * cols + j) * 3;
                out[p] = n.x;
                out[p + 1] = n.y;
                out[p + 2] = n.z;
            }
        }
}

void orc_svd3(const double *H, double *U, double *S, double *V) { svd3(H, U, S, V); }

// kokkosICP(View d1, View d2, tx, ty, type, rmse) (kokkosICP.cpp:25-210).
// Writes the best Txy (row-major) and the lowest RMSE; returns the number of
// iterations run. stats (optional, 10 x 4): per iteration n_cors, rmse,
// fitness, and whether it became the best.
int orc_kokkos_icp(const uint16_t *d1, const uint16_t *d2, int rows, int cols, float fx, float fy,
                   float cx, float cy, const double *tx, const double *ty, int type, double *out,
                   float *rmse_out, double *stats) {
    std::vector<float> x((size_t)rows * cols * 3), y((size_t)rows * cols * 3), yn((size_t)rows * cols * 3),
        xn((size_t)rows * cols * 3);
    orc_depth_to_pcd(d1, rows, cols, fx, fy, cx, cy, x.data());
    orc_depth_to_pcd(d2, rows, cols, fx, fy, cx, cy, y.data());
    orc_normals(y.data(), rows, cols, yn.data());
    const float ci = rows - cy, cj = cx;
    const int n_search = 5, n_it = 10;
    const float max_dist = 0.075f;
    double tyi[16], Txy_e[16];
    inverse4d(ty, tyi);
    matmul4d(tyi, tx, Txy_e);
    float Txy[16];
    for (int k = 0; k < 16; k++) Txy[k] = (float)Txy_e[k];
    float lowest = 1e6f;
    double best[16];
    for (int k = 0; k < 16; k++) best[k] = (k % 5 == 0) ? 1.0 : 0.0;
    auto X = [&](const std::vector<float> &a, int i, int j) {
        size_t p = ((size_t)i * cols + j) * 3;
        return V3{a[p], a[p + 1], a[p + 2]};
    };
    for (int it = 0; it < n_it; it++) {
        std::fill(xn.begin(), xn.end(), 0.f);
#pragma omp parallel for schedule(dynamic, 4)
        for (int i = 0; i < rows; i++)
            for (int j = 0; j < cols; j++) {
                V3 xp = X(x, i, j);
                if (xp.z == 0) continue;
                V3 px = xform(Txy, xp);
                float c0 = px.y * fy / px.z + ci, c1 = px.x * fx / px.z + cj;
                int centeri = f2i(c0), centerj = f2i(c1);
                float smallest = 1e6f;
                if (!(centeri > n_search && centeri < rows - n_search && centerj > n_search &&
                      centerj < cols - n_search))
                    continue;
                size_t o = ((size_t)i * cols + j) * 3;
                for (int k = centeri - n_search; k < centeri + n_search; k++)
                    for (int l = centerj - n_search; l < centerj + n_search; l++) {
                        V3 py = X(y, k, l);
                        if (type == 0) {
                            if (py.z != 0) {
                                float dist = length(sub(py, px));
                                if (dist < smallest && dist < max_dist) {
                                    smallest = dist;
                                    xn[o] = py.x;
                                    xn[o + 1] = py.y;
                                    xn[o + 2] = py.z;
                                }
                            }
                        } else {
                            V3 nn = X(yn, k, l);
                            if (py.z != 0 && nn.x != 0) {
                                float d = dot(sub(py, px), nn);
                                float dist = std::fabs(d);
                                if (dist < smallest && dist < max_dist) {
                                    smallest = dist;
                                    V3 q = add(px, smul(d, nn));
                                    xn[o] = q.x;
                                    xn[o + 1] = q.y;
                                    xn[o + 2] = q.z;
                                }
                            }
                        }
                    }
            }
        // host part (kokkosICP.cpp:121-185), sequential, row-major
        double ccx[3] = {0, 0, 0}, ccy[3] = {0, 0, 0};
        float rsme = 0, n_cors = 0, n_x = 0;
        for (int i = 0; i < rows; i++)
            for (int j = 0; j < cols; j++) {
                V3 a = X(x, i, j), b = X(xn, i, j);
                if (b.z != 0) {
                    ccx[0] += a.x; ccx[1] += a.y; ccx[2] += a.z;
                    ccy[0] += b.x; ccy[1] += b.y; ccy[2] += b.z;
                    n_cors++;
                    double a4[4] = {a.x, a.y, a.z, 1.0}, e[4];
                    for (int r = 0; r < 4; r++) {
                        double s = 0;
                        for (int c = 0; c < 4; c++) s += Txy_e[r * 4 + c] * a4[c];
                        e[r] = (r < 3 ? (double)(&b.x)[r] : 1.0) - s;
                    }
                    float tmp = (float)std::sqrt(e[0] * e[0] + e[1] * e[1] + e[2] * e[2] + e[3] * e[3]);
                    rsme += tmp * tmp;
                }
                if (a.z != 0) n_x++;
            }
        for (int k = 0; k < 3; k++) {
            ccx[k] = ccx[k] / n_cors;
            ccy[k] = ccy[k] / n_cors;
        }
        rsme /= n_cors;
        rsme = std::sqrt(rsme);
        float fitness = n_cors / n_x;
        double H[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
        for (int i = 0; i < rows; i++)
            for (int j = 0; j < cols; j++) {
                V3 a = X(x, i, j), b = X(xn, i, j);
                if (a.z != 0 && b.z != 0) {
                    double xa[3] = {a.x - ccx[0], a.y - ccx[1], a.z - ccx[2]};
                    double yb[3] = {b.x - ccy[0], b.y - ccy[1], b.z - ccy[2]};
                    for (int r = 0; r < 3; r++)
                        for (int c = 0; c < 3; c++) H[r * 3 + c] += xa[r] * yb[c];
                }
            }
        double U[9], S[3], V[9], R[9];
        svd3(H, U, S, V);
        for (int r = 0; r < 3; r++)
            for (int c = 0; c < 3; c++) {
                double s = 0;
                for (int k = 0; k < 3; k++) s += V[r * 3 + k] * U[c * 3 + k];
                R[r * 3 + c] = s;
            }
        for (int k = 0; k < 16; k++) Txy_e[k] = (k % 5 == 0) ? 1.0 : 0.0;
        for (int r = 0; r < 3; r++) {
            for (int c = 0; c < 3; c++) Txy_e[r * 4 + c] = R[r * 3 + c];
            Txy_e[r * 4 + 3] = ccy[r] - (R[r * 3] * ccx[0] + R[r * 3 + 1] * ccx[1] + R[r * 3 + 2] * ccx[2]);
        }
        for (int k = 0; k < 16; k++) Txy[k] = (float)Txy_e[k];
        bool became_best = false;
        if (rsme < lowest) {
            lowest = rsme;
            std::memcpy(best, Txy_e, sizeof(best));
            became_best = true;
        }
        if (stats) {
            stats[it * 4 + 0] = n_cors;
            stats[it * 4 + 1] = rsme;
            stats[it * 4 + 2] = fitness;
            stats[it * 4 + 3] = became_best ? 1.0 : 0.0;
        }
    }
    std::memcpy(out, best, sizeof(best));
    if (rmse_out) *rmse_out = lowest;
    return n_it;
}

// Kmat4f * Kvec4f (kokkosFunctions.h:702-711, rows dotted left to right),
// the operation exe/Test.cpp:117-181 checks against Eigen.
void orc_mat4_vec4(const float *M, const float *v, float *out) {
    for (int r = 0; r < 4; r++)
        out[r] = M[r * 4 + 0] * v[0] + M[r * 4 + 1] * v[1] + M[r * 4 + 2] * v[2] + M[r * 4 + 3] * v[3];
}

int orc_threads() {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

}  // extern "C"
