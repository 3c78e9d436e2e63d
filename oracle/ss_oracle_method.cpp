// ss_oracle_method.cpp — FP64 oracle of the per-frame method.
//
// TEST INFRASTRUCTURE ONLY (see ss_oracle.cpp's header). This is the FP64
// restatement of the method the GPU pipeline runs (FP64 TSDF, trilinear
// raycast with at most max_steps steps, frame-to-model point-to-plane
// Gauss-Newton over a 3-level pyramid), against which the FP32 and FP16 GPU
// forms state their errors. Block allocation is the reference's (float,
// GPUVoxelGrid.cpp:471-514, as in ss_oracle.cpp), so both sides fuse into the
// same set of blocks; everything after allocation is double precision.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include "ss_ref_math.h"

namespace {

using namespace orc;

struct Block64 {
    int vb[3];
    double sdf[kVox];
    double w[kVox];
};

struct Grid64 {
    float vl, vbl, trunc;  // float parameters of the allocation
    int resi, resj;
    float fx, fy, cx, cy, ci, cj;
    double max_weight;
    float rmin = 0.2f;
    int round_pixel = 1;  // 1: nearest pixel of the voxel's projection; 0: truncation (GPUVoxelGrid.cpp:348)
    std::unordered_map<uint64_t, int> map;
    std::vector<Block64 *> blocks;
    std::unordered_set<uint64_t> supers;  // super-blocks (8^3 blocks) holding an allocated block
};

inline int floordiv8(int v) { return v >= 0 ? v / 8 : -((-v + 7) / 8); }
inline uint64_t super_key(int sx, int sy, int sz) {
    return ((uint64_t)(uint32_t)(sx + 1024) << 22) | ((uint64_t)(uint32_t)(sy + 1024) << 11) |
           (uint64_t)(uint32_t)(sz + 1024);
}

struct D3 {
    double x, y, z;
};

inline D3 dxform(const double *T, D3 p) {
    return {T[0] * p.x + T[1] * p.y + T[2] * p.z + T[3], T[4] * p.x + T[5] * p.y + T[6] * p.z + T[7],
            T[8] * p.x + T[9] * p.y + T[10] * p.z + T[11]};
}

void rigid_inverse(const double *T, double *Ti) {
    for (int r = 0; r < 3; r++) {
        for (int c = 0; c < 3; c++) Ti[r * 4 + c] = T[c * 4 + r];
        Ti[r * 4 + 3] = -(T[r] * T[3] + T[4 + r] * T[7] + T[8 + r] * T[11]);
    }
    Ti[12] = Ti[13] = Ti[14] = 0;
    Ti[15] = 1;
}

// Reference block allocation with the float pose (the GPU fuses with the float
// cast of the same pose). Returns touched block indices.
std::vector<int> collect64(Grid64 &g, const uint16_t *depth, const float *E) {
    std::vector<int> touched;
    std::unordered_map<int, uint64_t> frame;
    for (int i = 0; i < g.resi; i++)
        for (int j = 0; j < g.resj; j++) {
            const float d = (float)(depth[i * g.resj + j]) / 1000;
            V3 p{(j - g.cj) / g.fx * d, (i - g.ci) / g.fy * d, d};
            if (!(p.z > g.rmin)) continue;
            V3 pt = xform(E, p);
            V3 lo = sub(pt, V3{g.trunc, g.trunc, g.trunc}), hi = add(pt, V3{g.trunc, g.trunc, g.trunc});
            for (int x = idx_rule(lo.x, g.vbl); x <= idx_rule(hi.x, g.vbl); x++)
                for (int y = idx_rule(lo.y, g.vbl); y <= idx_rule(hi.y, g.vbl); y++)
                    for (int z = idx_rule(lo.z, g.vbl); z <= idx_rule(hi.z, g.vbl); z++) {
                        if (!packable(x, y, z)) continue;
                        const uint64_t key = prime_hash(x, y, z), pk = pack_coords(x, y, z);
                        auto it = g.map.find(key);
                        int idx;
                        if (it == g.map.end()) {
                            idx = (int)g.blocks.size();
                            Block64 *b = new Block64;
                            std::memset(b, 0, sizeof(Block64));
                            g.blocks.push_back(b);
                            g.map.emplace(key, idx);
                            g.supers.insert(super_key(floordiv8(x), floordiv8(y), floordiv8(z)));
                        } else {
                            idx = it->second;
                        }
                        auto f = frame.find(idx);
                        if (f == frame.end()) {
                            frame.emplace(idx, pk);
                            touched.push_back(idx);
                        } else if (pk > f->second) {
                            f->second = pk;
                        }
                    }
        }
    for (int idx : touched) {
        I3 v = unpack_coords(frame[idx]);
        g.blocks[idx]->vb[0] = v.x;
        g.blocks[idx]->vb[1] = v.y;
        g.blocks[idx]->vb[2] = v.z;
    }
    return touched;
}

const Block64 *find64(const Grid64 &g, int bx, int by, int bz) {
    if (!packable(bx, by, bz)) return nullptr;
    auto it = g.map.find(prime_hash(bx, by, bz));
    return it == g.map.end() ? nullptr : g.blocks[it->second];
}

struct Sample {
    bool valid;
    double f, gx, gy, gz;
};

struct Cache {
    int x = INT32_MIN, y = 0, z = 0;
    const Block64 *b = nullptr;
};

inline const Block64 *cached(const Grid64 &g, Cache &c, int bx, int by, int bz) {
    if (bx != c.x || by != c.y || bz != c.z) {
        c.x = bx;
        c.y = by;
        c.z = bz;
        c.b = find64(g, bx, by, bz);
    }
    return c.b;
}

Sample trilinear64(const Grid64 &g, double px, double py, double pz, Cache &c) {
    Sample r{false, 0, 0, 0, 0};
    const double vl = g.vl;
    const double ux = px / vl - 0.5, uy = py / vl - 0.5, uz = pz / vl - 0.5;
    const double fx0 = std::floor(ux), fy0 = std::floor(uy), fz0 = std::floor(uz);
    const int ix = (int)fx0, iy = (int)fy0, iz = (int)fz0;
    const double ax = ux - fx0, ay = uy - fy0, az = uz - fz0;
    double s[8];
    for (int k = 0; k < 8; k++) {
        const int vx = ix + (k & 1), vy = iy + ((k >> 1) & 1), vz = iz + (k >> 2);
        const int bx = floordiv8(vx), by = floordiv8(vy), bz = floordiv8(vz);
        const Block64 *b = cached(g, c, bx, by, bz);
        if (!b) return r;
        const int v = (vx - 8 * bx) + 8 * (vy - 8 * by) + 64 * (vz - 8 * bz);
        if (!(b->w[v] > 0)) return r;
        s[k] = b->sdf[v];
    }
    const double s00 = s[0] + ax * (s[1] - s[0]), s10 = s[2] + ax * (s[3] - s[2]);
    const double s01 = s[4] + ax * (s[5] - s[4]), s11 = s[6] + ax * (s[7] - s[6]);
    const double s0 = s00 + ay * (s10 - s00), s1 = s01 + ay * (s11 - s01);
    r.valid = true;
    r.f = s0 + az * (s1 - s0);
    const double dx00 = s[1] - s[0], dx10 = s[3] - s[2], dx01 = s[5] - s[4], dx11 = s[7] - s[6];
    const double dx0 = dx00 + ay * (dx10 - dx00), dx1 = dx01 + ay * (dx11 - dx01);
    r.gx = (dx0 + az * (dx1 - dx0)) / vl;
    r.gy = ((s10 - s00) + az * ((s11 - s01) - (s10 - s00))) / vl;
    r.gz = (s1 - s0) / vl;
    return r;
}

}  // namespace

extern "C" {

void *orm_grid_new(float vl, float trunc, int resi, int resj, float fx, float fy, float cx, float cy,
                   double max_weight) {
    Grid64 *g = new Grid64;
    g->vl = vl;
    g->vbl = kEdge * vl;
    g->trunc = trunc;
    g->resi = resi;
    g->resj = resj;
    g->fx = fx;
    g->fy = fy;
    g->cx = cx;
    g->cy = cy;
    g->ci = resi - cy;
    g->cj = cx;
    g->max_weight = max_weight;
    g->map.reserve(1 << 18);
    return g;
}

void orm_grid_free(void *h) {
    Grid64 *g = (Grid64 *)h;
    for (Block64 *b : g->blocks) delete b;
    delete g;
}

int orm_grid_count(void *h) { return (int)((Grid64 *)h)->map.size(); }

void orm_grid_set_round_pixel(void *h, int on) { ((Grid64 *)h)->round_pixel = on; }

// FP64 integrate (deint = 0) / deintegrate (deint = 1) at pose T (double).
int orm_grid_fuse(void *h, const uint16_t *depth, const double *T, int deint) {
    Grid64 &g = *(Grid64 *)h;
    float Ef[16];
    for (int k = 0; k < 16; k++) Ef[k] = (float)T[k];
    std::vector<int> touched = collect64(g, depth, Ef);
    double Ti[16];
    rigid_inverse(T, Ti);
    const double ezn = std::sqrt(T[2] * T[2] + T[6] * T[6] + T[10] * T[10]);
    const D3 Ez{T[2] / ezn, T[6] / ezn, T[10] / ezn};
    const double vl = g.vl, vbl = g.vbl, trunc = g.trunc;
#pragma omp parallel for schedule(dynamic, 8)
    for (size_t t = 0; t < touched.size(); t++) {
        Block64 &b = *g.blocks[touched[t]];
        for (int v = 0; v < kVox; v++) {
            const int k = v & 7, l = (v >> 3) & 7, m = v >> 6;
            const D3 vm{b.vb[0] * vbl + (k + 0.5) * vl, b.vb[1] * vbl + (l + 0.5) * vl, b.vb[2] * vbl + (m + 0.5) * vl};
            const D3 q = dxform(Ti, vm);
            const double c0 = q.y * g.fy / q.z + g.ci, c1 = q.x * g.fx / q.z + g.cj;
            if (!(c0 > -1.0 && c1 > -1.0 && c0 < g.resi && c1 < g.resj)) continue;
            const int i = g.round_pixel ? (int)std::floor(c0 + 0.5) : (int)c0;
            const int j = g.round_pixel ? (int)std::floor(c1 + 0.5) : (int)c1;
            if (i < 0 || j < 0 || i >= g.resi || j >= g.resj) continue;
            const double d = depth[i * g.resj + j] / 1000.0;
            if (!(d > g.rmin)) continue;
            const D3 pc{(j - g.cj) / g.fx * d, (i - g.ci) / g.fy * d, d};
            const D3 pw = dxform(T, pc);
            const double sdf = (pw.x - vm.x) * Ez.x + (pw.y - vm.y) * Ez.y + (pw.z - vm.z) * Ez.z;
            if (!(std::fabs(sdf) < trunc)) continue;
            double &s = b.sdf[v], &w = b.w[v];
            if (!deint) {
                s = (s * w + sdf) / (w + 1);
                w = (g.max_weight > 0 && w + 1 > g.max_weight) ? g.max_weight : w + 1;
            } else if (w != 0) {
                if (w != 1) {
                    s = (s * w - sdf) / (w - 1);
                    w -= 1;
                } else {
                    s = 0;
                    w = 0;
                }
            }
        }
    }
    return (int)touched.size();
}

// Canonical dump sorted by key (sdf and w in double).
int orm_grid_export(void *h, int max_blocks, uint64_t *keys, int32_t *coords, double *sdf, double *w) {
    Grid64 &g = *(Grid64 *)h;
    std::vector<std::pair<uint64_t, int>> items(g.map.begin(), g.map.end());
    std::sort(items.begin(), items.end());
    int n = 0;
    for (auto &it : items) {
        if (n >= max_blocks) break;
        const Block64 &b = *g.blocks[it.second];
        keys[n] = it.first;
        for (int k = 0; k < 3; k++) coords[n * 3 + k] = b.vb[k];
        std::memcpy(sdf + (size_t)n * kVox, b.sdf, sizeof(b.sdf));
        std::memcpy(w + (size_t)n * kVox, b.w, sizeof(b.w));
        n++;
    }
    return n;
}

// One march of the trilinear raycast from t0 (same step rules as the GPU
// kernel, in double); returns true on a zero crossing with t = hit depth.
static double refine64(const Grid64 &g, Cache &cache, double ox, double oy, double oz, double dx, double dy,
                       double dz, double ta, double fa, double tb, double fb) {
    for (int r = 0; r < 2; r++) {
        const double tc = ta + (tb - ta) * fa / (fa - fb);
        const Sample q = trilinear64(g, ox + tc * dx, oy + tc * dy, oz + tc * dz, cache);
        if (!q.valid) break;
        if (q.f > 0) {
            ta = tc;
            fa = q.f;
        } else {
            tb = tc;
            fb = q.f;
        }
    }
    return ta + (tb - ta) * fa / (fa - fb);
}

static bool march64_from(const Grid64 &g, Cache &cache, double ox, double oy, double oz, double dx, double dy,
                         double dz, double inv_len, double t0, double t_max, int max_steps, int &steps, double &t,
                         bool prev_valid, double t_prev, double f_prev) {
    const double vl = g.vl, vbl = g.vbl, sbl = 8 * vbl;
    t = t0;
    while (steps < max_steps && t < t_max) {
        const double px = ox + t * dx, py = oy + t * dy, pz = oz + t * dz;
        const int bx = (int)std::floor(px / vbl), by = (int)std::floor(py / vbl), bz = (int)std::floor(pz / vbl);
        steps++;
        const int sx = floordiv8(bx), sy = floordiv8(by), sz = floordiv8(bz);
        if (!g.supers.count(super_key(sx, sy, sz))) {
            double te = INFINITY;
            if (dx != 0) te = std::fmin(te, ((sx + (dx > 0)) * sbl - ox) / dx);
            if (dy != 0) te = std::fmin(te, ((sy + (dy > 0)) * sbl - oy) / dy);
            if (dz != 0) te = std::fmin(te, ((sz + (dz > 0)) * sbl - oz) / dz);
            t = std::fmax(te, t) + 1e-4 * vl * inv_len;
            prev_valid = false;
            continue;
        }
        if (!cached(g, cache, bx, by, bz)) {
            double te = INFINITY;
            if (dx != 0) te = std::fmin(te, ((bx + (dx > 0)) * vbl - ox) / dx);
            if (dy != 0) te = std::fmin(te, ((by + (dy > 0)) * vbl - oy) / dy);
            if (dz != 0) te = std::fmin(te, ((bz + (dz > 0)) * vbl - oz) / dz);
            t = std::fmax(te, t) + 1e-4 * vl * inv_len;
            prev_valid = false;
            continue;
        }
        const Sample sm = trilinear64(g, px, py, pz, cache);
        if (!sm.valid) {
            prev_valid = false;
            t += vl * inv_len;
            continue;
        }
        if (sm.f < 0) {
            if (!(prev_valid && f_prev > 0)) return false;
            t = refine64(g, cache, ox, oy, oz, dx, dy, dz, t_prev, f_prev, t, sm.f);
            return true;
        }
        prev_valid = true;
        t_prev = t;
        f_prev = sm.f;
        t += std::fmax(vl, 0.8 * sm.f) * inv_len;
    }
    return false;
}

static bool march64(const Grid64 &g, Cache &cache, double ox, double oy, double oz, double dx, double dy, double dz,
                    double inv_len, double t0, double t_max, int max_steps, int &steps, double &t) {
    return march64_from(g, cache, ox, oy, oz, dx, dy, dz, inv_len, t0, t_max, max_steps, steps, t, false, 0, 0);
}

// Search from a depth hint td within [t_lo, t_hi] (the GPU raycast's
// ray_search, seek mode): unobserved at td: no hit; positive: forward to t_hi;
// negative: back to a positive sample (unobserved or below t_lo: no hit).
static bool seek64(const Grid64 &g, Cache &cache, double ox, double oy, double oz, double dx, double dy, double dz,
                   double inv_len, double td, double t_lo, double t_hi, int max_steps, int &steps, double &t) {
    const double vl = g.vl;
    steps++;
    const Sample s0 = trilinear64(g, ox + td * dx, oy + td * dy, oz + td * dz, cache);
    if (!s0.valid) return false;
    if (s0.f >= 0)
        return march64_from(g, cache, ox, oy, oz, dx, dy, dz, inv_len, td + std::fmax(vl, 0.8 * s0.f) * inv_len, t_hi,
                            max_steps, steps, t, true, td, s0.f);
    double tb = td, fb = s0.f;
    while (true) {
        const double ta = tb - std::fmax(vl, -0.8 * fb) * inv_len;
        if (ta < t_lo || !(steps < max_steps)) return false;
        steps++;
        const Sample s = trilinear64(g, ox + ta * dx, oy + ta * dy, oz + ta * dz, cache);
        if (!s.valid) return false;
        if (s.f > 0) {
            t = refine64(g, cache, ox, oy, oz, dx, dy, dz, ta, s.f, tb, fb);
            return true;
        }
        tb = ta;
        fb = s.f;
    }
}

// Trilinear raycast in double. vmap [rows][cols][4] = (x, y, z, depth), nmap
// [rows][cols][4]; misses zero. hint (optional) is a u16-mm depth image at
// this pose: a ray whose pixel has depth d searches [d - m, d + m] starting
// at d (seek64: forward from a positive sample, back to a positive sample
// from a negative one, no hit from an unobserved one); a ray without depth
// takes as d the smaller depth of the nearest pixels with depth to its left
// and right in its 32-pixel row segment (m = hint_margin). steps_out
// (optional) receives the march steps used per pixel.
void orm_raycast(void *h, const double *T, int max_steps, double t_min, double t_max, const uint16_t *hint,
                 double hint_margin, double *vmap, double *nmap, int *steps_out) {
    const Grid64 &g = *(Grid64 *)h;
#pragma omp parallel for schedule(dynamic, 2)
    for (int i = 0; i < g.resi; i++) {
        Cache cache;
        for (int j = 0; j < g.resj; j++) {
            const double dcx = (j - (double)g.cj) / g.fx, dcy = (i - (double)g.ci) / g.fy;
            const double dx = T[0] * dcx + T[1] * dcy + T[2], dy = T[4] * dcx + T[5] * dcy + T[6],
                         dz = T[8] * dcx + T[9] * dcy + T[10];
            const double ox = T[3], oy = T[7], oz = T[11];
            const double inv_len = 1.0 / std::sqrt(dx * dx + dy * dy + dz * dz);
            const size_t pix = (size_t)i * g.resj + j;
            int steps = 0;
            double t = t_min;
            bool hit;
            // hint: own depth, else the smaller depth of the nearest pixels with depth
            // to the left and right within the 32-pixel row segment (one GPU warp)
            unsigned hmm = hint ? hint[pix] : 0u;
            if (hint && hmm == 0) {
                const int j0 = j / 32 * 32, j1 = std::min(j0 + 32, g.resj);
                unsigned dl = 0, dr = 0;
                for (int q = j - 1; q >= j0 && !dl; q--) dl = hint[(size_t)i * g.resj + q];
                for (int q = j + 1; q < j1 && !dr; q++) dr = hint[(size_t)i * g.resj + q];
                hmm = dl && dr ? std::min(dl, dr) : (dl ? dl : dr);
            }
            const double th = hint ? hmm * 1e-3 - hint_margin : 0.0;
            if (hint && th > t_min) {
                hit = seek64(g, cache, ox, oy, oz, dx, dy, dz, inv_len, th + hint_margin, th,
                             std::fmin(t_max, th + 2 * hint_margin), max_steps, steps, t);
            } else {
                hit = march64(g, cache, ox, oy, oz, dx, dy, dz, inv_len, t_min, t_max, max_steps, steps, t);
            }
            double *v = vmap + pix * 4, *n = nmap + pix * 4;
            for (int k = 0; k < 4; k++) v[k] = n[k] = 0;
            if (hit) {
                const double px = ox + t * dx, py = oy + t * dy, pz = oz + t * dz;
                const Sample q = trilinear64(g, px, py, pz, cache);
                const double gn = q.valid ? std::sqrt(q.gx * q.gx + q.gy * q.gy + q.gz * q.gz) : 0;
                if (gn > 0) {
                    v[0] = px;
                    v[1] = py;
                    v[2] = pz;
                    v[3] = t;
                    n[0] = q.gx / gn;
                    n[1] = q.gy / gn;
                    n[2] = q.gz / gn;
                }
            }
            if (steps_out) steps_out[pix] = steps;
        }
    }
}

// Loads blocks (coords, sdf and weight per voxel) into an FP64 grid.
void orm_grid_import(void *h, int n, const int32_t *coords, const float *sdf, const float *w) {
    Grid64 &g = *(Grid64 *)h;
    for (int q = 0; q < n; q++) {
        const int x = coords[q * 3], y = coords[q * 3 + 1], z = coords[q * 3 + 2];
        const uint64_t key = prime_hash(x, y, z);
        auto it = g.map.find(key);
        int idx;
        if (it == g.map.end()) {
            idx = (int)g.blocks.size();
            Block64 *b = new Block64;
            std::memset(b, 0, sizeof(Block64));
            g.blocks.push_back(b);
            g.map.emplace(key, idx);
            g.supers.insert(super_key(floordiv8(x), floordiv8(y), floordiv8(z)));
        } else {
            idx = it->second;
        }
        Block64 &b = *g.blocks[idx];
        b.vb[0] = x;
        b.vb[1] = y;
        b.vb[2] = z;
        for (int v = 0; v < kVox; v++) {
            b.sdf[v] = sdf[(size_t)q * kVox + v];
            b.w[v] = w[(size_t)q * kVox + v];
        }
    }
}

// Adds delta to the TSDF value of voxel v of block (x, y, z); returns 0 if the block is absent.
int orm_grid_add_voxel(void *h, int x, int y, int z, int v, double delta) {
    Grid64 &g = *(Grid64 *)h;
    auto it = g.map.find(prime_hash(x, y, z));
    if (it == g.map.end()) return 0;
    g.blocks[it->second]->sdf[v] += delta;
    return 1;
}

// Loss of the differentiable raycast (the GPU's ss_raycast_loss) in FP64:
// trilinear march from t_min, Newton steps to the root of the trilinear field,
// L = sum of r^2 + lambda (r n.d)^2 over valid pixels (r = t* - d_obs).
double orm_raycast_loss_pixels(void *h, const double *T, const uint16_t *obs, double lambda_n, double r_max,
                               int max_steps, double t_min, double t_max, long long *valid_out, double *per_pixel,
                               double *hit_depth);

double orm_raycast_loss(void *h, const double *T, const uint16_t *obs, double lambda_n, double r_max,
                        int max_steps, double t_min, double t_max, long long *valid_out) {
    return orm_raycast_loss_pixels(h, T, obs, lambda_n, r_max, max_steps, t_min, t_max, valid_out, nullptr,
                                   nullptr);
}

// orm_raycast_loss with each pixel's term in per_pixel and its hit depth t* in
// hit_depth ([resi][resj] each, NaN where the pixel is not valid), each when given.
double orm_raycast_loss_pixels(void *h, const double *T, const uint16_t *obs, double lambda_n, double r_max,
                               int max_steps, double t_min, double t_max, long long *valid_out, double *per_pixel,
                               double *hit_depth) {
    const Grid64 &g = *(Grid64 *)h;
    double total = 0;
    long long valid = 0;
    for (size_t q = 0; q < (size_t)g.resi * g.resj; q++) {
        if (per_pixel) per_pixel[q] = std::nan("");
        if (hit_depth) hit_depth[q] = std::nan("");
    }
#pragma omp parallel for schedule(dynamic, 2) reduction(+ : total, valid)
    for (int i = 0; i < g.resi; i++) {
        Cache cache;
        for (int j = 0; j < g.resj; j++) {
            const double dcx = (j - (double)g.cj) / g.fx, dcy = (i - (double)g.ci) / g.fy;
            const double dx = T[0] * dcx + T[1] * dcy + T[2], dy = T[4] * dcx + T[5] * dcy + T[6],
                         dz = T[8] * dcx + T[9] * dcy + T[10];
            const double ox = T[3], oy = T[7], oz = T[11];
            const double inv_len = 1.0 / std::sqrt(dx * dx + dy * dy + dz * dz);
            int steps = 0;
            double t = t_min;
            if (!march64(g, cache, ox, oy, oz, dx, dy, dz, inv_len, t_min, t_max, max_steps, steps, t)) continue;
            Sample q{false, 0, 0, 0, 0};
            bool ok = true;
            for (int it = 0; it < 6; it++) {
                q = trilinear64(g, ox + t * dx, oy + t * dy, oz + t * dz, cache);
                if (!q.valid) {
                    ok = false;
                    break;
                }
                const double gd = q.gx * dx + q.gy * dy + q.gz * dz;
                if (!(gd < 0)) {
                    ok = false;
                    break;
                }
                const double dt = -q.f / gd;
                if (std::fabs(dt) > 2 * g.vl * inv_len) {
                    ok = false;
                    break;
                }
                t += dt;
                if (std::fabs(dt) < 1e-7 * t) break;
            }
            if (!ok) continue;
            q = trilinear64(g, ox + t * dx, oy + t * dy, oz + t * dz, cache);
            if (!q.valid) continue;
            const double d_obs = obs[(size_t)i * g.resj + j] * 1e-3;
            if (!(d_obs > g.rmin)) continue;
            const double gn = std::sqrt(q.gx * q.gx + q.gy * q.gy + q.gz * q.gz);
            const double c = (q.gx * dx + q.gy * dy + q.gz * dz) / gn;
            const double r = t - d_obs;
            if (!(std::fabs(r) < r_max && c < -0.05)) continue;
            const double term = r * r + lambda_n * (r * c) * (r * c);
            total += term;
            if (per_pixel) per_pixel[(size_t)i * g.resj + j] = term;
            if (hit_depth) hit_depth[(size_t)i * g.resj + j] = t;
            valid++;
        }
    }
    if (valid_out) *valid_out = valid;
    return total;
}

struct Cell64 {
    bool valid;
    double f, g[3], Hxy, Hxz, Hyz, a, b, c;
    const Block64 *blk[8];
    int vox[8];
};

static Cell64 cell64(const Grid64 &g, double px, double py, double pz, Cache &cache) {
    Cell64 r;
    r.valid = false;
    const double vl = g.vl;
    const double ux = px / vl - 0.5, uy = py / vl - 0.5, uz = pz / vl - 0.5;
    const double fx0 = std::floor(ux), fy0 = std::floor(uy), fz0 = std::floor(uz);
    const int ix = (int)fx0, iy = (int)fy0, iz = (int)fz0;
    r.a = ux - fx0;
    r.b = uy - fy0;
    r.c = uz - fz0;
    double s[8];
    for (int k = 0; k < 8; k++) {
        const int vx = ix + (k & 1), vy = iy + ((k >> 1) & 1), vz = iz + (k >> 2);
        const int bx = floordiv8(vx), by = floordiv8(vy), bz = floordiv8(vz);
        const Block64 *b = cached(g, cache, bx, by, bz);
        if (!b) return r;
        const int v = (vx - 8 * bx) + 8 * (vy - 8 * by) + 64 * (vz - 8 * bz);
        if (!(b->w[v] > 0)) return r;
        s[k] = b->sdf[v];
        r.blk[k] = b;
        r.vox[k] = v;
    }
    double f = 0, ga = 0, gb = 0, gc = 0, hab = 0, hac = 0, hbc = 0;
    for (int k = 0; k < 8; k++) {
        const double wx = (k & 1) ? r.a : 1 - r.a, wy = ((k >> 1) & 1) ? r.b : 1 - r.b, wz = (k >> 2) ? r.c : 1 - r.c;
        const double sx = (k & 1) ? 1 : -1, sy = ((k >> 1) & 1) ? 1 : -1, sz = (k >> 2) ? 1 : -1;
        f += s[k] * wx * wy * wz;
        ga += s[k] * sx * wy * wz;
        gb += s[k] * wx * sy * wz;
        gc += s[k] * wx * wy * sz;
        hab += s[k] * sx * sy * wz;
        hac += s[k] * sx * wy * sz;
        hbc += s[k] * wx * sy * sz;
    }
    r.f = f;
    r.g[0] = ga / vl;
    r.g[1] = gb / vl;
    r.g[2] = gc / vl;
    r.Hxy = hab / (vl * vl);
    r.Hxz = hac / (vl * vl);
    r.Hyz = hbc / (vl * vl);
    r.valid = true;
    return r;
}

// Adjoint of orm_raycast_loss in FP64 (same formulas as the GPU adjoint):
// grad[6] = dL/d(omega, upsilon) of the left increment; gvox (optional,
// [blocks][512], zeroed by the caller) accumulates
// dL/d(voxel TSDF value), blocks in the order of orm_grid_export (sorted by
// key). Sequential.
double orm_raycast_loss_grad(void *h, const double *T, const uint16_t *obs, double lambda_n, double r_max,
                             int max_steps, double t_min, double t_max, double *grad, double *gvox) {
    const Grid64 &g = *(Grid64 *)h;
    double total = 0;
    for (int k = 0; k < 6; k++) grad[k] = 0;
    std::unordered_map<const Block64 *, size_t> index_of;
    if (gvox) {
        std::vector<std::pair<uint64_t, int>> items(g.map.begin(), g.map.end());
        std::sort(items.begin(), items.end());
        for (size_t q = 0; q < items.size(); q++) index_of.emplace(g.blocks[items[q].second], q);
    }
    for (int i = 0; i < g.resi; i++) {
        Cache cache;
        for (int j = 0; j < g.resj; j++) {
            const double dcx = (j - (double)g.cj) / g.fx, dcy = (i - (double)g.ci) / g.fy;
            const double d[3] = {T[0] * dcx + T[1] * dcy + T[2], T[4] * dcx + T[5] * dcy + T[6],
                                 T[8] * dcx + T[9] * dcy + T[10]};
            const double ox = T[3], oy = T[7], oz = T[11];
            const double inv_len = 1.0 / std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
            int steps = 0;
            double t = t_min;
            if (!march64(g, cache, ox, oy, oz, d[0], d[1], d[2], inv_len, t_min, t_max, max_steps, steps, t)) continue;
            Cell64 cs;
            bool ok = true;
            for (int it = 0; it < 6; it++) {
                cs = cell64(g, ox + t * d[0], oy + t * d[1], oz + t * d[2], cache);
                if (!cs.valid) {
                    ok = false;
                    break;
                }
                const double gd = cs.g[0] * d[0] + cs.g[1] * d[1] + cs.g[2] * d[2];
                if (!(gd < 0)) {
                    ok = false;
                    break;
                }
                const double dt = -cs.f / gd;
                if (std::fabs(dt) > 2 * g.vl * inv_len) {
                    ok = false;
                    break;
                }
                t += dt;
                if (std::fabs(dt) < 1e-7 * t) break;
            }
            if (!ok) continue;
            cs = cell64(g, ox + t * d[0], oy + t * d[1], oz + t * d[2], cache);
            if (!cs.valid) continue;
            const double d_obs = obs[(size_t)i * g.resj + j] * 1e-3;
            if (!(d_obs > g.rmin)) continue;
            const double gn = std::sqrt(cs.g[0] * cs.g[0] + cs.g[1] * cs.g[1] + cs.g[2] * cs.g[2]);
            const double n[3] = {cs.g[0] / gn, cs.g[1] / gn, cs.g[2] / gn};
            const double c = n[0] * d[0] + n[1] * d[1] + n[2] * d[2];
            const double r = t - d_obs;
            if (!(std::fabs(r) < r_max && c < -0.05)) continue;
            total += r * r + lambda_n * (r * c) * (r * c);
            const double p[3] = {ox + t * d[0], oy + t * d[1], oz + t * d[2]};
            const double a = 2 * r * (1 + lambda_n * c * c), b = 2 * lambda_n * r * r * c;
            const double gd = cs.g[0] * d[0] + cs.g[1] * d[1] + cs.g[2] * d[2];
            double m[3];
            for (int q = 0; q < 3; q++) m[q] = (d[q] - n[q] * c) / gn;
            const double hh[3] = {cs.Hxy * m[1] + cs.Hxz * m[2], cs.Hxy * m[0] + cs.Hyz * m[2], cs.Hxz * m[0] + cs.Hyz * m[1]};
            const double e = (a + b * (hh[0] * d[0] + hh[1] * d[1] + hh[2] * d[2])) / gd;
            const double pg[3] = {p[1] * cs.g[2] - p[2] * cs.g[1], p[2] * cs.g[0] - p[0] * cs.g[2], p[0] * cs.g[1] - p[1] * cs.g[0]};
            const double ph[3] = {p[1] * hh[2] - p[2] * hh[1], p[2] * hh[0] - p[0] * hh[2], p[0] * hh[1] - p[1] * hh[0]};
            const double dn[3] = {d[1] * n[2] - d[2] * n[1], d[2] * n[0] - d[0] * n[2], d[0] * n[1] - d[1] * n[0]};
            for (int q = 0; q < 3; q++) {
                grad[q] += -e * pg[q] + b * (ph[q] + dn[q]);
                grad[3 + q] += -e * cs.g[q] + b * hh[q];
            }
            if (gvox) {
                for (int k = 0; k < 8; k++) {
                    const double wx = (k & 1) ? cs.a : 1 - cs.a, wy = ((k >> 1) & 1) ? cs.b : 1 - cs.b;
                    const double wz = (k >> 2) ? cs.c : 1 - cs.c;
                    const double sx = (k & 1) ? 1 : -1, sy = ((k >> 1) & 1) ? 1 : -1, sz = (k >> 2) ? 1 : -1;
                    const double mdw = (m[0] * sx * wy * wz + m[1] * wx * sy * wz + m[2] * wx * wy * sz) / g.vl;
                    gvox[index_of.at(cs.blk[k]) * kVox + cs.vox[k]] += -e * (wx * wy * wz) + b * mdw;
                }
            }
        }
    }
    return total;
}

static double *g_track_log = nullptr;  // optional per-iteration step norms [level][16] (tests)
static double g_track_eps = 1e-7;        // convergence threshold on the step norm

void orm_track_debug(double *log, double eps) {
    g_track_log = log;
    g_track_eps = eps;
}

static bool chol6(const double *A, const double *b, double *x) {
    double L[36] = {0};
    for (int i = 0; i < 6; i++)
        for (int j = 0; j <= i; j++) {
            double s = A[i * 6 + j];
            for (int k = 0; k < j; k++) s -= L[i * 6 + k] * L[j * 6 + k];
            if (i == j) {
                if (!(s > 1e-12)) return false;
                L[i * 6 + i] = std::sqrt(s);
            } else {
                L[i * 6 + j] = s / L[j * 6 + j];
            }
        }
    double y[6];
    for (int i = 0; i < 6; i++) {
        double s = b[i];
        for (int k = 0; k < i; k++) s -= L[i * 6 + k] * y[k];
        y[i] = s / L[i * 6 + i];
    }
    for (int i = 5; i >= 0; i--) {
        double s = y[i];
        for (int k = i + 1; k < 6; k++) s -= L[k * 6 + i] * x[k];
        x[i] = s / L[i * 6 + i];
    }
    return true;
}

static void se3_left(const double *xi, double *T) {
    const double wx = xi[0], wy = xi[1], wz = xi[2];
    const double th2 = wx * wx + wy * wy + wz * wz, th = std::sqrt(th2);
    double A, B, C;
    if (th < 1e-8) {
        A = 1 - th2 / 6;
        B = 0.5 - th2 / 24;
        C = 1.0 / 6 - th2 / 120;
    } else {
        A = std::sin(th) / th;
        B = (1 - std::cos(th)) / th2;
        C = (th - std::sin(th)) / (th2 * th);
    }
    const double K[9] = {0, -wz, wy, wz, 0, -wx, -wy, wx, 0};
    double K2[9], R[9], V[9];
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) K2[r * 3 + c] = K[r * 3] * K[c] + K[r * 3 + 1] * K[3 + c] + K[r * 3 + 2] * K[6 + c];
    for (int k = 0; k < 9; k++) {
        const double I = (k % 4 == 0) ? 1 : 0;
        R[k] = I + A * K[k] + B * K2[k];
        V[k] = I + B * K[k] + C * K2[k];
    }
    const double t[3] = {V[0] * xi[3] + V[1] * xi[4] + V[2] * xi[5], V[3] * xi[3] + V[4] * xi[4] + V[5] * xi[5],
                         V[6] * xi[3] + V[7] * xi[4] + V[8] * xi[5]};
    double N[12];
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 4; c++)
            N[r * 4 + c] = R[r * 3] * T[c] + R[r * 3 + 1] * T[4 + c] + R[r * 3 + 2] * T[8 + c] + (c == 3 ? t[r] : 0);
    for (int k = 0; k < 12; k++) T[k] = N[k];
}

// Frame-to-model point-to-plane Gauss-Newton in FP64 (the method of
// ss_track.cu): source = depth (level-l pixels are the level-0 pixels
// (i 2^l, j 2^l)), model maps vmap/nmap [rows][cols][4] raycast at Tprev.
// T is the start pose on input and the result on output. Returns the
// inliers of the last iteration.
int orm_track(const uint16_t *depth, int rows, int cols, float fx, float fy, float cx, float cy, const double *vmap,
              const double *nmap, const double *Tprev, double *T, int levels, const int *iters, const double *dist,
              double rmin, double dmax) {
    const double ci = rows - (double)cy, cj = cx;
    double Pi[16];
    rigid_inverse(Tprev, Pi);
    int last_n = 0;
    for (int level = levels - 1; level >= 0; level--) {
        const int lr = (rows + (1 << level) - 1) >> level, lc = (cols + (1 << level) - 1) >> level;
        for (int it = 0; it < iters[level]; it++) {
            double S[29] = {0};
            for (int p = 0; p < lr * lc; p++) {
                const int i = (p / lc) << level, j = (p % lc) << level;
                const double d = depth[(size_t)i * cols + j] * 1e-3;
                if (!(d > rmin) || !(d < dmax)) continue;
                const D3 pc{(j - cj) / fx * d, (i - ci) / fy * d, d};
                const D3 w = dxform(T, pc);
                const D3 q = dxform(Pi, w);
                if (!(q.z > 1e-3)) continue;
                const int ii = (int)std::floor(q.y * fy / q.z + ci + 0.5), jj = (int)std::floor(q.x * fx / q.z + cj + 0.5);
                if (ii < 0 || ii >= rows || jj < 0 || jj >= cols) continue;
                const double *n = nmap + ((size_t)ii * cols + jj) * 4, *v = vmap + ((size_t)ii * cols + jj) * 4;
                if (n[0] == 0 && n[1] == 0 && n[2] == 0) continue;
                const double ex = w.x - v[0], ey = w.y - v[1], ez = w.z - v[2];
                if (ex * ex + ey * ey + ez * ez > dist[level] * dist[level]) continue;
                const double r = n[0] * ex + n[1] * ey + n[2] * ez;
                const double J[6] = {w.y * n[2] - w.z * n[1], w.z * n[0] - w.x * n[2], w.x * n[1] - w.y * n[0],
                                     n[0], n[1], n[2]};
                int k = 0;
                for (int a = 0; a < 6; a++)
                    for (int b = a; b < 6; b++) S[k++] += J[a] * J[b];
                for (int a = 0; a < 6; a++) S[21 + a] += J[a] * r;
                S[27] += r * r;
                S[28] += 1;
            }
            last_n = (int)S[28];
            if (S[28] < 60) break;
            double A[36], b[6], x[6];
            int k = 0;
            for (int r = 0; r < 6; r++)
                for (int c = r; c < 6; c++) A[r * 6 + c] = A[c * 6 + r] = S[k++];
            for (int r = 0; r < 6; r++) b[r] = -S[21 + r];
            if (!chol6(A, b, x)) break;
            se3_left(x, T);
            double step = 0;
            for (int r = 0; r < 6; r++) step += x[r] * x[r];
            if (g_track_log) g_track_log[level * 16 + it] = std::sqrt(step);
            if (std::sqrt(step) < g_track_eps) break;
        }
    }
    return last_n;
}

}  // extern "C"

// ---- mesh of the zero level set (the GPU's ss_grid_extract_mesh) in FP64 ----
// Marching tetrahedra: each cell of 8 observed voxel centres is split into
// the 6 tetrahedra along the diagonal from corner 0 to corner 7 (corner
// n = dx + 2 dy + 4 dz); sdf < 0 is inside; edge vertices by linear
// interpolation; triangles face from the inside corners to the outside ones.
namespace {
const int kTet64[6][4] = {{0, 1, 3, 7}, {0, 1, 5, 7}, {0, 2, 3, 7}, {0, 2, 6, 7}, {0, 4, 5, 7}, {0, 4, 6, 7}};

struct P3 {
    double x, y, z;
};

P3 edge64(const P3 &p, double sp, const P3 &q, double sq) {
    const double t = sp / (sp - sq);
    return {p.x + t * (q.x - p.x), p.y + t * (q.y - p.y), p.z + t * (q.z - p.z)};
}

void emit64(std::vector<double> &out, P3 a, P3 b, P3 c, const P3 &dir) {
    const double ux = b.x - a.x, uy = b.y - a.y, uz = b.z - a.z, vx = c.x - a.x, vy = c.y - a.y, vz = c.z - a.z;
    const double nx = uy * vz - uz * vy, ny = uz * vx - ux * vz, nz = ux * vy - uy * vx;
    if (nx * dir.x + ny * dir.y + nz * dir.z < 0) std::swap(b, c);
    for (const P3 *q : {&a, &b, &c}) {
        out.push_back(q->x);
        out.push_back(q->y);
        out.push_back(q->z);
    }
}

void tetra64(std::vector<double> &out, const P3 *p, const double *s, const int *t) {
    int in[4], outc[4], ni = 0, no = 0;
    for (int k = 0; k < 4; k++) {
        if (s[t[k]] < 0) in[ni++] = t[k];
        else outc[no++] = t[k];
    }
    if (ni == 0 || ni == 4) return;
    P3 ci{0, 0, 0}, co{0, 0, 0};
    for (int k = 0; k < ni; k++) ci = {ci.x + p[in[k]].x, ci.y + p[in[k]].y, ci.z + p[in[k]].z};
    for (int k = 0; k < no; k++) co = {co.x + p[outc[k]].x, co.y + p[outc[k]].y, co.z + p[outc[k]].z};
    const P3 dir{co.x / no - ci.x / ni, co.y / no - ci.y / ni, co.z / no - ci.z / ni};
    if (ni == 1 || ni == 3) {
        const int a = ni == 1 ? in[0] : outc[0];
        const int *r = ni == 1 ? outc : in;
        emit64(out, edge64(p[a], s[a], p[r[0]], s[r[0]]), edge64(p[a], s[a], p[r[1]], s[r[1]]),
               edge64(p[a], s[a], p[r[2]], s[r[2]]), dir);
    } else {
        const int a = in[0], b = in[1], c = outc[0], d = outc[1];
        const P3 ac = edge64(p[a], s[a], p[c], s[c]), ad = edge64(p[a], s[a], p[d], s[d]);
        const P3 bd = edge64(p[b], s[b], p[d], s[d]), bc = edge64(p[b], s[b], p[c], s[c]);
        emit64(out, ac, ad, bd, dir);
        emit64(out, ac, bd, bc, dir);
    }
}
}  // namespace

// ---- marching cubes (the GPU's ss_grid_extract_mesh_cubes) in FP64 ----
// Cube corners m = 0..7 at (0,0,0) (1,0,0) (1,1,0) (0,1,0) (0,0,1) (1,0,1)
// (1,1,1) (0,1,1), edges 0-3 / 4-7 around the z = 0 / z = 1 faces, 8-11
// upwards; corner bit set when sdf < 0. A case's polygons: per cube face the
// sign-changing edges are paired (two: one segment; four: each negative
// corner's two edges), segments chain into loops, a loop is oriented by its
// Newell normal through the edge midpoints against the negative -> positive
// corner directions, and fanned from its first vertex.
namespace {
const int kMcEdge[12][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}, {4, 5}, {5, 6}, {6, 7}, {7, 4}, {0, 4}, {1, 5}, {2, 6}, {3, 7}};
const int kMcPos[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0}, {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
const int kMcFaceCorner[6][4] = {{0, 1, 2, 3}, {4, 5, 6, 7}, {0, 1, 5, 4}, {3, 2, 6, 7}, {0, 3, 7, 4}, {1, 2, 6, 5}};
const int kMcFaceEdge[6][4] = {{0, 1, 2, 3}, {4, 5, 6, 7}, {0, 9, 4, 8}, {2, 10, 6, 11}, {3, 11, 7, 8}, {1, 10, 5, 9}};

std::vector<int> mc_case(int cs) {
    std::vector<int> adj[12];
    bool cross[12];
    for (int e = 0; e < 12; e++) cross[e] = ((cs >> kMcEdge[e][0]) & 1) != ((cs >> kMcEdge[e][1]) & 1);
    for (int f = 0; f < 6; f++) {
        std::vector<int> cr;
        for (int q = 0; q < 4; q++)
            if (cross[kMcFaceEdge[f][q]]) cr.push_back(q);
        if (cr.size() == 2) {
            adj[kMcFaceEdge[f][cr[0]]].push_back(kMcFaceEdge[f][cr[1]]);
            adj[kMcFaceEdge[f][cr[1]]].push_back(kMcFaceEdge[f][cr[0]]);
        } else if (cr.size() == 4) {
            for (int q = 0; q < 4; q++) {
                if (!((cs >> kMcFaceCorner[f][q]) & 1)) continue;
                const int a = kMcFaceEdge[f][q], b = kMcFaceEdge[f][(q + 3) % 4];
                adj[a].push_back(b);
                adj[b].push_back(a);
            }
        }
    }
    std::vector<int> tri;
    bool used[12] = {};
    for (int e = 0; e < 12; e++) {
        if (!cross[e] || used[e]) continue;
        std::vector<int> loop;
        int prev = -1, cur = e;
        while (!used[cur]) {
            used[cur] = true;
            loop.push_back(cur);
            const int nx = adj[cur][0] != prev ? adj[cur][0] : adj[cur][1];
            prev = cur;
            cur = nx;
        }
        long n[3] = {0, 0, 0}, d[3] = {0, 0, 0};
        for (size_t k = 0; k < loop.size(); k++) {
            const int ea = loop[k], eb = loop[(k + 1) % loop.size()];
            long pa[3], pb[3];
            for (int c = 0; c < 3; c++) {
                pa[c] = kMcPos[kMcEdge[ea][0]][c] + kMcPos[kMcEdge[ea][1]][c];
                pb[c] = kMcPos[kMcEdge[eb][0]][c] + kMcPos[kMcEdge[eb][1]][c];
            }
            n[0] += (pa[1] - pb[1]) * (pa[2] + pb[2]);
            n[1] += (pa[2] - pb[2]) * (pa[0] + pb[0]);
            n[2] += (pa[0] - pb[0]) * (pa[1] + pb[1]);
            const int c0 = kMcEdge[ea][0], c1 = kMcEdge[ea][1];
            const int neg = ((cs >> c0) & 1) ? c0 : c1, pos = neg == c0 ? c1 : c0;
            for (int c = 0; c < 3; c++) d[c] += kMcPos[pos][c] - kMcPos[neg][c];
        }
        const bool flip = n[0] * d[0] + n[1] * d[1] + n[2] * d[2] < 0;
        for (size_t k = 1; k + 1 < loop.size(); k++) {
            tri.push_back(loop[0]);
            tri.push_back(flip ? loop[k + 1] : loop[k]);
            tri.push_back(flip ? loop[k] : loop[k + 1]);
        }
    }
    return tri;
}
}  // namespace

// Marching-cubes triangles (9 doubles each) into tris (up to cap); returns the total count.
extern "C" long long orm_extract_mesh_cubes(void *h, long long cap, double *tris) {
    const Grid64 &g = *(Grid64 *)h;
    static const int kCell[8] = {0, 1, 3, 2, 4, 5, 7, 6};  // table corner -> cell corner dx + 2 dy + 4 dz
    std::vector<std::vector<int>> table(256);
    for (int cs = 0; cs < 256; cs++) table[cs] = mc_case(cs);
    std::vector<double> out;
    Cache cache;
    for (const Block64 *blk : g.blocks) {
        const int bx = blk->vb[0], by = blk->vb[1], bz = blk->vb[2];
        for (int c = 0; c < kVox; c++) {
            const int i = c & 7, j = (c >> 3) & 7, k = c >> 6;
            P3 p[8];
            double s[8];
            bool ok = true;
            int cs = 0;
            for (int m = 0; m < 8 && ok; m++) {
                const int n = kCell[m];
                const int vi = i + (n & 1), vj = j + ((n >> 1) & 1), vk = k + (n >> 2);
                const Block64 *b = cached(g, cache, bx + (vi >> 3), by + (vj >> 3), bz + (vk >> 3));
                const int v = (vi & 7) + 8 * (vj & 7) + 64 * (vk & 7);
                if (!b || !(b->w[v] > 0)) {
                    ok = false;
                    break;
                }
                s[m] = b->sdf[v];
                if (s[m] < 0) cs |= 1 << m;
                p[m] = {((double)(bx * 8 + vi) + 0.5) * g.vl, ((double)(by * 8 + vj) + 0.5) * g.vl,
                        ((double)(bz * 8 + vk) + 0.5) * g.vl};
            }
            if (!ok || cs == 0 || cs == 255) continue;
            for (int e : table[cs]) {
                // from the edge's lower-coordinate end
                int a = kMcEdge[e][0], b = kMcEdge[e][1];
                if (kMcPos[a][0] + kMcPos[a][1] + kMcPos[a][2] > kMcPos[b][0] + kMcPos[b][1] + kMcPos[b][2]) std::swap(a, b);
                const P3 q = edge64(p[a], s[a], p[b], s[b]);
                out.push_back(q.x);
                out.push_back(q.y);
                out.push_back(q.z);
            }
        }
    }
    const long long n = (long long)out.size() / 9;
    if (tris) std::memcpy(tris, out.data(), (size_t)std::min(n, cap) * 9 * sizeof(double));
    return n;
}

// Triangles (9 doubles each) into tris (up to cap); returns the total count.
extern "C" long long orm_extract_mesh(void *h, long long cap, double *tris) {
    const Grid64 &g = *(Grid64 *)h;
    std::vector<double> out;
    Cache cache;
    for (const Block64 *blk : g.blocks) {
        const int bx = blk->vb[0], by = blk->vb[1], bz = blk->vb[2];
        for (int c = 0; c < kVox; c++) {
            const int i = c & 7, j = (c >> 3) & 7, k = c >> 6;
            P3 p[8];
            double s[8];
            bool ok = true;
            for (int n = 0; n < 8 && ok; n++) {
                const int vi = i + (n & 1), vj = j + ((n >> 1) & 1), vk = k + (n >> 2);
                const Block64 *b = cached(g, cache, bx + (vi >> 3), by + (vj >> 3), bz + (vk >> 3));
                if (!b) {
                    ok = false;
                    break;
                }
                const int v = (vi & 7) + 8 * (vj & 7) + 64 * (vk & 7);
                if (!(b->w[v] > 0)) {
                    ok = false;
                    break;
                }
                s[n] = b->sdf[v];
                p[n] = {((double)(bx * 8 + vi) + 0.5) * g.vl, ((double)(by * 8 + vj) + 0.5) * g.vl,
                        ((double)(bz * 8 + vk) + 0.5) * g.vl};
            }
            if (!ok) continue;
            for (int t = 0; t < 6; t++) tetra64(out, p, s, kTet64[t]);
        }
    }
    const long long n = (long long)out.size() / 9;
    if (tris) std::memcpy(tris, out.data(), (size_t)std::min(n, cap) * 9 * sizeof(double));
    return n;
}
