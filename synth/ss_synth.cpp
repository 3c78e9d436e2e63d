// ss_synth.cpp — seeded synthetic RGB-D sequences (analytic rooms with
// spheres and boxes) that stand in for the reference's recorded scenes.
//
// Camera model of the reference (GPUVoxelGrid.h:229-237, with ci = rows - cy,
// cj = cx): pixel (i, j) at depth z back-projects to
// ((j - cj) / fx * z, (i - ci) / fy * z, z), so every rendered frame is a valid
// input of the reference's integrate. Depth is the camera-frame z of the
// first surface hit, in uint16 millimetres; rendering is exact ray-primitive
// intersection in double precision. Noise model (depth-dependent Gaussian,
// sigma = 0.0012 + 0.0019 (z - 0.4)^2 m) and pixel dropout use a counter-based
// generator keyed by (seed, frame, pixel), so frames can be rendered in any
// order and in parallel with identical results.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

namespace {

struct Prim {
    int kind;  // 0 sphere, 1 box
    double c[3], r;
    double lo[3], hi[3];
    uint8_t col[3];
};

struct Scene {
    double room_lo[3], room_hi[3];
    uint8_t wall_col[6][3];
    std::vector<Prim> prims;
};

inline uint64_t splitmix(uint64_t x) {
    x += 0x9e3779b97f4a7c15ull;
    x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
    x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
    return x ^ (x >> 31);
}

struct Rng {
    uint64_t s;
    explicit Rng(uint64_t seed) : s(splitmix(seed)) {}
    uint64_t next() {
        s = splitmix(s);
        return s;
    }
    double uni() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
    double range(double a, double b) { return a + (b - a) * uni(); }
};

inline double u01(uint64_t key) { return ((double)(splitmix(key) >> 11) + 0.5) * (1.0 / 9007199254740992.0); }

// Trajectory of the camera centre: a smooth closed curve around the room
// centre (radius 0.16 of the smaller horizontal extent, one loop per 500
// frames) at 0.3 of the room height. The camera turns 0.6 deg per frame about
// the vertical and looks 25 +- 8 deg downwards, so every view holds a wall,
// the floor and the objects standing on it (a view of one flat wall and one
// sphere leaves a rotation that point-to-plane ICP cannot observe).
// Per-frame motion: <= 6 mm and < 1 deg.
void traj_point(const Scene &s, int t, int n, double phase, double *p, double *yaw, double *pitch) {
    const double cx = 0.5 * (s.room_lo[0] + s.room_hi[0]), cy = 0.5 * (s.room_lo[1] + s.room_hi[1]);
    const double h = s.room_hi[2] - s.room_lo[2];
    const double ext = std::fmin(s.room_hi[0] - s.room_lo[0], s.room_hi[1] - s.room_lo[1]);
    const double rad = 0.16 * ext;
    const double w = 2.0 * M_PI / 500.0;  // one loop per 500 frames
    p[0] = cx + rad * std::cos(w * t + phase);
    p[1] = cy + 0.8 * rad * std::sin(w * t + phase);
    p[2] = s.room_lo[2] + 0.30 * h + 0.04 * h * std::sin(2.3 * w * t);
    *yaw = phase + (0.6 * M_PI / 180.0) * t;
    *pitch = -(25.0 * M_PI / 180.0) + (8.0 * M_PI / 180.0) * std::sin(1.7 * w * t + phase);
    (void)n;
}

// camera -> world rotation for yaw about world z (up) and pitch about camera x.
// Camera axes: x right, y down, z forward.
void cam_rot(double yaw, double pitch, double *R) {
    const double f[3] = {std::cos(yaw) * std::cos(pitch), std::sin(yaw) * std::cos(pitch), std::sin(pitch)};
    const double up[3] = {0, 0, 1};
    double rx[3] = {f[1] * up[2] - f[2] * up[1], f[2] * up[0] - f[0] * up[2], f[0] * up[1] - f[1] * up[0]};
    const double nrx = std::sqrt(rx[0] * rx[0] + rx[1] * rx[1] + rx[2] * rx[2]);
    for (double &v : rx) v /= nrx;
    // camera y (down) = z x x
    const double dy[3] = {f[1] * rx[2] - f[2] * rx[1], f[2] * rx[0] - f[0] * rx[2], f[0] * rx[1] - f[1] * rx[0]};
    for (int r = 0; r < 3; r++) {
        R[r * 3 + 0] = rx[r];
        R[r * 3 + 1] = dy[r];
        R[r * 3 + 2] = f[r];
    }
}

bool ray_sphere(const Prim &p, const double *o, const double *d, double &t) {
    const double oc[3] = {o[0] - p.c[0], o[1] - p.c[1], o[2] - p.c[2]};
    const double a = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
    const double b = oc[0] * d[0] + oc[1] * d[1] + oc[2] * d[2];
    const double c = oc[0] * oc[0] + oc[1] * oc[1] + oc[2] * oc[2] - p.r * p.r;
    const double disc = b * b - a * c;
    if (disc < 0) return false;
    const double sq = std::sqrt(disc);
    double t0 = (-b - sq) / a;
    if (t0 <= 1e-9) t0 = (-b + sq) / a;
    if (t0 <= 1e-9) return false;
    t = t0;
    return true;
}

bool ray_box(const double *lo, const double *hi, const double *o, const double *d, double &t, int &axis) {
    double tn = -1e300, tf = 1e300;
    int ax = -1;
    for (int k = 0; k < 3; k++) {
        if (std::fabs(d[k]) < 1e-15) {
            if (o[k] < lo[k] || o[k] > hi[k]) return false;
            continue;
        }
        double t1 = (lo[k] - o[k]) / d[k], t2 = (hi[k] - o[k]) / d[k];
        if (t1 > t2) std::swap(t1, t2);
        if (t1 > tn) {
            tn = t1;
            ax = k;
        }
        tf = std::fmin(tf, t2);
    }
    if (tn > tf || tn <= 1e-9) return false;
    t = tn;
    axis = ax;
    return true;
}

void make_scene(Scene &s, int kind, uint64_t seed) {
    Rng rng(seed);
    int ns, nb;
    double L[3];
    if (kind == 1) {  // 2x2x2 m, 6 spheres (r 0.1-0.4), 4 boxes
        L[0] = 2;
        L[1] = 2;
        L[2] = 2;
        ns = 6;
        nb = 4;
    } else {  // 4x4x3 m, 40 primitives
        L[0] = 4;
        L[1] = 4;
        L[2] = 3;
        ns = 24;
        nb = 16;
    }
    for (int k = 0; k < 3; k++) {
        s.room_lo[k] = 0;
        s.room_hi[k] = L[k];
    }
    for (int w = 0; w < 6; w++)
        for (int c = 0; c < 3; c++) s.wall_col[w][c] = (uint8_t)rng.range(60, 230);
    // keep primitives away from the camera path (a ring around the centre)
    const double cx = 0.5 * L[0], cy = 0.5 * L[1];
    const double ext = std::fmin(L[0], L[1]);
    const double rad = 0.16 * ext;
    auto clear_of_path = [&](const double *c, double r) {
        const double dx = c[0] - cx, dy = c[1] - cy;
        const double rho = std::sqrt(dx * dx + dy * dy);
        return std::fabs(rho - rad) > r + 0.45 && rho > r + 0.25;
    };
    // Objects along the walls give every view structure in three directions
    // (a view of only a wall and the floor cannot fix the motion along their
    // intersection): spheres and boxes are spread over the four walls in turn.
    int tries = 0;
    while ((int)s.prims.size() < ns && tries < 100000) {
        tries++;
        Prim p{};
        p.kind = 0;
        p.r = rng.range(0.1, 0.4);
        for (int k = 0; k < 3; k++) p.c[k] = rng.range(p.r + 0.05, L[k] - p.r - 0.05);
        const int idx = (int)s.prims.size();
        if (idx % 2 == 0) {  // every other sphere rests on the floor near a wall
            const int wall = (idx / 2) % 4;
            const int ax = wall / 2;
            p.c[ax] = (wall & 1) ? L[ax] - p.r - rng.range(0.05, 0.5) : p.r + rng.range(0.05, 0.5);
            p.c[2] = p.r;
        }
        if (!clear_of_path(p.c, p.r)) continue;
        for (int c = 0; c < 3; c++) p.col[c] = (uint8_t)rng.range(30, 255);
        s.prims.push_back(p);
    }
    int nbox = 0;
    while (nbox < nb && tries < 200000) {
        tries++;
        Prim p{};
        p.kind = 1;
        double half[3], c[3];
        for (int k = 0; k < 3; k++) half[k] = rng.range(0.08, 0.3);
        for (int k = 0; k < 3; k++) c[k] = rng.range(half[k] + 0.05, L[k] - half[k] - 0.05);
        if (nbox % 4 != 3) {  // three boxes in four stand on the floor against a wall
            const int wall = nbox % 4;
            const int ax = wall / 2;
            c[ax] = (wall & 1) ? L[ax] - half[ax] : half[ax];
            c[2] = half[2];
        } else if (kind == 1 || rng.uni() < 0.5) {
            c[2] = half[2];
        }
        const double rr = std::sqrt(half[0] * half[0] + half[1] * half[1]);
        if (!clear_of_path(c, rr)) continue;
        for (int k = 0; k < 3; k++) {
            p.lo[k] = c[k] - half[k];
            p.hi[k] = c[k] + half[k];
            p.c[k] = c[k];
        }
        for (int q = 0; q < 3; q++) p.col[q] = (uint8_t)rng.range(30, 255);
        s.prims.push_back(p);
        nbox++;
    }
}

// Renders rows [r0, r1) of one frame into the full-frame buffers.
void render(const Scene &s, const double *pose, int rows, int cols, double fx, double fy, double cx, double cy,
            int noise, uint64_t seed, int frame, int r0, int r1, uint16_t *depth, uint8_t *rgb) {
    const double ci = rows - cy, cj = cx;
    const double R[9] = {pose[0], pose[1], pose[2], pose[4], pose[5], pose[6], pose[8], pose[9], pose[10]};
    const double o[3] = {pose[3], pose[7], pose[11]};
    const double light[3] = {0.3, 0.5, -0.81};
    for (int i = r0; i < r1; i++) {
        for (int j = 0; j < cols; j++) {
            const double dc[3] = {(j - cj) / fx, (i - ci) / fy, 1.0};
            const double d[3] = {R[0] * dc[0] + R[1] * dc[1] + R[2] * dc[2], R[3] * dc[0] + R[4] * dc[1] + R[5] * dc[2],
                                 R[6] * dc[0] + R[7] * dc[1] + R[8] * dc[2]};
            // room interior: nearest exit plane
            double tbest = 1e300;
            int wall = -1;
            for (int k = 0; k < 3; k++) {
                if (std::fabs(d[k]) < 1e-15) continue;
                const double t = d[k] > 0 ? (s.room_hi[k] - o[k]) / d[k] : (s.room_lo[k] - o[k]) / d[k];
                if (t > 0 && t < tbest) {
                    tbest = t;
                    wall = k * 2 + (d[k] > 0 ? 1 : 0);
                }
            }
            const uint8_t *col = wall >= 0 ? s.wall_col[wall] : s.wall_col[0];
            double nrm[3] = {0, 0, 0};
            if (wall >= 0) nrm[wall / 2] = (wall & 1) ? -1.0 : 1.0;
            for (const Prim &p : s.prims) {
                double t;
                if (p.kind == 0) {
                    if (ray_sphere(p, o, d, t) && t < tbest) {
                        tbest = t;
                        col = p.col;
                        for (int k = 0; k < 3; k++) nrm[k] = (o[k] + t * d[k] - p.c[k]) / p.r;
                    }
                } else {
                    int ax;
                    if (ray_box(p.lo, p.hi, o, d, t, ax) && t < tbest) {
                        tbest = t;
                        col = p.col;
                        nrm[0] = nrm[1] = nrm[2] = 0;
                        nrm[ax] = d[ax] > 0 ? -1.0 : 1.0;
                    }
                }
            }
            const size_t pix = (size_t)i * cols + j;
            double z = tbest;  // dc.z == 1, so the ray parameter is the camera-frame depth
            const uint64_t key = splitmix(seed ^ splitmix((uint64_t)frame * 0x100000001ull + pix));
            if (noise) {
                const double sigma = 0.0012 + 0.0019 * (z - 0.4) * (z - 0.4);
                const double u1 = u01(key), u2 = u01(key ^ 0xabcdef1234567ull);
                const double g = std::sqrt(-2.0 * std::log(u1)) * std::cos(2.0 * M_PI * u2);
                z += sigma * g;
                if (u01(key ^ 0x5555aaaa5555aaaaull) < 0.05) z = 0;  // 5% dropout
            }
            double mm = std::floor(z * 1000.0 + 0.5);
            if (!(z > 0) || mm > 65535.0 || wall < 0) mm = 0;
            depth[pix] = (uint16_t)mm;
            if (rgb) {
                const double lam = std::fabs(nrm[0] * light[0] + nrm[1] * light[1] + nrm[2] * light[2]);
                const double shade = 0.35 + 0.65 * lam;
                // 10 cm checker on every surface gives colour texture
                const double P[3] = {o[0] + tbest * d[0], o[1] + tbest * d[1], o[2] + tbest * d[2]};
                const int chk = ((int)std::floor(P[0] * 10) + (int)std::floor(P[1] * 10) + (int)std::floor(P[2] * 10)) & 1;
                for (int c = 0; c < 3; c++) {
                    double v = col[c] * shade * (chk ? 1.0 : 0.8);
                    rgb[pix * 3 + c] = (uint8_t)std::fmin(255.0, std::floor(v + 0.5));
                }
            }
        }
    }
}

}  // namespace

extern "C" {

void *synth_scene_new(int kind, uint64_t seed) {
    Scene *s = new Scene;
    make_scene(*s, kind, seed);
    return s;
}

void synth_scene_free(void *h) { delete (Scene *)h; }

int synth_num_primitives(void *h) { return (int)((Scene *)h)->prims.size(); }

// Primitive table: per primitive 11 doubles (kind, c[3], r, lo[3], hi[3]).
void synth_primitives(void *h, double *out) {
    const Scene &s = *(Scene *)h;
    for (size_t k = 0; k < s.prims.size(); k++) {
        const Prim &p = s.prims[k];
        double *o = out + k * 11;
        o[0] = p.kind;
        for (int q = 0; q < 3; q++) o[1 + q] = p.c[q];
        o[4] = p.r;
        for (int q = 0; q < 3; q++) o[5 + q] = p.lo[q];
        for (int q = 0; q < 3; q++) o[8 + q] = p.hi[q];
    }
}

// Camera->world poses, row-major 4x4 doubles, n frames.
void synth_trajectory(void *h, int n, uint64_t seed, double *poses) {
    const Scene &s = *(Scene *)h;
    Rng rng(seed);
    const double phase = rng.range(0.0, 2.0 * M_PI);
    for (int t = 0; t < n; t++) {
        double p[3], yaw, pitch, R[9];
        traj_point(s, t, n, phase, p, &yaw, &pitch);
        cam_rot(yaw, pitch, R);
        double *T = poses + (size_t)t * 16;
        for (int r = 0; r < 3; r++) {
            for (int c = 0; c < 3; c++) T[r * 4 + c] = R[r * 3 + c];
            T[r * 4 + 3] = p[r];
        }
        T[12] = T[13] = T[14] = 0;
        T[15] = 1;
    }
}

// Renders n frames (poses n x 16) in parallel into depth [n][rows][cols] and
// rgb [n][rows][cols][3] (rgb may be null). frame0 offsets the noise keys.
void synth_render(void *h, int n, const double *poses, int rows, int cols, double fx, double fy, double cx, double cy,
                  int noise, uint64_t seed, int frame0, uint16_t *depth, uint8_t *rgb) {
    const Scene &s = *(Scene *)h;
    const size_t npix = (size_t)rows * cols;
#pragma omp parallel for schedule(dynamic, 1) collapse(2)
    for (int f = 0; f < n; f++) {
        for (int band = 0; band < 16; band++) {
            const int r0 = rows * band / 16, r1 = rows * (band + 1) / 16;
            render(s, poses + (size_t)f * 16, rows, cols, fx, fy, cx, cy, noise, seed, f + frame0, r0, r1,
                   depth + f * npix, rgb ? rgb + f * npix * 3 : nullptr);
        }
    }
}

}  // extern "C"
