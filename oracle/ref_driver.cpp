// ref_driver.cpp — C entry points over the reference's OWN hot-path code.
//
// TEST INFRASTRUCTURE ONLY. Linked into oracle/_ref/libss_ref.so together
// with the reference's unmodified sources, compiled where they lie
// (src/VoxelGrid/GPUVoxelGrid.cpp, kokkosFunctions.cpp,
// src/postprocessing/kokkosICP.cpp, src/utils/imageutil.cpp,
// src/utils/kokkosUtil.cpp) against ref_stub/ in place of Kokkos, Eigen,
// Open3D and OpenCV (what each stand-in does is written in
// ref_stub/ss_ref_stub.h). Tests and the fixture script call it to pin the
// oracle (ss_oracle.cpp) and, through committed fixtures, the CUDA path.
//
// Entry points (row-major images and 4x4 matrices, as the library's C-ABI):
//   ssref_grid_new / _free            GPUVoxelGrid(c, trunc, vl, resi, resj)  GPUVoxelGrid.cpp:10-30
//   ssref_set_intrinsic               setIntrinsic                            GPUVoxelGrid.cpp:253-266
//   ssref_fuse                        integrate / deIntegrate (View overload)  GPUVoxelGrid.cpp:41-136
//   ssref_raycast                     raycast + rayPcd / rayColorPcd           GPUVoxelGrid.cpp:139-147
//   ssref_clean                       cleanMemory                              GPUVoxelGrid.cpp:185-196
//   ssref_count / ssref_dump          the map's live entries (UnorderedMap valid_at / value_at)
//   ssref_mc_units                    marchingCubesHost's voxel copy into the Open3D units
//                                                                              GPUVoxelGrid.cpp:200-251
//   ssref_depth_to_pcd, ssref_normals CreatePcdFromDepthView, CalculateNormalsFromPCDView
//                                                                              imageutil.cpp:89-157
//   ssref_kokkos_icp                  kokkosICP(View, View, tx, ty, type, rmse) kokkosICP.cpp:25-210
#include <algorithm>
#include <cmath>
#include <cstring>
#include <sstream>

#include "VoxelGrid/GPUVoxelGrid.h"
#include "postprocessing/kokkosICP.h"
#include "utils/imageutil.h"

// ---- definitions the reference keeps in files outside the path ---------------
namespace threadCom {
std::atomic<bool> unmeshed_data{false};  // src/core/threadCom.cpp:18
}
open3d::camera::PinholeCameraIntrinsic g_intrinsic;  // src/core/threadCom.cpp:75
std::shared_ptr<open3d::geometry::LineSet> getOrigin() { return std::make_shared<open3d::geometry::LineSet>(); }

namespace open3d {
namespace pipelines {
namespace integration {
std::shared_ptr<ScalableTSDFVolume> ss_stub_last_volume;
}
}  // namespace pipelines
}  // namespace open3d

// ---- Eigen stand-ins ----------------------------------------------------------
namespace {

double det3(const double a[9]) {  // row-major 3x3, expanded along its first row
    return a[0] * (a[4] * a[8] - a[5] * a[7]) - a[1] * (a[3] * a[8] - a[5] * a[6]) +
           a[2] * (a[3] * a[7] - a[4] * a[6]);
}

// Row-major 4x4 inverse by the adjugate in double, rounded to float once —
// the same function as the library's host-side inverse of an integration pose.
void inverse4_adjugate(const float *E, float *out) {
    double m[16], cof[16];
    for (int k = 0; k < 16; k++) m[k] = E[k];
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) {
            double sub[9];
            int n = 0;
            for (int r = 0; r < 4; r++)
                if (r != i)
                    for (int c = 0; c < 4; c++)
                        if (c != j) sub[n++] = m[4 * r + c];
            const double d = det3(sub);
            cof[4 * i + j] = ((i + j) & 1) ? -d : d;
        }
    const double det = m[0] * cof[0] + m[1] * cof[1] + m[2] * cof[2] + m[3] * cof[3];
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) out[4 * j + i] = (float)(cof[4 * i + j] / det);
}

// Symmetric 3x3 eigen-decomposition by cyclic Jacobi rotations (A row-major,
// destroyed): eigenvalues on A's diagonal, eigenvectors in the columns of Q.
void sym_eig3(double A[9], double Q[9]) {
    for (int k = 0; k < 9; k++) Q[k] = (k % 4 == 0) ? 1.0 : 0.0;
    for (int sweep = 0; sweep < 50; sweep++) {
        const double off = A[1] * A[1] + A[2] * A[2] + A[5] * A[5];
        if (off == 0.0) break;
        for (int p = 0; p < 2; p++)
            for (int q = p + 1; q < 3; q++) {
                const double apq = A[3 * p + q];
                if (apq == 0.0) continue;
                const double theta = (A[3 * q + q] - A[3 * p + p]) / (2.0 * apq);
                const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
                const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
                for (int k = 0; k < 3; k++) {  // A <- A J  (columns p, q)
                    const double akp = A[3 * k + p], akq = A[3 * k + q];
                    A[3 * k + p] = c * akp - s * akq;
                    A[3 * k + q] = s * akp + c * akq;
                }
                for (int k = 0; k < 3; k++) {  // A <- J^T A  (rows p, q)
                    const double apk = A[3 * p + k], aqk = A[3 * q + k];
                    A[3 * p + k] = c * apk - s * aqk;
                    A[3 * q + k] = s * apk + c * aqk;
                }
                for (int k = 0; k < 3; k++) {
                    const double qkp = Q[3 * k + p], qkq = Q[3 * k + q];
                    Q[3 * k + p] = c * qkp - s * qkq;
                    Q[3 * k + q] = s * qkp + c * qkq;
                }
            }
    }
}

}  // namespace

namespace Eigen {

void ss_stub_inverse4f(const float *cm, float *cm_out) {
    float rm[16], ri[16];
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) rm[4 * i + j] = cm[i + 4 * j];
    inverse4_adjugate(rm, ri);
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) cm_out[i + 4 * j] = ri[4 * i + j];
}

void ss_stub_inverse4d(const double *cm, double *cm_out) {
    double a[4][8];
    for (int r = 0; r < 4; r++)
        for (int c = 0; c < 8; c++) a[r][c] = c < 4 ? cm[r + 4 * c] : (c - 4 == r ? 1.0 : 0.0);
    for (int col = 0; col < 4; col++) {
        int piv = col;
        for (int r = col + 1; r < 4; r++)
            if (std::fabs(a[r][col]) > std::fabs(a[piv][col])) piv = r;
        if (piv != col)
            for (int c = 0; c < 8; c++) std::swap(a[piv][c], a[col][c]);
        const double d = a[col][col];
        for (int c = 0; c < 8; c++) a[col][c] /= d;
        for (int r = 0; r < 4; r++)
            if (r != col) {
                const double f = a[r][col];
                for (int c = 0; c < 8; c++) a[r][c] -= f * a[col][c];
            }
    }
    for (int r = 0; r < 4; r++)
        for (int c = 0; c < 4; c++) cm_out[r + 4 * c] = a[r][4 + c];
}

// H = U diag(S) V^T from the eigen-decomposition of H^T H: V its eigenvectors,
// S the square roots of its eigenvalues, U = H V / S (full-rank H; a zero
// singular value takes the cross product of the other two columns of U).
void ss_stub_svd3(const double *Hc, double *Uc, double *S, double *Vc) {
    double H[9], A[9], V[9], U[9];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) H[3 * i + j] = Hc[i + 3 * j];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            double s = 0;
            for (int k = 0; k < 3; k++) s += H[3 * k + i] * H[3 * k + j];
            A[3 * i + j] = s;
        }
    sym_eig3(A, V);
    int order[3] = {0, 1, 2};
    std::sort(order, order + 3, [&](int a, int b) { return A[4 * a] > A[4 * b]; });
    double Vs[9];
    for (int j = 0; j < 3; j++) {
        S[j] = std::sqrt(std::max(A[4 * order[j]], 0.0));
        for (int i = 0; i < 3; i++) Vs[3 * i + j] = V[3 * i + order[j]];
    }
    int zero_col = -1;
    for (int j = 0; j < 3; j++) {
        if (S[j] > 1e-300 * (S[0] + 1e-300) && S[j] > 0) {
            for (int i = 0; i < 3; i++) {
                double s = 0;
                for (int k = 0; k < 3; k++) s += H[3 * i + k] * Vs[3 * k + j];
                U[3 * i + j] = s / S[j];
            }
        } else {
            zero_col = j;
            for (int i = 0; i < 3; i++) U[3 * i + j] = 0;
        }
    }
    if (zero_col >= 0) {
        const int a = (zero_col + 1) % 3, b = (zero_col + 2) % 3;
        U[zero_col] = U[3 + a] * U[6 + b] - U[6 + a] * U[3 + b];
        U[3 + zero_col] = U[6 + a] * U[b] - U[a] * U[6 + b];
        U[6 + zero_col] = U[a] * U[3 + b] - U[3 + a] * U[b];
    }
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            Uc[i + 3 * j] = U[3 * i + j];
            Vc[i + 3 * j] = Vs[3 * i + j];
        }
}

}  // namespace Eigen

namespace open3d {
namespace pipelines {
namespace integration {
std::shared_ptr<geometry::TriangleMesh> ScalableTSDFVolume::ExtractTriangleMesh() {
    ss_stub_last_volume = std::make_shared<ScalableTSDFVolume>(*this);
    return std::make_shared<geometry::TriangleMesh>();
}
}  // namespace integration
}  // namespace pipelines
}  // namespace open3d

// ---- the entry points -------------------------------------------------------------
namespace {

struct Quiet {  // the reference prints progress lines from kokkosICP; keep test output clean
    std::streambuf *old;
    std::ostringstream sink;
    Quiet() : old(std::cout.rdbuf(sink.rdbuf())) {}
    ~Quiet() { std::cout.rdbuf(old); }
};

Kokkos::View<unsigned short **> depth_view(const uint16_t *d, int rows, int cols) {
    Kokkos::View<unsigned short **> v("depth", rows, cols);
    std::memcpy(v.data(), d, sizeof(uint16_t) * rows * cols);
    return v;
}

Eigen::Matrix4f mat4f(const float *rm) {
    Eigen::Matrix4f m;
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) m(i, j) = rm[4 * i + j];
    return m;
}

Eigen::Matrix4d mat4d(const double *rm) {
    Eigen::Matrix4d m;
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) m(i, j) = rm[4 * i + j];
    return m;
}

struct RefGrid {
    GPUVoxelGrid grid;
    Kokkos::Cuda space;
    RefGrid(unsigned c, float trunc, float vl, int resi, int resj) : grid(c, trunc, vl, resi, resj) {}
};

}  // namespace

extern "C" {

void *ssref_grid_new(unsigned capacity_voxels, float trunc, float vl, int resi, int resj) {
    return new RefGrid(capacity_voxels, trunc, vl, resi, resj);
}

void ssref_grid_free(void *h) { delete static_cast<RefGrid *>(h); }

void ssref_set_intrinsic(void *h, float fx, float fy, float cx, float cy) {
    RefGrid *r = static_cast<RefGrid *>(h);
    open3d::camera::PinholeCameraIntrinsic in(r->grid.resj, r->grid.resi, fx, fy, cx, cy);
    r->grid.setIntrinsic(r->space, in);
}

// deint = 0: integrate, 1: deIntegrate. rgb may be NULL when with_color = 0.
void ssref_fuse(void *h, const uint16_t *depth, const uint8_t *rgb, const float *extr, int with_color, int deint) {
    RefGrid *r = static_cast<RefGrid *>(h);
    const int rows = r->grid.resi, cols = r->grid.resj;
    Kokkos::View<unsigned char **[3]> rgbv("rgb", rows, cols);
    if (rgb) std::memcpy(rgbv.data(), rgb, (size_t)rows * cols * 3);
    auto dv = depth_view(depth, rows, cols);
    const Eigen::Matrix4f E = mat4f(extr);
    if (deint)
        r->grid.deIntegrate(r->space, rgbv, dv, E, with_color != 0);
    else
        r->grid.integrate(r->space, rgbv, dv, E, with_color != 0);
}

void ssref_raycast(void *h, const float *extr, float *pcd, float *color) {
    RefGrid *r = static_cast<RefGrid *>(h);
    r->grid.raycast(r->space, mat4f(extr));
    const size_t n = (size_t)r->grid.resi * r->grid.resj;
    for (size_t p = 0; p < n; p++) {
        const Kvec3f &a = r->grid.rayPcd.data()[p];
        const Kvec3f &c = r->grid.rayColorPcd.data()[p];
        pcd[3 * p] = a.x, pcd[3 * p + 1] = a.y, pcd[3 * p + 2] = a.z;
        if (color) color[3 * p] = c.x, color[3 * p + 1] = c.y, color[3 * p + 2] = c.z;
    }
}

void ssref_clean(void *h) {
    RefGrid *r = static_cast<RefGrid *>(h);
    r->grid.cleanMemory(r->space);
}

int ssref_count(void *h) { return (int)static_cast<RefGrid *>(h)->grid.voxelMap2.size(); }

// The live entries in slot order (callers sort by key): key, vbInd, pzero and
// the 512 voxels (sdf, w, r, g, b). Returns the number written.
int ssref_dump(void *h, int cap, uint64_t *keys, int32_t *coords, float *pzero, float *sdf, int16_t *w,
               float *rgb) {
    RefGrid *r = static_cast<RefGrid *>(h);
    const auto &m = r->grid.voxelMap2;
    int n = 0;
    for (uint32_t i = 0; i < m.capacity() && n < cap; i++) {
        if (!m.valid_at(i)) continue;
        const Voxelblock &vb = m.value_at(i);
        keys[n] = m.key_at(i);
        coords[3 * n] = vb.vbInd.x, coords[3 * n + 1] = vb.vbInd.y, coords[3 * n + 2] = vb.vbInd.z;
        if (pzero) pzero[3 * n] = vb.pzero.x, pzero[3 * n + 1] = vb.pzero.y, pzero[3 * n + 2] = vb.pzero.z;
        for (int v = 0; v < voxelPerBlock; v++) {
            if (sdf) sdf[(size_t)n * voxelPerBlock + v] = vb.voxel[v].sdf;
            if (w) w[(size_t)n * voxelPerBlock + v] = vb.voxel[v].w;
            if (rgb) {
                rgb[((size_t)n * 3 + 0) * voxelPerBlock + v] = vb.voxel[v].r;
                rgb[((size_t)n * 3 + 1) * voxelPerBlock + v] = vb.voxel[v].g;
                rgb[((size_t)n * 3 + 2) * voxelPerBlock + v] = vb.voxel[v].b;
            }
        }
        n++;
    }
    return n;
}

// Runs marchingCubesHost and returns the Open3D volume units it built: unit
// index [n][3] and each unit's tsdf and weight in Open3D's voxel order
// (IndexOf(x, y, z) = 64 x + 8 y + z). Returns the number of units.
int ssref_mc_units(void *h, int cap, int32_t *index, float *tsdf, float *weight) {
    RefGrid *r = static_cast<RefGrid *>(h);
    r->grid.marchingCubesHost();
    auto vol = open3d::pipelines::integration::ss_stub_last_volume;
    if (!vol) return -1;
    int n = 0;
    for (const auto &kv : vol->volume_units_) {
        if (n >= cap) break;
        const auto &u = kv.second;
        index[3 * n] = u.index_(0), index[3 * n + 1] = u.index_(1), index[3 * n + 2] = u.index_(2);
        for (int v = 0; v < 512; v++) {
            tsdf[(size_t)n * 512 + v] = u.volume_->voxels_[v].tsdf_;
            weight[(size_t)n * 512 + v] = u.volume_->voxels_[v].weight_;
        }
        n++;
    }
    return n;
}

void ssref_depth_to_pcd(const uint16_t *depth, int rows, int cols, float fx, float fy, float cx, float cy,
                        float *out) {
    Kokkos::Cuda space;
    open3d::camera::PinholeCameraIntrinsic in(cols, rows, fx, fy, cx, cy);
    auto v = CreatePcdFromDepthView(space, depth_view(depth, rows, cols), in);
    std::memcpy(out, v.data(), sizeof(float) * 3 * rows * cols);
}

void ssref_normals(const float *pcd, int rows, int cols, float *out) {
    Kokkos::Cuda space;
    Kokkos::View<Kvec3f **> p("pcd", rows, cols);
    std::memcpy(p.data(), pcd, sizeof(float) * 3 * rows * cols);
    auto n = CalculateNormalsFromPCDView(space, p);
    std::memcpy(out, n.data(), sizeof(float) * 3 * rows * cols);
}

// kokkosICP with g_intrinsic set to (fx, fy, cx, cy); T_out row-major.
void ssref_kokkos_icp(const uint16_t *d1, const uint16_t *d2, int rows, int cols, float fx, float fy, float cx,
                      float cy, const double *tx, const double *ty, int type, double *T_out, float *rmse_out) {
    Quiet q;
    Kokkos::Cuda space;
    g_intrinsic = open3d::camera::PinholeCameraIntrinsic(cols, rows, fx, fy, cx, cy);
    float rmse = 0;
    const Eigen::Matrix4d T = kokkosICP(space, depth_view(d1, rows, cols), depth_view(d2, rows, cols), mat4d(tx),
                                        mat4d(ty), type == 1 ? PointToPlane : PointToPoint, &rmse);
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) T_out[4 * i + j] = T(i, j);
    if (rmse_out) *rmse_out = rmse;
}

}  // extern "C"
