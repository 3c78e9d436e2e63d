// ss_ref_stub.h — the few Kokkos, Eigen, Open3D and OpenCV names that the
// reference's hot-path sources use, written here so that those sources compile
// UNCHANGED on the host (test infrastructure: builds oracle/_ref only).
//
// Force-included (-include) ahead of every reference translation unit in
// place of the reference's precompiled header (pchs/pch.h), which pulls in the
// real libraries (none of them is in this image). What each stand-in does:
//
//   Kokkos::View            reference-counted host array, row-major, with the
//                           extents of its data type (T**, T**[3], T[4][4],
//                           T*, T); views copy shallowly, as Kokkos views do;
//                           a new view reads as zero (see the constructor).
//                           create_mirror_view returns the view itself
//                           (Kokkos does so when the memory is host-accessible).
//   parallel_for            serial loops over the MDRange / Range, first index
//                           outermost: Kokkos::Cuda runs them unordered, so
//                           every result that does not depend on the order is
//                           the reference's; the order-dependent ones (list
//                           order, the last writer of an aliased key) take this
//                           order.
//   Kokkos::UnorderedMap    find / insert / valid_at / value_at / key_at /
//                           erase / capacity / size with Kokkos' observable
//                           semantics (default-constructed value on insert,
//                           invalid_index from a failed find). Its slot layout
//                           is Kokkos-internal and not reproduced (open
//                           addressing here); value_at(invalid_index) — which
//                           the reference's raycast reaches when it steps back
//                           into a missing block (GPUVoxelGrid.cpp:669-672) —
//                           returns an all-zero block.
//   atomics                 plain read-modify-write (serial execution).
//   Eigen::Matrix           fixed-size column-major matrices; products sum in
//                           index order k = 0..K-1 (Eigen's small fixed-size
//                           products may pair the terms differently: a
//                           last-bit difference in double at most).
//   Matrix4f::inverse()     cofactors in double, rounded to float; Eigen's own
//                           routine (vectorised, in float) is third-party code
//                           that is absent here, so the last bit of E^-1 may
//                           differ from the reference binary's.
//   Matrix4d::inverse()     Gauss-Jordan with partial pivoting in double.
//   JacobiSVD (3x3)         one-sided Jacobi in double (R = V U^T does not
//                           depend on the SVD's sign and order conventions for
//                           a full-rank H).
//   open3d, cv              data holders only (the intrinsic's matrix; the
//                           marching-cubes volume records the voxels the
//                           reference hands to Open3D; images, point clouds).
#pragma once

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <functional>
#include <iostream>
#include <list>
#include <memory>
#include <mutex>
#include <string>
#include <type_traits>
#include <unordered_map>
#include <vector>

#define KOKKOS_INLINE_FUNCTION inline
#define KOKKOS_FUNCTION
#define KOKKOS_LAMBDA [=]
#define EIGEN_MAKE_ALIGNED_OPERATOR_NEW

// ============================================================ Eigen ======
namespace Eigen {

enum { ComputeFullU = 4, ComputeFullV = 16, ComputeThinU = 8, ComputeThinV = 32 };
constexpr int Dynamic = -1;

template <typename S, int R, int C>
class Matrix;

template <typename S, int R, int C, int BR, int BC>
struct BlockRef {
    Matrix<S, R, C> &m;
    int r0, c0;
    BlockRef &operator=(const Matrix<S, BR, BC> &b) {
        for (int i = 0; i < BR; ++i)
            for (int j = 0; j < BC; ++j) m(r0 + i, c0 + j) = b(i, j);
        return *this;
    }
};

template <typename S, int R, int C>
class Matrix {
    static_assert(R > 0 && C > 0, "stub: fixed sizes only");
    S a_[R * C];  // column-major, as Eigen's default

public:
    Matrix() { std::fill(a_, a_ + R * C, S(0)); }
    Matrix(S x, S y) { static_assert(R * C == 2, "size"); a_[0] = x; a_[1] = y; }
    Matrix(S x, S y, S z) { static_assert(R * C == 3, "size"); a_[0] = x; a_[1] = y; a_[2] = z; }
    Matrix(S x, S y, S z, S w) { static_assert(R * C == 4, "size"); a_[0] = x; a_[1] = y; a_[2] = z; a_[3] = w; }

    static Matrix Zero() { return Matrix(); }
    static Matrix Identity() {
        Matrix m;
        for (int i = 0; i < std::min(R, C); ++i) m(i, i) = S(1);
        return m;
    }
    S &operator()(int i, int j) { return a_[i + R * j]; }
    const S &operator()(int i, int j) const { return a_[i + R * j]; }
    S &operator()(int i) { return a_[i]; }
    const S &operator()(int i) const { return a_[i]; }
    S &operator[](int i) { return a_[i]; }
    const S &operator[](int i) const { return a_[i]; }
    S *data() { return a_; }
    const S *data() const { return a_; }
    int rows() const { return R; }
    int cols() const { return C; }

    template <typename T>
    Matrix<T, R, C> cast() const {
        Matrix<T, R, C> o;
        for (int k = 0; k < R * C; ++k) o.data()[k] = static_cast<T>(a_[k]);
        return o;
    }
    Matrix<S, C, R> transpose() const {
        Matrix<S, C, R> o;
        for (int i = 0; i < R; ++i)
            for (int j = 0; j < C; ++j) o(j, i) = (*this)(i, j);
        return o;
    }
    S squaredNorm() const {
        S s = 0;
        for (int k = 0; k < R * C; ++k) s += a_[k] * a_[k];
        return s;
    }
    S norm() const { return std::sqrt(squaredNorm()); }
    template <int BR, int BC>
    BlockRef<S, R, C, BR, BC> block(int r0, int c0) { return {*this, r0, c0}; }

    Matrix operator+(const Matrix &b) const { Matrix o; for (int k = 0; k < R * C; ++k) o.a_[k] = a_[k] + b.a_[k]; return o; }
    Matrix operator-(const Matrix &b) const { Matrix o; for (int k = 0; k < R * C; ++k) o.a_[k] = a_[k] - b.a_[k]; return o; }
    Matrix &operator+=(const Matrix &b) { for (int k = 0; k < R * C; ++k) a_[k] += b.a_[k]; return *this; }
    Matrix &operator-=(const Matrix &b) { for (int k = 0; k < R * C; ++k) a_[k] -= b.a_[k]; return *this; }
    template <typename T, typename = std::enable_if_t<std::is_arithmetic<T>::value>>
    Matrix operator*(T s) const { Matrix o; for (int k = 0; k < R * C; ++k) o.a_[k] = a_[k] * S(s); return o; }
    template <typename T, typename = std::enable_if_t<std::is_arithmetic<T>::value>>
    Matrix operator/(T s) const { Matrix o; for (int k = 0; k < R * C; ++k) o.a_[k] = a_[k] / S(s); return o; }
    template <int K>
    Matrix<S, R, K> operator*(const Matrix<S, C, K> &b) const {
        Matrix<S, R, K> o;
        for (int i = 0; i < R; ++i)
            for (int j = 0; j < K; ++j) {
                S s = (*this)(i, 0) * b(0, j);
                for (int k = 1; k < C; ++k) s = s + (*this)(i, k) * b(k, j);
                o(i, j) = s;
            }
        return o;
    }
    Matrix inverse() const;
};

template <typename T, typename S, int R, int C, typename = std::enable_if_t<std::is_arithmetic<T>::value>>
Matrix<S, R, C> operator*(T s, const Matrix<S, R, C> &m) { return m * s; }

using Matrix3d = Matrix<double, 3, 3>;
using Matrix4d = Matrix<double, 4, 4>;
using Matrix3f = Matrix<float, 3, 3>;
using Matrix4f = Matrix<float, 4, 4>;
using Vector3d = Matrix<double, 3, 1>;
using Vector4d = Matrix<double, 4, 1>;
using Vector3f = Matrix<float, 3, 1>;
using Vector4f = Matrix<float, 4, 1>;
using Vector3i = Matrix<int, 3, 1>;
using Vector6d = Matrix<double, 6, 1>;
// MatrixXd appears only as JacobiSVD's template argument (kokkosICP.cpp:173).
struct MatrixXd {};

// 4x4 inverse of a float matrix: cofactors expanded in double, rounded to float.
void ss_stub_inverse4f(const float *colmajor_in, float *colmajor_out);
// 4x4 inverse of a double matrix: Gauss-Jordan with partial pivoting.
void ss_stub_inverse4d(const double *colmajor_in, double *colmajor_out);
// 3x3 SVD H = U diag(S) V^T in double (one-sided Jacobi), column-major.
void ss_stub_svd3(const double *H, double *U, double *S, double *V);

template <>
inline Matrix4f Matrix4f::inverse() const { Matrix4f o; ss_stub_inverse4f(a_, o.data()); return o; }
template <>
inline Matrix4d Matrix4d::inverse() const { Matrix4d o; ss_stub_inverse4d(a_, o.data()); return o; }

template <typename M>
class JacobiSVD {
    Matrix3d U_, V_;
    Vector3d S_;

public:
    JacobiSVD() = default;
    void compute(const Matrix3d &H, int) { ss_stub_svd3(H.data(), U_.data(), S_.data(), V_.data()); }
    const Matrix3d &matrixU() const { return U_; }
    const Matrix3d &matrixV() const { return V_; }
    const Vector3d &singularValues() const { return S_; }
};

}  // namespace Eigen

// ============================================================ Kokkos =====
namespace Kokkos {

class Cuda {};
class HostSpace {};
class LayoutLeft {};
class LayoutRight {};
template <unsigned N>
struct Rank { static constexpr unsigned value = N; };
template <typename T>
struct IndexType {};

inline void fence() {}

template <typename T>
T atomic_exchange(T *p, T v) { T o = *p; *p = v; return o; }
template <typename T>
T atomic_fetch_add(T *p, T v) { T o = *p; *p = o + v; return o; }

namespace stub {
// data type -> (value type, dynamic rank, static trailing extents)
template <typename T>
struct Dims {
    using value = T;
    static constexpr int dyn = 0;
    static constexpr int nstat = 0;
    static void stat(size_t *) {}
};
template <typename T>
struct Dims<T *> {
    using value = typename Dims<T>::value;
    static constexpr int dyn = Dims<T>::dyn + 1;
    static constexpr int nstat = Dims<T>::nstat;
    static void stat(size_t *e) { Dims<T>::stat(e); }
};
template <typename T, size_t N>
struct Dims<T[N]> {  // T**[3]: the array of the pointer type — 2 dynamic, then 1 static extent
    using value = typename Dims<T>::value;
    static constexpr int dyn = Dims<T>::dyn;
    static constexpr int nstat = Dims<T>::nstat + 1;
    static void stat(size_t *e) { e[0] = N; Dims<T>::stat(e + 1); }
};
}  // namespace stub

template <typename DataType, typename... Props>
class View {
    using D = stub::Dims<DataType>;

public:
    using value_type = typename D::value;
    static constexpr int rank = D::dyn + D::nstat;

    View() { std::fill(ext_, ext_ + 8, size_t(0)); }
    template <typename... N>
    explicit View(const std::string &, N... n) {
        static_assert(sizeof...(N) == D::dyn, "stub View: one size per dynamic extent");
        std::fill(ext_, ext_ + 8, size_t(1));
        size_t dyn[] = {size_t(n)..., 0};
        for (int k = 0; k < D::dyn; ++k) ext_[k] = dyn[k];
        D::stat(ext_ + D::dyn);
        size_t total = 1;
        for (int k = 0; k < rank; ++k) total *= ext_[k];
        // Fresh device allocations read as zero; Kokkos runs a class type's
        // default constructor over them, which for Kvec3f (kokkosFunctions.h:149)
        // writes nothing, so the bytes are zeroed after construction here.
        value_type *p = new value_type[total];
        std::memset(static_cast<void *>(p), 0, sizeof(value_type) * total);
        data_ = std::shared_ptr<value_type>(p, std::default_delete<value_type[]>());
    }
    size_t extent(int k) const { return k < rank ? ext_[k] : 1; }
    int extent_int(int k) const { return int(extent(k)); }
    size_t size() const { size_t t = 1; for (int k = 0; k < rank; ++k) t *= ext_[k]; return t; }
    value_type *data() const { return data_.get(); }

    value_type &operator()() const { return data_.get()[0]; }
    value_type &operator()(size_t i) const { return data_.get()[i]; }
    value_type &operator()(size_t i, size_t j) const { return data_.get()[i * ext_[1] + j]; }
    value_type &operator()(size_t i, size_t j, size_t k) const {
        return data_.get()[(i * ext_[1] + j) * ext_[2] + k];
    }

    template <typename O, typename... P>
    friend class View;
    template <typename O, typename... P>
    View(const View<O, P...> &o) : data_(o.data_) { std::copy(o.ext_, o.ext_ + 8, ext_); }

private:
    std::shared_ptr<value_type> data_;
    size_t ext_[8];
};

template <typename V>
V create_mirror_view(const V &v) { return v; }

template <typename A, typename B>
void deep_copy(const A &dst, const B &src) {
    if (dst.data() != src.data()) std::copy(src.data(), src.data() + src.size(), dst.data());
}

namespace stub {
template <typename... A>
struct TagOf { using type = void; };
template <typename T, typename... A>
struct TagOf<T, A...> {
    using rest = typename TagOf<A...>::type;
    static constexpr bool plain = std::is_same<T, Cuda>::value || std::is_same<T, HostSpace>::value;
    using type = std::conditional_t<plain, rest, T>;
};
template <unsigned N>
struct TagOf<Rank<N>> { using type = void; };
template <unsigned N, typename... A>
struct TagOf<Rank<N>, A...> { using type = typename TagOf<A...>::type; };
template <typename I, typename... A>
struct TagOf<IndexType<I>, A...> { using type = typename TagOf<A...>::type; };
template <typename I>
struct TagOf<IndexType<I>> { using type = void; };

template <typename... A>
struct RankOf { static constexpr unsigned value = 0; };
template <typename T, typename... A>
struct RankOf<T, A...> { static constexpr unsigned value = RankOf<A...>::value; };
template <unsigned N, typename... A>
struct RankOf<Rank<N>, A...> { static constexpr unsigned value = N; };
}  // namespace stub

template <typename... A>
struct MDRangePolicy {
    using tag = typename stub::TagOf<A...>::type;
    static constexpr unsigned R = stub::RankOf<A...>::value;
    long long lo[8], hi[8];
    template <typename Sp, typename L, typename U>
    MDRangePolicy(Sp &, const L (&l)[R], const U (&u)[R]) {
        for (unsigned k = 0; k < R; ++k) { lo[k] = (long long)l[k]; hi[k] = (long long)u[k]; }
    }
    template <typename L, typename U>
    MDRangePolicy(const L (&l)[R], const U (&u)[R]) {
        for (unsigned k = 0; k < R; ++k) { lo[k] = (long long)l[k]; hi[k] = (long long)u[k]; }
    }
};

template <typename... A>
struct RangePolicy {
    using tag = typename stub::TagOf<A...>::type;
    long long lo, hi;
    template <typename Sp, typename L, typename U>
    RangePolicy(Sp &, L l, U u) : lo((long long)l), hi((long long)u) {}
    template <typename L, typename U>
    RangePolicy(L l, U u) : lo((long long)l), hi((long long)u) {}
};

namespace stub {
template <typename Tag, typename F, typename... I>
inline void call(const F &f, I... i) {
    if constexpr (std::is_void<Tag>::value) f(int(i)...);
    else f(Tag(), int(i)...);
}
}  // namespace stub

template <typename F, typename... A>
void parallel_for(const std::string &, const MDRangePolicy<A...> &p, const F &f) {
    using P = MDRangePolicy<A...>;
    using T = typename P::tag;
    if constexpr (P::R == 2) {
        for (long long i = p.lo[0]; i < p.hi[0]; ++i)
            for (long long j = p.lo[1]; j < p.hi[1]; ++j) stub::call<T>(f, i, j);
    } else if constexpr (P::R == 3) {
        for (long long i = p.lo[0]; i < p.hi[0]; ++i)
            for (long long j = p.lo[1]; j < p.hi[1]; ++j)
                for (long long k = p.lo[2]; k < p.hi[2]; ++k) stub::call<T>(f, i, j, k);
    } else {
        static_assert(P::R == 4, "stub: MDRange ranks 2-4");
        for (long long i = p.lo[0]; i < p.hi[0]; ++i)
            for (long long j = p.lo[1]; j < p.hi[1]; ++j)
                for (long long k = p.lo[2]; k < p.hi[2]; ++k)
                    for (long long l = p.lo[3]; l < p.hi[3]; ++l) stub::call<T>(f, i, j, k, l);
    }
}

template <typename F, typename... A>
void parallel_for(const std::string &, const RangePolicy<A...> &p, const F &f) {
    for (long long i = p.lo; i < p.hi; ++i) stub::call<typename RangePolicy<A...>::tag>(f, i);
}

struct UnorderedMapInsertResult {
    uint32_t idx;
    int state;  // 0 failed, 1 success, 2 existing
    uint32_t index() const { return idx; }
    bool success() const { return state == 1; }
    bool existing() const { return state == 2; }
    bool failed() const { return state == 0; }
};

template <typename K, typename V, typename Dev = Cuda>
class UnorderedMap {
    struct Store {
        std::vector<K> keys;
        std::vector<uint8_t> state;  // 0 empty, 1 live, 2 erased (probe chains pass it)
        std::vector<std::unique_ptr<V>> vals;
        uint32_t size = 0;
    };
    std::shared_ptr<Store> s_;

    static uint64_t mix(uint64_t k) {  // splitmix64 finaliser: spreads the prime-hash keys
        k ^= k >> 30; k *= 0xbf58476d1ce4e5b9ull;
        k ^= k >> 27; k *= 0x94d049bb133111ebull;
        return k ^ (k >> 31);
    }

public:
    static constexpr uint32_t invalid_index = ~0u;

    UnorderedMap() : UnorderedMap(0) {}
    explicit UnorderedMap(uint32_t capacity_hint) : s_(std::make_shared<Store>()) {
        uint32_t c = std::max<uint32_t>(128, (capacity_hint + 127) / 128 * 128);
        s_->keys.assign(c, K());
        s_->state.assign(c, 0);
        s_->vals.resize(c);
    }
    template <typename D2>
    friend class UnorderedMapCopy;
    uint32_t capacity() const { return uint32_t(s_->keys.size()); }
    uint32_t size() const { return s_->size; }
    bool valid_at(uint32_t i) const { return i < capacity() && s_->state[i] == 1; }
    V &value_at(uint32_t i) const {
        static V empty{};
        if (!valid_at(i)) { empty = V{}; return empty; }
        return *s_->vals[i];
    }
    K key_at(uint32_t i) const { return s_->keys[i]; }
    uint32_t find(K k) const {
        const uint32_t c = capacity();
        uint32_t h = uint32_t(mix(uint64_t(k)) % c);
        for (uint32_t n = 0; n < c; ++n, h = (h + 1) % c) {
            if (s_->state[h] == 0) return invalid_index;
            if (s_->state[h] == 1 && s_->keys[h] == k) return h;
        }
        return invalid_index;
    }
    UnorderedMapInsertResult insert(K k) const {
        uint32_t f = find(k);
        if (f != invalid_index) return {f, 2};
        const uint32_t c = capacity();
        uint32_t h = uint32_t(mix(uint64_t(k)) % c);
        for (uint32_t n = 0; n < c; ++n, h = (h + 1) % c) {
            if (s_->state[h] != 1) {
                s_->keys[h] = k;
                s_->state[h] = 1;
                s_->vals[h].reset(new V{});
                ++s_->size;
                return {h, 1};
            }
        }
        return {invalid_index, 0};
    }
    bool erase(K k) const {
        uint32_t i = find(k);
        if (i == invalid_index) return false;
        s_->state[i] = 2;
        s_->vals[i].reset();
        --s_->size;
        return true;
    }
    void begin_erase() const {}
    void end_erase() const {}

    template <typename D2>
    void copy_from(const UnorderedMap<K, V, D2> &o) {
        s_ = std::make_shared<Store>();
        const uint32_t c = o.capacity();
        s_->keys.assign(c, K());
        s_->state.assign(c, 0);
        s_->vals.resize(c);
        for (uint32_t i = 0; i < c; ++i)
            if (o.valid_at(i)) {
                s_->keys[i] = o.key_at(i);
                s_->state[i] = 1;
                s_->vals[i].reset(new V(o.value_at(i)));
                ++s_->size;
            }
    }
};

template <typename K, typename V, typename D1, typename D2>
void deep_copy(UnorderedMap<K, V, D1> &dst, const UnorderedMap<K, V, D2> &src) { dst.copy_from(src); }

}  // namespace Kokkos

// ============================================================ Open3D =====
namespace open3d {
namespace geometry {
struct Geometry { virtual ~Geometry() = default; };
struct PointCloud : Geometry {
    std::vector<Eigen::Vector3d> points_, colors_, normals_;
    bool HasNormals() const { return !normals_.empty() && normals_.size() == points_.size(); }
};
struct LineSet : Geometry {};
struct TriangleMesh : Geometry {
    std::vector<Eigen::Vector3d> vertices_, vertex_normals_;
    TriangleMesh &ComputeVertexNormals(bool = true) { return *this; }
};
struct Image : Geometry {
    int width_ = 0, height_ = 0, num_of_channels_ = 0, bytes_per_channel_ = 0;
    std::vector<uint8_t> data_;
    Image &Prepare(int w, int h, int ch, int bpc) {
        width_ = w; height_ = h; num_of_channels_ = ch; bytes_per_channel_ = bpc;
        data_.assign(size_t(w) * h * ch * bpc, 0);
        return *this;
    }
    template <typename T>
    T *PointerAt(int u, int v) { return reinterpret_cast<T *>(data_.data()) + (size_t(v) * width_ + u); }
    template <typename T>
    T *PointerAt(int u, int v, int ch) {
        return reinterpret_cast<T *>(data_.data()) + ((size_t(v) * width_ + u) * num_of_channels_ + ch);
    }
};
}  // namespace geometry

namespace camera {
struct PinholeCameraIntrinsic {
    int width_ = 0, height_ = 0;
    Eigen::Matrix3d intrinsic_matrix_ = Eigen::Matrix3d::Zero();
    PinholeCameraIntrinsic() = default;
    PinholeCameraIntrinsic(int w, int h, double fx, double fy, double cx, double cy) : width_(w), height_(h) {
        intrinsic_matrix_(0, 0) = fx;
        intrinsic_matrix_(1, 1) = fy;
        intrinsic_matrix_(0, 2) = cx;
        intrinsic_matrix_(1, 2) = cy;
        intrinsic_matrix_(2, 2) = 1.0;
    }
};
}  // namespace camera

namespace pipelines {
namespace integration {
enum class TSDFVolumeColorType { NoColor = 0, RGB8 = 1, Gray32 = 2 };
struct TSDFVoxel {
    Eigen::Vector3d color_;
    float tsdf_ = 0;
    float weight_ = 0;
};
// One Open3D volume unit: its voxels in Open3D's own index order
// (IndexOf(x, y, z) = x * res^2 + y * res + z).
struct UniformTSDFVolume {
    double voxel_length_;
    int resolution_;
    Eigen::Vector3d origin_;
    std::vector<TSDFVoxel> voxels_;
    UniformTSDFVolume(double length, int resolution, double, TSDFVolumeColorType, const Eigen::Vector3d &origin)
        : voxel_length_(length / resolution), resolution_(resolution), origin_(origin),
          voxels_(size_t(resolution) * resolution * resolution) {}
};
struct Vector3iHash {
    size_t operator()(const Eigen::Vector3i &v) const {
        return (size_t(uint32_t(v(0))) * 73856093u) ^ (size_t(uint32_t(v(1))) * 19349669u) ^
               (size_t(uint32_t(v(2))) * 83492791u);
    }
};
struct Vector3iEq {
    bool operator()(const Eigen::Vector3i &a, const Eigen::Vector3i &b) const {
        return a(0) == b(0) && a(1) == b(1) && a(2) == b(2);
    }
};
// Records the units the reference hands over; the mesh itself is Open3D's
// marching cubes, absent here (ExtractTriangleMesh returns an empty mesh).
struct ScalableTSDFVolume {
    struct VolumeUnit {
        std::shared_ptr<UniformTSDFVolume> volume_;
        Eigen::Vector3i index_;
    };
    double voxel_length_, sdf_trunc_;
    int volume_unit_resolution_;
    std::unordered_map<Eigen::Vector3i, VolumeUnit, Vector3iHash, Vector3iEq> volume_units_;
    ScalableTSDFVolume(double vl, double trunc, TSDFVolumeColorType, int res = 16, int = 4)
        : voxel_length_(vl), sdf_trunc_(trunc), volume_unit_resolution_(res) {}
    std::shared_ptr<geometry::TriangleMesh> ExtractTriangleMesh();
};
// The last volume whose mesh was extracted (for tests of marchingCubesHost's
// voxel copy); ExtractTriangleMesh records it and returns an empty mesh.
extern std::shared_ptr<ScalableTSDFVolume> ss_stub_last_volume;
}  // namespace integration
}  // namespace pipelines

namespace visualization {
inline bool DrawGeometries(const std::vector<std::shared_ptr<const geometry::Geometry>> &) { return true; }
}  // namespace visualization
}  // namespace open3d

// ============================================================ OpenCV =====
#define CV_8UC3 16
#define CV_16U 2
namespace cv {
class Mat {
    std::shared_ptr<std::vector<uint8_t>> buf_;
    int type_ = 0;

public:
    int rows = 0, cols = 0;
    Mat() = default;
    Mat(int r, int c, int type) : buf_(std::make_shared<std::vector<uint8_t>>()), type_(type), rows(r), cols(c) {
        buf_->assign(size_t(r) * c * elem(), 0);
    }
    size_t elem() const { return type_ == CV_8UC3 ? 3 : 2; }
    int channels() const { return type_ == CV_8UC3 ? 3 : 1; }
    template <typename T>
    T *ptr(int r) { return reinterpret_cast<T *>(buf_->data() + size_t(r) * cols * elem()); }
};
}  // namespace cv
