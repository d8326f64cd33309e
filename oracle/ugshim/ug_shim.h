/*
 * ug_shim.h -- a minimal stand-in for the parts of UG4's core library
 * (ugcore) that the reference's FV1 Navier-Stokes sources include, so that
 * the UNMODIFIED reference files
 *     navier_stokes_base.cpp, incompressible/incompressible_navier_stokes_base.cpp,
 *     incompressible/fv1/navier_stokes_fv1.cpp, incompressible/fv1/stabilization.cpp,
 *     upwind.cpp, upwind_interface.cpp
 * compile on the host and can be run element by element (oracle/ref_driver.cpp).
 *
 * TEST INFRASTRUCTURE: used only to build oracle/_ref/, the reference-backed
 * checker of the oracle. Nothing of the product links it.
 *
 * ugcore itself is not part of the reference tree (it is a separate project,
 * installed through ughub; no version is pinned there). What this file provides:
 *  - plumbing with the ugcore names and signatures the sources call
 *    (SmartPtr, MathVector, LocalVector/LocalMatrix, IElemDisc, DataImport,
 *    GeomProvider, Provider, ...): no numerics;
 *  - the numerics ugcore contributes to this path, restated from their
 *    published definitions: the FV1 box-method geometry (FV1Geometry::update),
 *    the element-side ray intersection used by the skewed upwinds, the P1
 *    Lagrange shape functions, a small dense inverse (GetInverse) and the
 *    2D SCVF ray intersection of the regular upwind.
 * Element types that the path does not run here (edges, pyramids, prisms,
 * manifold elements, Crouzeix-Raviart geometries) compile but throw if updated.
 */
#ifndef NSFV1_UG_SHIM_H
#define NSFV1_UG_SHIM_H

#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstddef>
#include <cstring>
#include <limits>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

namespace ug {

typedef double number;

/* ---- errors and logging (ugcore: common/error.h, common/log.h) ----------- */
struct UGError : public std::runtime_error {
    explicit UGError(const std::string& s) : std::runtime_error(s) {}
};

#define UG_THROW(msg)                                \
    do {                                             \
        std::stringstream ug_ss_;                    \
        ug_ss_ << msg;                               \
        throw ::ug::UGError(ug_ss_.str());           \
    } while (0)
#define UG_CATCH_THROW(msg)                                          \
    catch (::ug::UGError & ug_e_) {                                  \
        std::stringstream ug_ss_;                                    \
        ug_ss_ << msg << " (" << ug_e_.what() << ")";               \
        throw ::ug::UGError(ug_ss_.str());                           \
    }
// the reference enables its bounds asserts (upwind_interface.h:38, stabilization.h:38)
#define UG_ASSERT(cond, msg) \
    do {                     \
        if (!(cond)) UG_THROW("assertion failed: " << #cond << ": " << msg); \
    } while (0)
#define UG_LOG(msg) do {} while (0)
#define UG_WARNING(msg) do {} while (0)
#define PROFILE_FUNC()
#define PROFILE_BEGIN(x)
#define PROFILE_END()

template <int N> struct Int2Type { enum { value = N }; };

inline std::string TrimString(const std::string& s) {
    const size_t a = s.find_first_not_of(" \t\n\r"), z = s.find_last_not_of(" \t\n\r");
    return a == std::string::npos ? std::string() : s.substr(a, z - a + 1);
}

/* ---- reference-counted pointers (ugcore: common/util/smart_pointer.h) ----- */
struct NullSmartPtr {};
static const NullSmartPtr SPNULL = NullSmartPtr();

template <class T> class ConstSmartPtr;

template <class T>
class SmartPtr {
  public:
    SmartPtr() {}
    SmartPtr(T* p) : m_p(p) {}
    SmartPtr(NullSmartPtr) {}
    template <class U> SmartPtr(const SmartPtr<U>& o) : m_p(o.shared()) {}
    SmartPtr& operator=(NullSmartPtr) { m_p.reset(); return *this; }
    T* operator->() const { return m_p.get(); }
    T& operator*() const { return *m_p; }
    T* get() const { return m_p.get(); }
    bool valid() const { return (bool)m_p; }
    bool invalid() const { return !m_p; }
    const std::shared_ptr<T>& shared() const { return m_p; }
    template <class U> bool operator==(const SmartPtr<U>& o) const { return m_p.get() == o.get(); }
    template <class U> bool operator!=(const SmartPtr<U>& o) const { return m_p.get() != o.get(); }
    template <class U> bool operator==(const ConstSmartPtr<U>& o) const { return m_p.get() == o.get(); }
    template <class U> bool operator!=(const ConstSmartPtr<U>& o) const { return m_p.get() != o.get(); }

  private:
    std::shared_ptr<T> m_p;
};

template <class T>
class ConstSmartPtr {
  public:
    ConstSmartPtr() {}
    ConstSmartPtr(const T* p) : m_p(p) {}
    ConstSmartPtr(NullSmartPtr) {}
    template <class U> ConstSmartPtr(const SmartPtr<U>& o) : m_p(o.shared()) {}
    template <class U> ConstSmartPtr(const ConstSmartPtr<U>& o) : m_p(o.shared()) {}
    ConstSmartPtr& operator=(NullSmartPtr) { m_p.reset(); return *this; }
    const T* operator->() const { return m_p.get(); }
    const T& operator*() const { return *m_p; }
    const T* get() const { return m_p.get(); }
    bool valid() const { return (bool)m_p; }
    bool invalid() const { return !m_p; }
    const std::shared_ptr<const T>& shared() const { return m_p; }
    template <class U> bool operator==(const SmartPtr<U>& o) const { return m_p.get() == o.get(); }
    template <class U> bool operator!=(const SmartPtr<U>& o) const { return m_p.get() != o.get(); }
    template <class U> bool operator==(const ConstSmartPtr<U>& o) const { return m_p.get() == o.get(); }
    template <class U> bool operator!=(const ConstSmartPtr<U>& o) const { return m_p.get() != o.get(); }

  private:
    std::shared_ptr<const T> m_p;
};

template <class T> SmartPtr<T> make_sp(T* p) { return SmartPtr<T>(p); }

/* ---- small vectors and matrices (ugcore: common/math/math_vector_matrix) -- */
template <int N, typename T = number>
class MathVector {
  public:
    static const int Size = N;
    MathVector() { for (int i = 0; i < N; ++i) m_v[i] = T(0); }
    explicit MathVector(const T& s) { for (int i = 0; i < N; ++i) m_v[i] = s; }
    MathVector& operator=(const T& s) { for (int i = 0; i < N; ++i) m_v[i] = s; return *this; }
    T& operator[](size_t i) { return m_v[i]; }
    const T& operator[](size_t i) const { return m_v[i]; }
    T& coord(size_t i) { return m_v[i]; }
    const T& coord(size_t i) const { return m_v[i]; }
    static size_t size() { return N; }
    MathVector& operator+=(const MathVector& o) { for (int i = 0; i < N; ++i) m_v[i] += o.m_v[i]; return *this; }
    MathVector& operator-=(const MathVector& o) { for (int i = 0; i < N; ++i) m_v[i] -= o.m_v[i]; return *this; }
    MathVector& operator*=(const T& s) { for (int i = 0; i < N; ++i) m_v[i] *= s; return *this; }

  private:
    T m_v[N > 0 ? N : 1];
};

template <int N, int M, typename T = number>
class MathMatrix {
  public:
    MathMatrix() { for (int i = 0; i < N; ++i) for (int j = 0; j < M; ++j) m_a[i][j] = T(0); }
    MathMatrix& operator=(const T& s) { for (int i = 0; i < N; ++i) for (int j = 0; j < M; ++j) m_a[i][j] = s; return *this; }
    MathMatrix& operator*=(const T& s) { for (int i = 0; i < N; ++i) for (int j = 0; j < M; ++j) m_a[i][j] *= s; return *this; }
    T& operator()(size_t i, size_t j) { return m_a[i][j]; }
    const T& operator()(size_t i, size_t j) const { return m_a[i][j]; }
    T* operator[](size_t i) { return m_a[i]; }
    const T* operator[](size_t i) const { return m_a[i]; }
    static size_t num_rows() { return N; }
    static size_t num_cols() { return M; }

  private:
    T m_a[N > 0 ? N : 1][M > 0 ? M : 1];
};

template <int N> inline void VecSet(MathVector<N>& v, number s) { for (int i = 0; i < N; ++i) v[i] = s; }
template <int N> inline void VecScale(MathVector<N>& o, const MathVector<N>& v, number s) { for (int i = 0; i < N; ++i) o[i] = s * v[i]; }
template <int N> inline void VecScaleAppend(MathVector<N>& o, number s, const MathVector<N>& v) { for (int i = 0; i < N; ++i) o[i] += s * v[i]; }
template <int N> inline void VecScaleAppend(MathVector<N>& o, number s1, const MathVector<N>& v1, number s2, const MathVector<N>& v2) {
    for (int i = 0; i < N; ++i) o[i] += s1 * v1[i] + s2 * v2[i];
}
template <int N> inline void VecScaleAdd(MathVector<N>& o, number s1, const MathVector<N>& v1, number s2, const MathVector<N>& v2) {
    for (int i = 0; i < N; ++i) o[i] = s1 * v1[i] + s2 * v2[i];
}
template <int N> inline void VecAdd(MathVector<N>& o, const MathVector<N>& a, const MathVector<N>& b) { for (int i = 0; i < N; ++i) o[i] = a[i] + b[i]; }
template <int N> inline void VecSubtract(MathVector<N>& o, const MathVector<N>& a, const MathVector<N>& b) { for (int i = 0; i < N; ++i) o[i] = a[i] - b[i]; }
template <int N> inline void VecAppend(MathVector<N>& o, const MathVector<N>& a) { for (int i = 0; i < N; ++i) o[i] += a[i]; }
template <int N> inline number VecDot(const MathVector<N>& a, const MathVector<N>& b) { number s = 0; for (int i = 0; i < N; ++i) s += a[i] * b[i]; return s; }
template <int N> inline number VecProd(const MathVector<N>& a, const MathVector<N>& b) { return VecDot(a, b); }
template <int N> inline number VecTwoNormSq(const MathVector<N>& a) { return VecDot(a, a); }
template <int N> inline number VecTwoNorm(const MathVector<N>& a) { return std::sqrt(VecTwoNormSq(a)); }
template <int N> inline number VecLength(const MathVector<N>& a) { return VecTwoNorm(a); }
template <int N> inline number VecDistanceSq(const MathVector<N>& a, const MathVector<N>& b) {
    number s = 0;
    for (int i = 0; i < N; ++i) { const number x = a[i] - b[i]; s += x * x; }
    return s;
}
template <int N> inline number VecDistance(const MathVector<N>& a, const MathVector<N>& b) { return std::sqrt(VecDistanceSq(a, b)); }
template <int N> inline void VecNormalize(MathVector<N>& o, const MathVector<N>& a) { const number l = VecTwoNorm(a); for (int i = 0; i < N; ++i) o[i] = a[i] / l; }
inline void VecCross(MathVector<3>& o, const MathVector<3>& a, const MathVector<3>& b) {
    MathVector<3> c;
    c[0] = a[1] * b[2] - a[2] * b[1];
    c[1] = a[2] * b[0] - a[0] * b[2];
    c[2] = a[0] * b[1] - a[1] * b[0];
    o = c;
}
template <int N, int M> inline void MatVecMult(MathVector<N>& o, const MathMatrix<N, M>& A, const MathVector<M>& v) {
    for (int i = 0; i < N; ++i) { number s = 0; for (int j = 0; j < M; ++j) s += A(i, j) * v[j]; o[i] = s; }
}
template <int N, int M> inline void MatVecMultAppend(MathVector<N>& o, const MathMatrix<N, M>& A, const MathVector<M>& v) {
    for (int i = 0; i < N; ++i) { number s = 0; for (int j = 0; j < M; ++j) s += A(i, j) * v[j]; o[i] += s; }
}
template <int N, int M> inline void MatVecMultAdd(MathVector<N>& o, number a, const MathVector<N>& w, number b, const MathMatrix<N, M>& A,
                                                  const MathVector<M>& v) {
    for (int i = 0; i < N; ++i) { number s = 0; for (int j = 0; j < M; ++j) s += A(i, j) * v[j]; o[i] = a * w[i] + b * s; }
}
template <int N, int M> inline void TransposedMatVecMult(MathVector<M>& o, const MathMatrix<N, M>& A, const MathVector<N>& v) {
    for (int j = 0; j < M; ++j) { number s = 0; for (int i = 0; i < N; ++i) s += A(i, j) * v[i]; o[j] = s; }
}
// the diagonal entries set to s, the others kept
template <int N> inline void MatDiagSet(MathMatrix<N, N>& A, number s) { for (int i = 0; i < N; ++i) A(i, i) = s; }
template <int N, int M> inline void TransposedMatVecMultAdd(MathVector<M>& o, const MathMatrix<N, M>& A, const MathVector<N>& v) {
    for (int j = 0; j < M; ++j) { number s = 0; for (int i = 0; i < N; ++i) s += A(i, j) * v[i]; o[j] += s; }
}
template <int N, int M> inline void MatSet(MathMatrix<N, M>& A, number s) { A = s; }
template <int N, int M> inline void Transpose(MathMatrix<M, N>& o, const MathMatrix<N, M>& A) {
    for (int i = 0; i < N; ++i) for (int j = 0; j < M; ++j) o(j, i) = A(i, j);
}

/* ---- dense fixed-size algebra (ugcore: lib_algebra/small_algebra) --------- */
template <typename T, size_t N> struct FixedArray1 { T v[N]; };
template <typename T, size_t N, size_t M> struct FixedArray2 { T a[N][M]; };

template <class TStorage> class DenseVector;
template <typename T, size_t N>
class DenseVector<FixedArray1<T, N> > {
  public:
    DenseVector() { for (size_t i = 0; i < N; ++i) m.v[i] = T(0); }
    DenseVector& operator=(const T& s) { for (size_t i = 0; i < N; ++i) m.v[i] = s; return *this; }
    T& operator[](size_t i) { return m.v[i]; }
    const T& operator[](size_t i) const { return m.v[i]; }
    T& operator()(size_t i) { return m.v[i]; }
    const T& operator()(size_t i) const { return m.v[i]; }
    static size_t size() { return N; }

  private:
    FixedArray1<T, N> m;
};

template <class TStorage> class DenseMatrix;
template <typename T, size_t N, size_t M>
class DenseMatrix<FixedArray2<T, N, M> > {
  public:
    DenseMatrix() { *this = T(0); }
    DenseMatrix& operator=(const T& s) { for (size_t i = 0; i < N; ++i) for (size_t j = 0; j < M; ++j) m.a[i][j] = s; return *this; }
    T& operator()(size_t i, size_t j) { return m.a[i][j]; }
    const T& operator()(size_t i, size_t j) const { return m.a[i][j]; }
    static size_t num_rows() { return N; }
    static size_t num_cols() { return M; }

  private:
    FixedArray2<T, N, M> m;
};

template <class T> struct block_traits;
template <typename T, size_t N, size_t M> struct block_traits<DenseMatrix<FixedArray2<T, N, M> > > {
    typedef DenseMatrix<FixedArray2<T, N, M> > inverse_type;
};

// inverse by Gauss-Jordan elimination with partial pivoting; false if singular
template <typename T, size_t N>
bool GetInverse(DenseMatrix<FixedArray2<T, N, N> >& inv, const DenseMatrix<FixedArray2<T, N, N> >& A) {
    T w[N][2 * N];
    for (size_t i = 0; i < N; ++i)
        for (size_t j = 0; j < N; ++j) { w[i][j] = A(i, j); w[i][N + j] = (i == j) ? T(1) : T(0); }
    for (size_t c = 0; c < N; ++c) {
        size_t p = c;
        for (size_t q = c + 1; q < N; ++q) if (std::fabs(w[q][c]) > std::fabs(w[p][c])) p = q;
        if (w[p][c] == T(0)) return false;
        if (p != c) for (size_t j = 0; j < 2 * N; ++j) std::swap(w[p][j], w[c][j]);
        const T piv = T(1) / w[c][c];
        for (size_t j = 0; j < 2 * N; ++j) w[c][j] *= piv;
        for (size_t q = 0; q < N; ++q) {
            if (q == c) continue;
            const T f = w[q][c];
            if (f == T(0)) continue;
            for (size_t j = 0; j < 2 * N; ++j) w[q][j] -= f * w[c][j];
        }
    }
    for (size_t i = 0; i < N; ++i) for (size_t j = 0; j < N; ++j) inv(i, j) = w[i][N + j];
    return true;
}

// y = alpha * A x
template <typename T, size_t N, size_t M>
void MatMult(DenseVector<FixedArray1<T, N> >& y, const T& alpha, const DenseMatrix<FixedArray2<T, N, M> >& A,
             const DenseVector<FixedArray1<T, M> >& x) {
    for (size_t i = 0; i < N; ++i) {
        T s = 0;
        for (size_t j = 0; j < M; ++j) s += A(i, j) * x[j];
        y[i] = alpha * s;
    }
}
// y = a x + b z
template <typename T, size_t N>
void VecScaleAdd(DenseVector<FixedArray1<T, N> >& y, const T& a, const DenseVector<FixedArray1<T, N> >& x, const T& b,
                 const DenseVector<FixedArray1<T, N> >& z) {
    for (size_t i = 0; i < N; ++i) y[i] = a * x[i] + b * z[i];
}

/* ---- grid objects and reference elements (ugcore: lib_grid, lib_disc/reference_element) */
enum ReferenceObjectID {
    ROID_UNKNOWN = -1, ROID_VERTEX = 0, ROID_EDGE, ROID_TRIANGLE, ROID_QUADRILATERAL, ROID_TETRAHEDRON,
    ROID_PYRAMID, ROID_PRISM, ROID_OCTAHEDRON, ROID_HEXAHEDRON, NUM_REFERENCE_OBJECTS
};

class GridObject {};
// Subsets: index 0 is the element subset, 1 the boundary subset a driver marks
// (the element-local sides that lie on it are set per element with
// shim_boundary_sides() before the geometry update).
class ISubsetHandler {
  public:
    int num_subsets() const { return 2; }
};
class SubsetGroup {
  public:
    size_t size() const { return m_si.size(); }
    int operator[](size_t i) const { return m_si[i]; }
    void add(int si) { m_si.push_back(si); }

  private:
    std::vector<int> m_si;
};
inline unsigned& shim_boundary_sides() {
    static thread_local unsigned mask = 0;
    return mask;
}

// Reference-element tables in ugcore numbering: corners, edges (= the SCVFs of
// the FV1 dual mesh, oriented from corner 0 to corner 1) and sides.
struct RefTables {
    int dim, numCorners, numEdges, numSides;
    number co[8][3];
    int edge[12][2];
    int sideNco[6];
    int side[6][4];
};

inline RefTables make_ref_tables(ReferenceObjectID roid) {
    RefTables t;
    std::memset(&t, 0, sizeof(t));
    auto corners = [&](std::initializer_list<std::initializer_list<number> > c) {
        int i = 0;
        for (auto& p : c) { int d = 0; for (number x : p) t.co[i][d++] = x; ++i; }
        t.numCorners = i;
    };
    auto edges = [&](std::initializer_list<std::initializer_list<int> > e) {
        int i = 0;
        for (auto& p : e) { t.edge[i][0] = *p.begin(); t.edge[i][1] = *(p.begin() + 1); ++i; }
        t.numEdges = i;
    };
    auto sides = [&](std::initializer_list<std::initializer_list<int> > s) {
        int i = 0;
        for (auto& p : s) { int j = 0; for (int c : p) t.side[i][j++] = c; t.sideNco[i] = j; ++i; }
        t.numSides = i;
    };
    switch (roid) {
        case ROID_EDGE:
            t.dim = 1; corners({{0}, {1}}); edges({{0, 1}}); sides({{0}, {1}});
            break;
        case ROID_TRIANGLE:
            t.dim = 2; corners({{0, 0}, {1, 0}, {0, 1}}); edges({{0, 1}, {1, 2}, {2, 0}});
            sides({{0, 1}, {1, 2}, {2, 0}});
            break;
        case ROID_QUADRILATERAL:
            t.dim = 2; corners({{0, 0}, {1, 0}, {1, 1}, {0, 1}}); edges({{0, 1}, {1, 2}, {2, 3}, {3, 0}});
            sides({{0, 1}, {1, 2}, {2, 3}, {3, 0}});
            break;
        case ROID_TETRAHEDRON:
            t.dim = 3; corners({{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}});
            edges({{0, 1}, {1, 2}, {2, 0}, {0, 3}, {1, 3}, {2, 3}});
            sides({{0, 2, 1}, {0, 1, 3}, {1, 2, 3}, {0, 3, 2}});
            break;
        case ROID_PYRAMID:
            t.dim = 3; corners({{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0}, {0, 0, 1}});
            edges({{0, 1}, {1, 2}, {2, 3}, {3, 0}, {0, 4}, {1, 4}, {2, 4}, {3, 4}});
            sides({{0, 3, 2, 1}, {0, 1, 4}, {1, 2, 4}, {2, 3, 4}, {3, 0, 4}});
            break;
        case ROID_PRISM:
            t.dim = 3; corners({{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {1, 0, 1}, {0, 1, 1}});
            edges({{0, 1}, {1, 2}, {2, 0}, {0, 3}, {1, 4}, {2, 5}, {3, 4}, {4, 5}, {5, 3}});
            sides({{0, 2, 1}, {0, 1, 4, 3}, {1, 2, 5, 4}, {2, 0, 3, 5}, {3, 4, 5}});
            break;
        case ROID_HEXAHEDRON:
            t.dim = 3; corners({{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0}, {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}});
            edges({{0, 1}, {1, 2}, {2, 3}, {3, 0}, {0, 4}, {1, 5}, {2, 6}, {3, 7}, {4, 5}, {5, 6}, {6, 7}, {7, 4}});
            sides({{0, 3, 2, 1}, {0, 1, 5, 4}, {1, 2, 6, 5}, {2, 3, 7, 6}, {0, 4, 7, 3}, {4, 5, 6, 7}});
            break;
        default: throw UGError("reference element not available");
    }
    return t;
}

template <ReferenceObjectID ROID>
inline const RefTables& ref_tables() {
    static const RefTables t = make_ref_tables(ROID);
    return t;
}

template <int TDim, ReferenceObjectID ROID, int TNumCorners, int TNumEdges, int TNumSides>
class ReferenceElementBase {
  public:
    static const int dim = TDim;
    static const int numCorners = TNumCorners;
    static const int numEdges = TNumEdges;
    static const int numSides = TNumSides;
    static const ReferenceObjectID REFERENCE_OBJECT_ID = ROID;
    ReferenceObjectID roid() const { return ROID; }
    int dimension() const { return dim; }
    size_t num(int d) const { return d == 0 ? numCorners : d == 1 ? numEdges : d == dim - 1 ? numSides : 1; }
    // number of sub-objects of dimension dim_j of the sub-object i of dimension dim_i
    size_t num(int dim_i, size_t i, int dim_j) const {
        const RefTables& t = ref_tables<ROID>();
        if (dim_j != 0) UG_THROW("reference element: only corner sub-objects are tabulated");
        if (dim_i == dim) return numCorners;
        if (dim_i == 1) return 2;
        if (dim_i == dim - 1) return t.sideNco[i];
        if (dim_i == 0) return 1;
        UG_THROW("reference element: sub-object dimension");
    }
    // id of the j-th corner of the sub-object i of dimension dim_i
    size_t id(int dim_i, size_t i, int dim_j, size_t j) const {
        const RefTables& t = ref_tables<ROID>();
        if (dim_j != 0) UG_THROW("reference element: only corner sub-objects are tabulated");
        if (dim_i == dim) return j;
        if (dim_i == 1) return t.edge[i][j];
        if (dim_i == dim - 1) return t.side[i][j];
        if (dim_i == 0) return i;
        UG_THROW("reference element: sub-object dimension");
    }
    MathVector<TDim> corner(size_t i) const {
        MathVector<TDim> c;
        for (int d = 0; d < TDim; ++d) c[d] = ref_tables<ROID>().co[i][d];
        return c;
    }
};

class ReferenceEdge : public ReferenceElementBase<1, ROID_EDGE, 2, 1, 2> {};
class ReferenceTriangle : public ReferenceElementBase<2, ROID_TRIANGLE, 3, 3, 3> {};
class ReferenceQuadrilateral : public ReferenceElementBase<2, ROID_QUADRILATERAL, 4, 4, 4> {};
class ReferenceTetrahedron : public ReferenceElementBase<3, ROID_TETRAHEDRON, 4, 6, 4> {};
class ReferencePyramid : public ReferenceElementBase<3, ROID_PYRAMID, 5, 8, 5> {};
class ReferencePrism : public ReferenceElementBase<3, ROID_PRISM, 6, 9, 5> {};
class ReferenceHexahedron : public ReferenceElementBase<3, ROID_HEXAHEDRON, 8, 12, 6> {};

class RegularEdge : public GridObject { public: static const int dim = 1; };
class Triangle : public GridObject { public: static const int dim = 2; };
class Quadrilateral : public GridObject { public: static const int dim = 2; };
class Tetrahedron : public GridObject { public: static const int dim = 3; };
class Pyramid : public GridObject { public: static const int dim = 3; };
class Prism : public GridObject { public: static const int dim = 3; };
class Hexahedron : public GridObject { public: static const int dim = 3; };

template <class TElem> struct reference_element_traits;
template <> struct reference_element_traits<RegularEdge> { typedef ReferenceEdge reference_element_type; static const int dim = 1; };
template <> struct reference_element_traits<Triangle> { typedef ReferenceTriangle reference_element_type; static const int dim = 2; };
template <> struct reference_element_traits<Quadrilateral> { typedef ReferenceQuadrilateral reference_element_type; static const int dim = 2; };
template <> struct reference_element_traits<Tetrahedron> { typedef ReferenceTetrahedron reference_element_type; static const int dim = 3; };
template <> struct reference_element_traits<Pyramid> { typedef ReferencePyramid reference_element_type; static const int dim = 3; };
template <> struct reference_element_traits<Prism> { typedef ReferencePrism reference_element_type; static const int dim = 3; };
template <> struct reference_element_traits<Hexahedron> { typedef ReferenceHexahedron reference_element_type; static const int dim = 3; };

template <class TElem> struct geometry_traits {
    static const ReferenceObjectID REFERENCE_OBJECT_ID = reference_element_traits<TElem>::reference_element_type::REFERENCE_OBJECT_ID;
};

/* ---- providers (ugcore: common/util/provider.h, disc_util/geom_provider.h) - */
template <class T> class Provider {
  public:
    static T& get() { static T inst; return inst; }
};
template <class T> class GeomProvider {
  public:
    static T& get() { static T inst; return inst; }
};

/* ---- P1 Lagrange shape functions (ugcore: lib_disc/local_finite_element) --- */
struct LFEID {
    enum SpaceType { NONE = -1, LAGRANGE = 0, CROUZEIX_RAVIART, PIECEWISE_CONSTANT, DG, MINI, NEDELEC, USER_DEFINED };
    LFEID() : m_type(NONE), m_dim(-1), m_order(-1) {}
    LFEID(SpaceType t, int d, int o) : m_type(t), m_dim(d), m_order(o) {}
    SpaceType type() const { return m_type; }
    int dim() const { return m_dim; }
    int order() const { return m_order; }

  private:
    SpaceType m_type;
    int m_dim, m_order;
};

// P1 shape of corner k at the local point x: barycentric on simplices,
// multilinear on the tensor elements
inline number p1_shape(ReferenceObjectID roid, size_t k, const number* x) {
    switch (roid) {
        case ROID_EDGE: return k == 0 ? 1.0 - x[0] : x[0];
        case ROID_TRIANGLE: return k == 0 ? 1.0 - x[0] - x[1] : x[k - 1];
        case ROID_TETRAHEDRON: return k == 0 ? 1.0 - x[0] - x[1] - x[2] : x[k - 1];
        case ROID_QUADRILATERAL: {
            const number a = (k == 1 || k == 2) ? x[0] : 1.0 - x[0];
            const number b = (k >= 2) ? x[1] : 1.0 - x[1];
            return a * b;
        }
        case ROID_PRISM: {
            // triangle shape of corner k % 3 times the linear shape in z
            const size_t q = k % 3;
            const number t = q == 0 ? 1.0 - x[0] - x[1] : x[q - 1];
            return t * ((k >= 3) ? x[2] : 1.0 - x[2]);
        }
        case ROID_HEXAHEDRON: {
            const size_t q = k % 4;
            const number a = (q == 1 || q == 2) ? x[0] : 1.0 - x[0];
            const number b = (q >= 2) ? x[1] : 1.0 - x[1];
            const number c = (k >= 4) ? x[2] : 1.0 - x[2];
            return a * b * c;
        }
        default: UG_THROW("P1 shapes: element type not available here");
    }
}
// derivative of the P1 shape of corner k along local direction d at x
inline number p1_deriv(ReferenceObjectID roid, size_t k, int d, const number* x) {
    switch (roid) {
        case ROID_EDGE: return k == 0 ? -1.0 : 1.0;
        case ROID_TRIANGLE:
        case ROID_TETRAHEDRON: return k == 0 ? -1.0 : ((size_t)d == k - 1 ? 1.0 : 0.0);
        case ROID_QUADRILATERAL: {
            const number s0 = (k == 1 || k == 2) ? 1.0 : -1.0, s1 = (k >= 2) ? 1.0 : -1.0;
            const number a = (k == 1 || k == 2) ? x[0] : 1.0 - x[0];
            const number b = (k >= 2) ? x[1] : 1.0 - x[1];
            return d == 0 ? s0 * b : s1 * a;
        }
        case ROID_PRISM: {
            const size_t q = k % 3;
            const number t = q == 0 ? 1.0 - x[0] - x[1] : x[q - 1];
            const number z = (k >= 3) ? x[2] : 1.0 - x[2];
            if (d == 2) return (k >= 3) ? t : -t;
            const number dt = q == 0 ? -1.0 : ((size_t)d == q - 1 ? 1.0 : 0.0);
            return dt * z;
        }
        case ROID_HEXAHEDRON: {
            const size_t q = k % 4;
            const number s0 = (q == 1 || q == 2) ? 1.0 : -1.0, s1 = (q >= 2) ? 1.0 : -1.0, s2 = (k >= 4) ? 1.0 : -1.0;
            const number a = (q == 1 || q == 2) ? x[0] : 1.0 - x[0];
            const number b = (q >= 2) ? x[1] : 1.0 - x[1];
            const number c = (k >= 4) ? x[2] : 1.0 - x[2];
            return d == 0 ? s0 * b * c : d == 1 ? a * s1 * c : a * b * s2;
        }
        default: UG_THROW("P1 shapes: element type not available here");
    }
}

template <int TDim>
class LocalShapeFunctionSet {
  public:
    explicit LocalShapeFunctionSet(ReferenceObjectID roid = ROID_UNKNOWN) : m_roid(roid) {}
    number shape(size_t k, const MathVector<TDim>& x) const {
        number xx[3] = {0, 0, 0};
        for (int d = 0; d < TDim; ++d) xx[d] = x[d];
        return p1_shape(m_roid, k, xx);
    }

  private:
    ReferenceObjectID m_roid;
};

// P1 trial space of a reference element (used by the reference's data exports)
template <class TRefElem>
class LagrangeP1 {
  public:
    static const int dim = TRefElem::dim;
    static const size_t nsh = TRefElem::numCorners;
    size_t num_sh() const { return nsh; }
    number shape(size_t k, const MathVector<dim>& x) const { return p1_shape(TRefElem::REFERENCE_OBJECT_ID, k, pt(x).v); }
    void shapes(number* out, const MathVector<dim>& x) const {
        for (size_t k = 0; k < nsh; ++k) out[k] = p1_shape(TRefElem::REFERENCE_OBJECT_ID, k, pt(x).v);
    }
    void grads(MathVector<dim>* out, const MathVector<dim>& x) const {
        for (size_t k = 0; k < nsh; ++k)
            for (int d = 0; d < dim; ++d) out[k][d] = p1_deriv(TRefElem::REFERENCE_OBJECT_ID, k, d, pt(x).v);
    }

  private:
    struct P { number v[3]; };
    static P pt(const MathVector<dim>& x) { P p = {{0, 0, 0}}; for (int d = 0; d < dim; ++d) p.v[d] = x[d]; return p; }
};

// the multilinear map of a reference element onto its corners
template <class TRefElem, int TWorldDim>
class ReferenceMapping {
  public:
    static const int dim = TRefElem::dim;
    explicit ReferenceMapping(const MathVector<TWorldDim>* corners = nullptr) : m_co(corners) {}
    void update(const MathVector<TWorldDim>* corners) { m_co = corners; }
    void jacobian(MathMatrix<TWorldDim, dim>& J, const MathVector<dim>& x) const {
        number xx[3] = {0, 0, 0};
        for (int d = 0; d < dim; ++d) xx[d] = x[d];
        J = 0.0;
        for (size_t k = 0; k < TRefElem::numCorners; ++k)
            for (int r = 0; r < TWorldDim; ++r)
                for (int c = 0; c < dim; ++c) J(r, c) += m_co[k][r] * p1_deriv(TRefElem::REFERENCE_OBJECT_ID, k, c, xx);
    }
    number jacobian_transposed_inverse(MathMatrix<TWorldDim, dim>& G, const MathVector<dim>& x) const {
        if (dim != TWorldDim) UG_THROW("ReferenceMapping: manifold elements not available in this shim");
        MathMatrix<TWorldDim, dim> J;
        jacobian(J, x);
        number A[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, B[3][3];
        for (int r = 0; r < TWorldDim; ++r) for (int c = 0; c < dim; ++c) A[r][c] = J(r, c);
        const number det = shim_jt_inverse(dim, A, B);
        for (int r = 0; r < TWorldDim; ++r) for (int c = 0; c < dim; ++c) G(r, c) = B[r][c];
        return det;
    }
    void local_to_global(MathVector<TWorldDim>& g, const MathVector<dim>& x) const {
        number xx[3] = {0, 0, 0};
        for (int d = 0; d < dim; ++d) xx[d] = x[d];
        VecSet(g, 0.0);
        for (size_t k = 0; k < TRefElem::numCorners; ++k) VecScaleAppend(g, p1_shape(TRefElem::REFERENCE_OBJECT_ID, k, xx), m_co[k]);
    }

  private:
    static number shim_jt_inverse(int d, const number J[3][3], number G[3][3]);
    const MathVector<TWorldDim>* m_co;
};

class LocalFiniteElementProvider {
  public:
    template <int TDim>
    static const LocalShapeFunctionSet<TDim>& get(ReferenceObjectID roid, const LFEID& id) {
        if (id.type() != LFEID::LAGRANGE || id.order() != 1) UG_THROW("LocalFiniteElementProvider: only P1 Lagrange here");
        static LocalShapeFunctionSet<TDim> sets[NUM_REFERENCE_OBJECTS] = {};
        static bool init = false;
        if (!init) {
            for (int r = 0; r < NUM_REFERENCE_OBJECTS; ++r) sets[r] = LocalShapeFunctionSet<TDim>((ReferenceObjectID)r);
            init = true;
        }
        return sets[roid];
    }
};

/* ---- local algebra (ugcore: lib_disc/common/local_algebra.h) -------------- */
// Element-local vector u(fct, sh) and matrix J(fct1, sh1, fct2, sh2), stored
// fct-major: u[fct * nsh + sh], J[((f1 * nsh + s1) * nfct + f2) * nsh + s2].
class LocalVector {
  public:
    LocalVector() : m_nfct(0), m_nsh(0) {}
    LocalVector(size_t nfct, size_t nsh) { resize(nfct, nsh); }
    void resize(size_t nfct, size_t nsh) { m_nfct = nfct; m_nsh = nsh; m_v.assign(nfct * nsh, 0.0); }
    number& operator()(size_t fct, size_t sh) { return m_v[fct * m_nsh + sh]; }
    const number& operator()(size_t fct, size_t sh) const { return m_v[fct * m_nsh + sh]; }
    size_t num_all_dof(size_t) const { return m_nsh; }
    size_t num_all_fct() const { return m_nfct; }
    number* data() { return m_v.data(); }
    const number* data() const { return m_v.data(); }
    void zero() { std::fill(m_v.begin(), m_v.end(), 0.0); }

  private:
    size_t m_nfct, m_nsh;
    std::vector<number> m_v;
};

class LocalMatrix {
  public:
    LocalMatrix() : m_nfct(0), m_nsh(0) {}
    LocalMatrix(size_t nfct, size_t nsh) { resize(nfct, nsh); }
    void resize(size_t nfct, size_t nsh) { m_nfct = nfct; m_nsh = nsh; m_v.assign(nfct * nsh * nfct * nsh, 0.0); }
    number& operator()(size_t f1, size_t s1, size_t f2, size_t s2) { return m_v[((f1 * m_nsh + s1) * m_nfct + f2) * m_nsh + s2]; }
    const number& operator()(size_t f1, size_t s1, size_t f2, size_t s2) const { return m_v[((f1 * m_nsh + s1) * m_nfct + f2) * m_nsh + s2]; }
    number* data() { return m_v.data(); }
    void zero() { std::fill(m_v.begin(), m_v.end(), 0.0); }

  private:
    size_t m_nfct, m_nsh;
    std::vector<number> m_v;
};

class LocalVectorTimeSeries {
  public:
    size_t size() const { return m_sol.size(); }
    const LocalVector& solution(size_t i) const { return *m_sol[i]; }
    number time(size_t i) const { return m_time[i]; }
    void set(const LocalVector* cur, number tCur, const LocalVector* old, number tOld) {
        m_sol.assign({cur, old});
        m_time.assign({tCur, tOld});
    }

  private:
    std::vector<const LocalVector*> m_sol;
    std::vector<number> m_time;
};

/* ---- user data, imports, exports (ugcore: lib_disc/spatial_disc/user_data) - */
template <typename TData, int dim, typename TRet = void>
class CplUserData {
  public:
    virtual ~CplUserData() {}
    // value at any point (the const data this shim evaluates)
    virtual TData value() const = 0;
};

template <int dim>
class ConstUserNumber : public CplUserData<number, dim> {
  public:
    explicit ConstUserNumber(number v) : m_v(v) {}
    number value() const override { return m_v; }

  private:
    number m_v;
};

template <int dim>
class ConstUserVector : public CplUserData<MathVector<dim>, dim> {
  public:
    explicit ConstUserVector(number v) { for (int d = 0; d < dim; ++d) m_v[d] = v; }
    explicit ConstUserVector(const std::vector<number>& v) {
        if ((int)v.size() != dim) UG_THROW("ConstUserVector: need exactly " << dim << " components");
        for (int d = 0; d < dim; ++d) m_v[d] = v[d];
    }
    MathVector<dim> value() const override { return m_v; }

  private:
    MathVector<dim> m_v;
};

class IDataImport {
  public:
    virtual ~IDataImport() {}
};

template <typename TData, int dim>
class DataImport : public IDataImport {
  public:
    DataImport(bool bLinDefect = true) : m_rhs(false), m_mass(false) { (void)bLinDefect; }
    void set_data(SmartPtr<CplUserData<TData, dim> > data) {
        m_data = data;
        if (m_data.valid()) m_val = m_data->value();
    }
    SmartPtr<CplUserData<TData, dim> > user_data() { return m_data; }
    bool data_given() const { return m_data.valid(); }
    void set_rhs_part(bool b = true) { m_rhs = b; }
    void set_mass_part(bool b = true) { m_mass = b; }
    template <int refDim> void set_local_ips(const MathVector<refDim>*, size_t) {}
    void set_global_ips(const MathVector<dim>*, size_t n) { m_num = n; }
    size_t num_ip() const { return m_num; }
    const TData& operator[](size_t) const { return m_val; }

  private:
    SmartPtr<CplUserData<TData, dim> > m_data;
    TData m_val{};
    size_t m_num = 0;
    bool m_rhs, m_mass;
};

// data exports are compiled (the base classes hold them) but never evaluated here
template <typename TData, int dim>
class DataExport : public CplUserData<TData, dim> {
  public:
    explicit DataExport(const char* functions) : m_fcts(functions ? functions : "") {}
    TData value() const override { UG_THROW("DataExport: not evaluated in this shim"); }

  private:
    std::string m_fcts;
};

/* ---- domains and the element-disc base (ugcore: lib_disc/spatial_disc) ---- */
template <int TDim> struct Domain { static const int dim = TDim; };
typedef Domain<1> Domain1d;
typedef Domain<2> Domain2d;
typedef Domain<3> Domain3d;

inline std::vector<std::string> TokenizeTrimString(const std::string& s) {
    std::vector<std::string> out;
    std::stringstream ss(s);
    std::string item;
    while (std::getline(ss, item, ',')) {
        item = TrimString(item);
        if (!item.empty()) out.push_back(item);
    }
    return out;
}

template <typename TDomain>
class IElemDisc {
  public:
    typedef TDomain domain_type;
    static const int dim = TDomain::dim;
    IElemDisc(const char* functions, const char* subsets)
        : m_vFct(TokenizeTrimString(functions ? functions : "")), m_vSubset(TokenizeTrimString(subsets ? subsets : "")) {}
    IElemDisc(const std::vector<std::string>& vFct, const std::vector<std::string>& vSubset) : m_vFct(vFct), m_vSubset(vSubset) {}
    virtual ~IElemDisc() {}
    size_t num_fct() const { return m_vFct.size(); }
    void register_import(IDataImport&) {}
    virtual void prepare_setting(const std::vector<LFEID>&, bool) {}
    virtual bool requests_local_time_series() { return false; }
    virtual std::string disc_type() const { return ""; }
    // time dependence as set by the driver: the current and the old local solution
    bool is_time_dependent() const { return m_pTimeSeries != nullptr; }
    const LocalVectorTimeSeries* local_time_solutions() const { return m_pTimeSeries; }
    void set_time_series(const LocalVectorTimeSeries* ts) { m_pTimeSeries = ts; }
    const ISubsetHandler& subset_handler() const { return m_sh; }
    const std::vector<std::string>& symb_fcts() const { return m_vFct; }
    const std::vector<std::string>& symb_subsets() const { return m_vSubset; }
    // every boundary subset name maps to subset 1
    struct ApproxSpace {
        SubsetGroup subset_grp_by_name(const char*) const { SubsetGroup g; g.add(1); return g; }
    };
    struct FunctionPattern {
        const ISubsetHandler* sh;
        const ISubsetHandler* subset_handler() const { return sh; }
    };
    const ApproxSpace* approx_space() const { static const ApproxSpace a; return &a; }
    const FunctionPattern* function_pattern() const { m_fp.sh = &m_sh; return &m_fp; }

  protected:
    mutable FunctionPattern m_fp{nullptr};
    std::vector<std::string> m_vFct, m_vSubset;
    const LocalVectorTimeSeries* m_pTimeSeries = nullptr;
    ISubsetHandler m_sh;
};

/* ---- finite-volume geometries (ugcore: lib_disc/spatial_disc/disc_util) ---- */
class FVGeometryBase {};

inline size_t next_fv_geom_id() { static size_t n = 0; return n++; }
template <typename TFVGeom> size_t GetUniqueFVGeomID() { static const size_t id = next_fv_geom_id(); return id; }

template <int TDim, int TWorldDim> struct fv1_dim_traits;
template <> struct fv1_dim_traits<1, 1> { static const size_t maxNumSCVF = 1, maxNumSCV = 2, maxNSH = 2; };
template <> struct fv1_dim_traits<2, 2> { static const size_t maxNumSCVF = 4, maxNumSCV = 4, maxNSH = 4; };
template <> struct fv1_dim_traits<3, 3> { static const size_t maxNumSCVF = 12, maxNumSCV = 8, maxNSH = 8; };

}  // namespace ug

#include "fv1_geometry_impl.h"

namespace ug {
template <class TRefElem, int TWorldDim>
number ReferenceMapping<TRefElem, TWorldDim>::shim_jt_inverse(int d, const number J[3][3], number G[3][3]) {
    return shim_detail::det_jtinv(d, J, G);
}
}  // namespace ug

#endif  // NSFV1_UG_SHIM_H
