// Per-element FV1 Navier-Stokes math for the sm_103a kernels: the SCVF/SCV
// geometry, the convective upwind shapes, the stabilised velocity and the
// local defect / Jacobian contributions, computed in registers by one thread
// per element.
//
// Reference behaviour followed (file:line in UG4 plugin_NavierStokes):
//   add_def_A_elem            incompressible/fv1/navier_stokes_fv1.cpp:597-778
//   add_jac_A_elem            incompressible/fv1/navier_stokes_fv1.cpp:250-595
//   add_def_M_elem/jac_M      incompressible/fv1/navier_stokes_fv1.cpp:781-838
//   add_rhs_elem              incompressible/fv1/navier_stokes_fv1.cpp:841-869
//   peclet_blend              incompressible/fv1/navier_stokes_fv1.cpp:871-892
//   FIELDS / FLOW / without   incompressible/fv1/stabilization.cpp:122-241, 436-588, 805-850
//   diffusion lengths         incompressible/fv1/diffusion_length.h:48-199
//   no / full / skewed / LPS  upwind.cpp:52-80, 133-172, 337-430, 505-575
//   upwind_vel, downwind      upwind_interface.h:150-165, 333-358
//
// The stabilised velocity and the continuity-row Jacobian are evaluated in a
// regrouped but algebraically identical form: sum_k (a N_k + b U_k) u_k is
// computed as a StdVel + b UpVel, and the FLOW cross terms collapse to
// (S_k - V.g_k) n + (V.n) g_k. Results agree with the term-by-term reference
// order to rounding (the parity tests hold them to 1e-12 relative in FP64).
//
// The SCVF loop runs over a warp-uniform runtime index: per-SCVF constants
// (shapes and local gradients at the integration points, edge/face/side
// tables) come from __constant__ tables (broadcast loads), corner data with a
// runtime index is selected from registers without local-memory indexing.
#pragma once
#include <cstdint>
#include <type_traits>
#include "nsfv1_params.h"
#include "nsfv1_refelem.cuh"

namespace nsfv1 {

// ---------------------------------------------------------------------------
// per-element-type tables (generated at compile time from nsfv1_refelem.cuh)
// ---------------------------------------------------------------------------
// Tables in the arithmetic type F of the kernel (double or float): a float
// kernel reading double constants would convert every use on the FP64 pipe.
template <typename F>
struct ElemTabT {
    F ipLoc[12][3];   // local (reference) coordinates of the SCVF integration points
    F ipShape[12][8];
    F ipLGrad[12][8][3];
    F refCo[8][3];
    int edge[12][2];
    int edgeFace[12][2];
    int side[6][4];
    int sideNco[6];
    int sideMask[6];   // bit k set: corner k belongs to the side
};
typedef ElemTabT<double> ElemTab;

template <int ROID, typename F> constexpr ElemTabT<F> make_tab() {
    using R = Ref<ROID>;
    ElemTabT<F> t{};
    for (int ip = 0; ip < R::nip; ++ip) {
        for (int k = 0; k < R::nsh; ++k) {
            t.ipShape[ip][k] = F(ip_shape<ROID>(ip, k));
            for (int d = 0; d < R::dim; ++d) t.ipLGrad[ip][k][d] = F(ip_lgrad<ROID>(ip, k, d));
        }
        for (int d = 0; d < 3; ++d) t.ipLoc[ip][d] = F(d < R::dim ? loc_ip<R>(ip, d) : 0.0);
        t.edge[ip][0] = R::edge(ip, 0); t.edge[ip][1] = R::edge(ip, 1);
        t.edgeFace[ip][0] = R::edge_face(ip, 0); t.edgeFace[ip][1] = R::edge_face(ip, 1);
    }
    for (int c = 0; c < R::nsh; ++c)
        for (int d = 0; d < 3; ++d) t.refCo[c][d] = F(d < R::dim ? R::co(c, d) : 0.0);
    for (int s = 0; s < R::nside; ++s) {
        t.sideNco[s] = R::side_nco(s);
        int m = 0;
        for (int j = 0; j < 4; ++j) {
            t.side[s][j] = j < R::side_nco(s) ? R::side(s, j) : R::side(s, 0);
            if (j < R::side_nco(s)) m |= 1 << R::side(s, j);
        }
        t.sideMask[s] = m;
    }
    return t;
}

static __constant__ ElemTabT<double> c_tabTri = make_tab<ROID_TRIANGLE, double>();
static __constant__ ElemTabT<double> c_tabQuad = make_tab<ROID_QUADRILATERAL, double>();
static __constant__ ElemTabT<double> c_tabTet = make_tab<ROID_TETRAHEDRON, double>();
static __constant__ ElemTabT<double> c_tabPrism = make_tab<ROID_PRISM, double>();
static __constant__ ElemTabT<double> c_tabHex = make_tab<ROID_HEXAHEDRON, double>();
static __constant__ ElemTabT<float> c_tabTriF = make_tab<ROID_TRIANGLE, float>();
static __constant__ ElemTabT<float> c_tabQuadF = make_tab<ROID_QUADRILATERAL, float>();
static __constant__ ElemTabT<float> c_tabTetF = make_tab<ROID_TETRAHEDRON, float>();
static __constant__ ElemTabT<float> c_tabPrismF = make_tab<ROID_PRISM, float>();
static __constant__ ElemTabT<float> c_tabHexF = make_tab<ROID_HEXAHEDRON, float>();

template <int ROID, typename F = double> __device__ __forceinline__ const ElemTabT<F>& tab() {
    if constexpr (std::is_same<F, float>::value) {
        if constexpr (ROID == ROID_TRIANGLE) return c_tabTriF;
        else if constexpr (ROID == ROID_QUADRILATERAL) return c_tabQuadF;
        else if constexpr (ROID == ROID_TETRAHEDRON) return c_tabTetF;
        else if constexpr (ROID == ROID_PRISM) return c_tabPrismF;
        else return c_tabHexF;
    } else {
        if constexpr (ROID == ROID_TRIANGLE) return c_tabTri;
        else if constexpr (ROID == ROID_QUADRILATERAL) return c_tabQuad;
        else if constexpr (ROID == ROID_TETRAHEDRON) return c_tabTet;
        else if constexpr (ROID == ROID_PRISM) return c_tabPrism;
        else return c_tabHex;
    }
}

template <typename T> struct Num;
template <> struct Num<double> {
    static __device__ __forceinline__ double sqrt_(double x) { return sqrt(x); }
    static __device__ __forceinline__ double abs_(double x) { return fabs(x); }
};
template <> struct Num<float> {
    static __device__ __forceinline__ float sqrt_(float x) { return sqrtf(x); }
    static __device__ __forceinline__ float abs_(float x) { return fabsf(x); }
};

// ---------------------------------------------------------------------------
// Element-level geometry shared by all SCVFs: corners, centre, face centres,
// SCV volumes.
// ---------------------------------------------------------------------------
template <int ROID, typename T>
struct Elem {
    using R = Ref<ROID>;
    static constexpr int dim = R::dim, nsh = R::nsh, nip = R::nip, b = R::b, nside = R::nside;
    T x[nsh][dim];
    T cen[dim];
    T face[nside][dim];
    T vol[nsh];
    bool affine;        // the reference mapping is affine (simplex, parallelogram, parallelepiped)
    T JtInv[3][3];      // constant J^-T of an affine element
};

// -v by flipping the sign bit with an integer XOR: exact like the negation
// itself, and it keeps the negated copies of the fluxes and Jacobian entries
// (one per entry of every 'to' row) off the FP64 / FP32 arithmetic pipes
__device__ __forceinline__ double flip_sign(const double v) {
    return __longlong_as_double(__double_as_longlong(v) ^ (long long)0x8000000000000000ULL);
}
__device__ __forceinline__ float flip_sign(const float v) { return __int_as_float(__float_as_int(v) ^ (int)0x80000000u); }

// Affine test: simplices always, prisms never; a quadrilateral / hexahedron when every corner
// equals x0 + the sum of its edge vectors to within rtol of the element size.
// On such elements the mapping Jacobian is one constant matrix and the FV1
// quantities below are evaluated from it (algebraically identical to the
// per-ip evaluation, equal to rounding).
// running maximum that propagates NaN (fmax would drop it)
template <typename T> __device__ __forceinline__ T nanmax(const T a, const T b) { return (b <= a) ? a : b; }

template <int ROID, typename T>
__device__ __forceinline__ bool elem_is_affine(const Elem<ROID, T>& E) {
    if constexpr (ROID == ROID_TRIANGLE || ROID == ROID_TETRAHEDRON) return true;
    // prisms always take the general path (J at every integration point)
    if constexpr (ROID == ROID_PRISM) return false;
    const T rtol = sizeof(T) == 8 ? T(1e-14) : T(1e-6);
    T sz = T(0), dev = T(0);
    if constexpr (ROID == ROID_QUADRILATERAL) {
#pragma unroll
        for (int d = 0; d < 2; ++d) {
            sz = nanmax(sz, nanmax(Num<T>::abs_(E.x[1][d] - E.x[0][d]), Num<T>::abs_(E.x[3][d] - E.x[0][d])));
            dev = nanmax(dev, Num<T>::abs_((E.x[2][d] - E.x[1][d]) - (E.x[3][d] - E.x[0][d])));
        }
    } else {
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const T a = E.x[1][d] - E.x[0][d], b = E.x[3][d] - E.x[0][d], c = E.x[4][d] - E.x[0][d];
            sz = nanmax(sz, nanmax(Num<T>::abs_(a), nanmax(Num<T>::abs_(b), Num<T>::abs_(c))));
            dev = nanmax(dev, Num<T>::abs_((E.x[2][d] - E.x[0][d]) - (a + b)));
            dev = nanmax(dev, Num<T>::abs_((E.x[5][d] - E.x[0][d]) - (a + c)));
            dev = nanmax(dev, Num<T>::abs_((E.x[7][d] - E.x[0][d]) - (b + c)));
            dev = nanmax(dev, Num<T>::abs_((E.x[6][d] - E.x[0][d]) - (a + b + c)));
        }
    }
    return dev <= rtol * sz;   // false when anything is NaN
}

// J^-T and |det J| from a 2x2 / 3x3 Jacobian
template <int dim, typename T>
__device__ __forceinline__ T jt_inverse(const T (&J)[3][3], T (&JtInv)[3][3]) {
    if constexpr (dim == 2) {
        const T det = J[0][0] * J[1][1] - J[0][1] * J[1][0];
        const T id = T(1) / det;
        JtInv[0][0] = J[1][1] * id;  JtInv[0][1] = -J[1][0] * id;
        JtInv[1][0] = -J[0][1] * id; JtInv[1][1] = J[0][0] * id;
        return det;
    } else {
        T C[3][3];
        C[0][0] = J[1][1] * J[2][2] - J[1][2] * J[2][1];
        C[0][1] = J[1][2] * J[2][0] - J[1][0] * J[2][2];
        C[0][2] = J[1][0] * J[2][1] - J[1][1] * J[2][0];
        C[1][0] = J[0][2] * J[2][1] - J[0][1] * J[2][2];
        C[1][1] = J[0][0] * J[2][2] - J[0][2] * J[2][0];
        C[1][2] = J[0][1] * J[2][0] - J[0][0] * J[2][1];
        C[2][0] = J[0][1] * J[1][2] - J[0][2] * J[1][1];
        C[2][1] = J[0][2] * J[1][0] - J[0][0] * J[1][2];
        C[2][2] = J[0][0] * J[1][1] - J[0][1] * J[1][0];
        const T det = J[0][0] * C[0][0] + J[0][1] * C[0][1] + J[0][2] * C[0][2];
        const T id = T(1) / det;
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) JtInv[i][j] = C[i][j] * id;
        return det;
    }
}

// corner 'i' (runtime index) of a register array, by selects (no local memory)
template <int N, int D, typename T>
__device__ __forceinline__ void pick(const T (&a)[N][D], const int i, T* out) {
#pragma unroll
    for (int d = 0; d < D; ++d) {
        T v = a[0][d];
#pragma unroll
        for (int k = 1; k < N; ++k) v = (k == i) ? a[k][d] : v;
        out[d] = v;
    }
}

template <typename T> __device__ __forceinline__ T tet6(const T* a, const T* b, const T* c, const T* d) {
    T u[3], v[3], w[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) { u[k] = b[k] - a[k]; v[k] = c[k] - a[k]; w[k] = d[k] - a[k]; }
    const T x0 = v[1] * w[2] - v[2] * w[1];
    const T x1 = v[2] * w[0] - v[0] * w[2];
    const T x2 = v[0] * w[1] - v[1] * w[0];
    return u[0] * x0 + u[1] * x1 + u[2] * x2;
}

template <int ROID, typename T>
__device__ __forceinline__ void elem_setup(Elem<ROID, T>& E) {
    using R = Ref<ROID>;
    constexpr int dim = R::dim, nsh = R::nsh;
#pragma unroll
    for (int d = 0; d < dim; ++d) {
        T s = T(0);
#pragma unroll
        for (int c = 0; c < nsh; ++c) s += E.x[c][d];
        E.cen[d] = s * T(1.0 / nsh);
    }
    if constexpr (dim == 3) {
#pragma unroll
        for (int f = 0; f < R::nside; ++f)
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                T s = T(0);
#pragma unroll
                for (int j = 0; j < R::side_nco(f); ++j) s += E.x[R::side(f, j)][d];
                E.face[f][d] = s * T(1.0 / R::side_nco(f));
            }
    }
    E.affine = elem_is_affine<ROID, T>(E);
    if (E.affine) {
        // constant Jacobian: columns are the edge vectors of the reference axes
        T J[3][3] = {{T(0), T(0), T(0)}, {T(0), T(0), T(0)}, {T(0), T(0), T(0)}};
        constexpr int ax1 = (ROID == ROID_QUADRILATERAL || ROID == ROID_HEXAHEDRON) ? 3 : 2;
        constexpr int ax2 = (ROID == ROID_HEXAHEDRON) ? 4 : 3;
#pragma unroll
        for (int r = 0; r < dim; ++r) {
            J[r][0] = E.x[1][r] - E.x[0][r];
            J[r][1] = E.x[ax1][r] - E.x[0][r];
            if constexpr (dim == 3) J[r][2] = E.x[ax2][r] - E.x[0][r];
        }
        const T det = jt_inverse<dim, T>(J, E.JtInv);
        // SCV measure: |det J| x reference measure / number of corners
        constexpr double frac = ROID == ROID_TRIANGLE ? 1.0 / 6.0 : ROID == ROID_QUADRILATERAL ? 0.25
                              : ROID == ROID_TETRAHEDRON ? 1.0 / 24.0 : 0.125;
        const T v = Num<T>::abs_(det) * T(frac);
#pragma unroll
        for (int a = 0; a < nsh; ++a) E.vol[a] = v;
        return;
    }
    // SCV volumes
#pragma unroll
    for (int a = 0; a < nsh; ++a) {
        if constexpr (dim == 2) {
            const int nxt = a;                    // edge a starts at corner a
            const int prv = (a + nsh - 1) % nsh;  // edge a-1 ends at corner a
            T p1[2], p3[2];
#pragma unroll
            for (int d = 0; d < 2; ++d) {
                p1[d] = T(0.5) * (E.x[R::edge(nxt, 0)][d] + E.x[R::edge(nxt, 1)][d]);
                p3[d] = T(0.5) * (E.x[R::edge(prv, 0)][d] + E.x[R::edge(prv, 1)][d]);
            }
            const T cr = (E.cen[0] - E.x[a][0]) * (p3[1] - p1[1]) - (E.cen[1] - E.x[a][1]) * (p3[0] - p1[0]);
            E.vol[a] = T(0.5) * Num<T>::abs_(cr);
        } else {
            T q1[3], q2[3], q3[3], q4[3], q5[3], q7[3];
            const int e0 = R::scv_tab(a, 0), f01 = R::scv_tab(a, 1), e1 = R::scv_tab(a, 2);
            const int e2 = R::scv_tab(a, 3), f02 = R::scv_tab(a, 4), f12 = R::scv_tab(a, 5);
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                q1[d] = T(0.5) * (E.x[R::edge(e0, 0)][d] + E.x[R::edge(e0, 1)][d]);
                q3[d] = T(0.5) * (E.x[R::edge(e1, 0)][d] + E.x[R::edge(e1, 1)][d]);
                q4[d] = T(0.5) * (E.x[R::edge(e2, 0)][d] + E.x[R::edge(e2, 1)][d]);
                q2[d] = E.face[f01][d]; q5[d] = E.face[f02][d]; q7[d] = E.face[f12][d];
            }
            const T* q0 = E.x[a];
            const T* q6 = E.cen;
            const T s6 = tet6(q0, q1, q2, q6) + tet6(q0, q2, q3, q6) + tet6(q0, q3, q7, q6)
                       + tet6(q0, q7, q4, q6) + tet6(q0, q4, q5, q6) + tet6(q0, q5, q1, q6);
            E.vol[a] = Num<T>::abs_(s6) / T(6.0);
        }
    }
}

// ---------------------------------------------------------------------------
// Per-SCVF geometry: normal, global ip, corners, J^-T at the local ip.
// ---------------------------------------------------------------------------
template <typename T> struct IpGeo {
    int from, to;
    T n[3], gip[3], em[3], xf[3], xt[3];
    T JtInv[3][3];
};

template <int ROID, typename T>
__device__ __forceinline__ void ip_geom(const Elem<ROID, T>& E, const int ip, IpGeo<T>& G) {
    using R = Ref<ROID>;
    constexpr int dim = R::dim, nsh = R::nsh;
    const auto& tb = tab<ROID, T>();
    G.from = tb.edge[ip][0]; G.to = tb.edge[ip][1];
    pick(E.x, G.from, G.xf);
    pick(E.x, G.to, G.xt);
#pragma unroll
    for (int d = 0; d < dim; ++d) G.em[d] = T(0.5) * (G.xf[d] + G.xt[d]);
    if constexpr (dim == 2) {
        const T dx = E.cen[0] - G.em[0], dy = E.cen[1] - G.em[1];
        G.n[0] = dy; G.n[1] = -dx; G.n[2] = T(0);
#pragma unroll
        for (int d = 0; d < 2; ++d) G.gip[d] = (G.em[d] + E.cen[d]) * T(0.5);
        G.gip[2] = T(0);
    } else {
        T f1[3], f2[3];
        pick(E.face, tb.edgeFace[ip][0], f1);
        pick(E.face, tb.edgeFace[ip][1], f2);
        T a[3], c[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) { a[d] = E.cen[d] - G.em[d]; c[d] = f2[d] - f1[d]; }
        G.n[0] = T(0.5) * (a[1] * c[2] - a[2] * c[1]);
        G.n[1] = T(0.5) * (a[2] * c[0] - a[0] * c[2]);
        G.n[2] = T(0.5) * (a[0] * c[1] - a[1] * c[0]);
#pragma unroll
        for (int d = 0; d < 3; ++d) G.gip[d] = (G.em[d] + f1[d] + E.cen[d] + f2[d]) * T(0.25);
    }
    if (E.affine) {
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) G.JtInv[i][j] = E.JtInv[i][j];
        return;
    }
    // Jacobian of the reference mapping at the local ip
    T J[3][3] = {{T(0), T(0), T(0)}, {T(0), T(0), T(0)}, {T(0), T(0), T(0)}};
#pragma unroll
    for (int r = 0; r < dim; ++r)
#pragma unroll
        for (int c = 0; c < dim; ++c) {
            T s = T(0);
#pragma unroll
            for (int k = 0; k < nsh; ++k) s += E.x[k][r] * T(tb.ipLGrad[ip][k][c]);
            J[r][c] = s;
        }
    jt_inverse<dim, T>(J, G.JtInv);
}

// P1 shapes and local gradients at the local point x (the element's trial space:
// linear on simplices, multilinear on quadrilaterals / hexahedra, ugcore corner order)
template <int ROID>
__device__ __forceinline__ void p1_eval(const double* x, double (&N)[Ref<ROID>::nsh], double (&G)[Ref<ROID>::nsh][3]) {
    const double a = x[0], b = x[1], c = x[2];
    if constexpr (ROID == ROID_TRIANGLE) {
        N[0] = 1.0 - a - b; N[1] = a; N[2] = b;
        G[0][0] = -1.0; G[0][1] = -1.0; G[1][0] = 1.0; G[1][1] = 0.0; G[2][0] = 0.0; G[2][1] = 1.0;
    } else if constexpr (ROID == ROID_QUADRILATERAL) {
        N[0] = (1.0 - a) * (1.0 - b); N[1] = a * (1.0 - b); N[2] = a * b; N[3] = (1.0 - a) * b;
        G[0][0] = -(1.0 - b); G[0][1] = -(1.0 - a); G[1][0] = 1.0 - b; G[1][1] = -a;
        G[2][0] = b;          G[2][1] = a;          G[3][0] = -b;      G[3][1] = 1.0 - a;
    } else if constexpr (ROID == ROID_PRISM) {
        const double t[3] = {1.0 - a - b, a, b}, dt[3][2] = {{-1.0, -1.0}, {1.0, 0.0}, {0.0, 1.0}};
#pragma unroll
        for (int k = 0; k < 6; ++k) {
            const int i = k % 3;
            const double z = k >= 3 ? c : 1.0 - c, dz = k >= 3 ? 1.0 : -1.0;
            N[k] = t[i] * z;
            G[k][0] = dt[i][0] * z; G[k][1] = dt[i][1] * z; G[k][2] = t[i] * dz;
        }
    } else if constexpr (ROID == ROID_TETRAHEDRON) {
        N[0] = 1.0 - a - b - c; N[1] = a; N[2] = b; N[3] = c;
#pragma unroll
        for (int k = 0; k < 4; ++k)
#pragma unroll
            for (int d = 0; d < 3; ++d) G[k][d] = (k == 0) ? -1.0 : (k == d + 1 ? 1.0 : 0.0);
    } else {
        const double ma = 1.0 - a, mb = 1.0 - b, mc = 1.0 - c;
        N[0] = ma * mb * mc; N[1] = a * mb * mc; N[2] = a * b * mc; N[3] = ma * b * mc;
        N[4] = ma * mb * c;  N[5] = a * mb * c;  N[6] = a * b * c;  N[7] = ma * b * c;
        G[0][0] = -mb * mc; G[0][1] = -ma * mc; G[0][2] = -ma * mb;
        G[1][0] = mb * mc;  G[1][1] = -a * mc;  G[1][2] = -a * mb;
        G[2][0] = b * mc;   G[2][1] = a * mc;   G[2][2] = -a * b;
        G[3][0] = -b * mc;  G[3][1] = ma * mc;  G[3][2] = -ma * b;
        G[4][0] = -mb * c;  G[4][1] = -ma * c;  G[4][2] = ma * mb;
        G[5][0] = mb * c;   G[5][1] = -a * c;   G[5][2] = a * mb;
        G[6][0] = b * c;    G[6][1] = a * c;    G[6][2] = a * b;
        G[7][0] = -b * c;   G[7][1] = ma * c;   G[7][2] = ma * b;
    }
}

// global gradient of shape k at the SCVF ip
template <int ROID, typename T>
__device__ __forceinline__ void ip_grad(const IpGeo<T>& G, const int ip, const int k, T g[3]) {
    constexpr int dim = Ref<ROID>::dim;
    const auto& tb = tab<ROID, T>();
#pragma unroll
    for (int r = 0; r < dim; ++r) {
        T s = T(0);
#pragma unroll
        for (int c = 0; c < dim; ++c) s += G.JtInv[r][c] * T(tb.ipLGrad[ip][k][c]);
        g[r] = s;
    }
}

template <int ROID, typename T>
__device__ __forceinline__ T ipN(const int ip, const int k) { return T(tab<ROID, T>().ipShape[ip][k]); }

// ---------------------------------------------------------------------------
// Upwind shapes of one SCVF (INavierStokesUpwind::compute, upwind.cpp)
// ---------------------------------------------------------------------------
template <typename T, int dim> __device__ __forceinline__ T dist(const T* a, const T* b) {
    T s = T(0);
#pragma unroll
    for (int d = 0; d < dim; ++d) { const T x = a[d] - b[d]; s += x * x; }
    return Num<T>::sqrt_(s);
}

// Ray from 'from' along 'dir' against the element sides in reference order
// (quadrilateral faces as triangles (0,1,2), (0,2,3)); the first side hit with
// t <= 0 is the upwind side (ElementSideRayIntersection, restated). LPS takes
// the element P1 shapes of the side corners at the local intersection, skewed
// the side corner nearest to the intersection. Returns false when no side is
// found (the reference throws).
template <int ROID, typename T>
__device__ __forceinline__ bool ray_upwind(const Elem<ROID, T>& E, const T* from, const T* dir, const bool lps,
                                           T (&up)[Ref<ROID>::nsh], T& convLen) {
    using R = Ref<ROID>;
    constexpr int dim = R::dim, nsh = R::nsh;
    const auto& tb = tab<ROID, T>();
    const T tol = T(1e-12);
    int hitSide = -1;
    T gInt[3] = {T(0), T(0), T(0)}, lInt[3] = {T(0), T(0), T(0)};
#pragma unroll 1
    for (int s = 0; s < R::nside && hitSide < 0; ++s) {
        // quadrilateral sides as two triangles (a prism mixes triangle and quadrilateral sides)
        constexpr int ntriMax = (dim == 3 && (R::side_nco(0) == 4 || ROID == ROID_PRISM)) ? 2 : 1;
        const int ntri = (ROID == ROID_PRISM) ? (tb.sideNco[s] == 4 ? 2 : 1) : ntriMax;
#pragma unroll
        for (int tr = 0; tr < ntriMax; ++tr) {
            if (hitSide >= 0 || tr >= ntri) break;
            if constexpr (dim == 2) {
                const int i0 = tb.side[s][0], i1 = tb.side[s][1];
                T p0[2], p1[2];
                pick(E.x, i0, p0);
                pick(E.x, i1, p1);
                const T a00 = p1[0] - p0[0], a01 = -dir[0];
                const T a10 = p1[1] - p0[1], a11 = -dir[1];
                const T det = a00 * a11 - a01 * a10;
                if (det != T(0)) {
                    const T r0 = from[0] - p0[0], r1 = from[1] - p0[1];
                    const T bc = (r0 * a11 - a01 * r1) / det;
                    const T t = (a00 * r1 - r0 * a10) / det;
                    if (!(bc < -tol || bc > T(1) + tol) && t <= T(0)) {
                        hitSide = s;
#pragma unroll
                        for (int d = 0; d < 2; ++d) {
                            gInt[d] = p0[d] + bc * (p1[d] - p0[d]);
                            lInt[d] = T(tb.refCo[i0][d]) + bc * (T(tb.refCo[i1][d]) - T(tb.refCo[i0][d]));
                        }
                    }
                }
            } else {
                const int i0 = tb.side[s][0];
                const int i1 = tb.side[s][tr == 0 ? 1 : 2];
                const int i2 = tb.side[s][tr == 0 ? 2 : 3];
                T q0[3], q1[3], q2[3];
                pick(E.x, i0, q0);
                pick(E.x, i1, q1);
                pick(E.x, i2, q2);
                T e1[3], e2[3], nd[3], r[3];
#pragma unroll
                for (int d = 0; d < 3; ++d) { e1[d] = q1[d] - q0[d]; e2[d] = q2[d] - q0[d]; nd[d] = -dir[d]; r[d] = from[d] - q0[d]; }
                const T c0 = e2[1] * nd[2] - e2[2] * nd[1];
                const T c1 = e2[2] * nd[0] - e2[0] * nd[2];
                const T c2 = e2[0] * nd[1] - e2[1] * nd[0];
                const T det = e1[0] * c0 + e1[1] * c1 + e1[2] * c2;
                if (det != T(0)) {
                    const T a = (r[0] * c0 + r[1] * c1 + r[2] * c2) / det;
                    const T w0 = r[1] * nd[2] - r[2] * nd[1];
                    const T w1 = r[2] * nd[0] - r[0] * nd[2];
                    const T w2 = r[0] * nd[1] - r[1] * nd[0];
                    const T bb = (e1[0] * w0 + e1[1] * w1 + e1[2] * w2) / det;
                    const T v0 = e2[1] * r[2] - e2[2] * r[1];
                    const T v1 = e2[2] * r[0] - e2[0] * r[2];
                    const T v2 = e2[0] * r[1] - e2[1] * r[0];
                    const T t = (e1[0] * v0 + e1[1] * v1 + e1[2] * v2) / det;
                    if (!(a < -tol || bb < -tol || a + bb > T(1) + tol) && t <= T(0)) {
                        hitSide = s;
#pragma unroll
                        for (int d = 0; d < 3; ++d) {
                            gInt[d] = q0[d] + a * e1[d] + bb * e2[d];
                            lInt[d] = T(tb.refCo[i0][d]) + a * (T(tb.refCo[i1][d]) - T(tb.refCo[i0][d]))
                                    + bb * (T(tb.refCo[i2][d]) - T(tb.refCo[i0][d]));
                        }
                    }
                }
            }
        }
    }
    if (hitSide < 0) return false;
    const int mask = tb.sideMask[hitSide];
    if (lps) {
#pragma unroll
        for (int k = 0; k < nsh; ++k) {
            T v;
            if constexpr (ROID == ROID_TRIANGLE) v = (k == 0) ? T(1) - lInt[0] - lInt[1] : (k == 1 ? lInt[0] : lInt[1]);
            else if constexpr (ROID == ROID_TETRAHEDRON) v = (k == 0) ? T(1) - lInt[0] - lInt[1] - lInt[2] : lInt[k - 1];
            else if constexpr (ROID == ROID_QUADRILATERAL) {
                const T xa = (k == 1 || k == 2) ? lInt[0] : T(1) - lInt[0];
                const T xb = (k == 2 || k == 3) ? lInt[1] : T(1) - lInt[1];
                v = xa * xb;
            } else if constexpr (ROID == ROID_PRISM) {
                const int q = k % 3;
                const T t = q == 0 ? T(1) - lInt[0] - lInt[1] : lInt[q - 1];
                v = t * ((k >= 3) ? lInt[2] : T(1) - lInt[2]);
            } else {
                const T xa = (k == 1 || k == 2 || k == 5 || k == 6) ? lInt[0] : T(1) - lInt[0];
                const T xb = (k == 2 || k == 3 || k == 6 || k == 7) ? lInt[1] : T(1) - lInt[1];
                const T xc = (k >= 4) ? lInt[2] : T(1) - lInt[2];
                v = xa * xb * xc;
            }
            up[k] = ((mask >> k) & 1) ? v : T(0);
        }
        convLen = dist<T, dim>(from, gInt);
    } else {
        // nearest side corner (GetNodeNextToCut, strict '<' keeps the first in side order)
        T mn = T(3.0e38);
        int coOut = tb.side[hitSide][0];
        const int nco = tb.sideNco[hitSide];
#pragma unroll 1
        for (int j = 0; j < nco; ++j) {
            const int co = tb.side[hitSide][j];
            T xc[3];
            pick(E.x, co, xc);
            T dd = T(0);
#pragma unroll
            for (int d = 0; d < dim; ++d) { const T x = gInt[d] - xc[d]; dd += x * x; }
            if (dd < mn) { mn = dd; coOut = co; }
        }
#pragma unroll
        for (int k = 0; k < nsh; ++k) up[k] = (k == coOut) ? T(1) : T(0);
        T xo[3];
        pick(E.x, coOut, xo);
        convLen = dist<T, dim>(from, xo);
    }
    return true;
}

// LPS on an affine element: the upwind ray gip - s vel (s >= 0) in reference
// coordinates xi(s) = xi_ip - s w, w = J^-1 vel, leaves the reference element
// through the side with the smallest crossing parameter s = num/den (ratios are
// compared by cross-multiplication, one division for the winner); the shapes
// are the P1 shapes at the exit point (its exit coordinate is set exactly on the
// side, so corners off the side get exactly zero) and the convection length is
// s |vel|. The downwind exit (velocity negated, FLOW) uses the same w with the
// opposite sign. Same point as the side-by-side ray test, in closed form.
template <int ROID, typename T>
__device__ __forceinline__ bool lps_affine(const ElemTabT<T>& tb, const T (&w)[3], const int ip, const bool down, const T vnorm,
                                           T (&up)[Ref<ROID>::nsh], T& convLen) {
    using R = Ref<ROID>;
    constexpr int dim = R::dim, nsh = R::nsh;
    constexpr bool tensor = (ROID == ROID_QUADRILATERAL || ROID == ROID_HEXAHEDRON);
    T xi[3];
#pragma unroll
    for (int a = 0; a < dim; ++a) xi[a] = T(tb.ipLoc[ip][a]);
    T bn = T(1), bd = T(0);   // best ratio bn / bd (bd = 0: none yet)
    int side = -1;            // a: lower side xi_a = 0 ; dim + a: upper side xi_a = 1 (tensor) ; dim: diagonal (simplex)
#pragma unroll
    for (int a = 0; a < dim; ++a) {
        const T wa = down ? -w[a] : w[a];   // the ray moves along -wa
        T num, den;
        int sd;
        if (wa > T(0)) { num = xi[a]; den = wa; sd = a; }
        else if (tensor && wa < T(0)) { num = T(1) - xi[a]; den = -wa; sd = dim + a; }
        else continue;
        if (side < 0 || num * bd < bn * den) { bn = num; bd = den; side = sd; }
    }
    if constexpr (!tensor) {
        T sw = T(0), sx = T(0);
#pragma unroll
        for (int a = 0; a < dim; ++a) { sw += down ? -w[a] : w[a]; sx += xi[a]; }
        if (sw < T(0)) {
            const T num = T(1) - sx, den = -sw;
            if (side < 0 || num * bd < bn * den) { bn = num; bd = den; side = dim; }
        }
    }
    if (side < 0) return false;
    const T best = bn / bd;
    T li[3];
#pragma unroll
    for (int a = 0; a < dim; ++a) {
        const T wa = down ? -w[a] : w[a];
        li[a] = xi[a] - best * wa;
        if (side == a) li[a] = T(0);
        if (tensor && side == dim + a) li[a] = T(1);
    }
#pragma unroll
    for (int k = 0; k < nsh; ++k) {
        T v;
        if constexpr (ROID == ROID_TRIANGLE) v = (k == 0) ? T(1) - li[0] - li[1] : (k == 1 ? li[0] : li[1]);
        else if constexpr (ROID == ROID_TETRAHEDRON) v = (k == 0) ? T(1) - li[0] - li[1] - li[2] : li[k - 1];
        else if constexpr (ROID == ROID_QUADRILATERAL) {
            const T xa = (k == 1 || k == 2) ? li[0] : T(1) - li[0];
            const T xb = (k == 2 || k == 3) ? li[1] : T(1) - li[1];
            v = xa * xb;
        } else {
            const T xa = (k == 1 || k == 2 || k == 5 || k == 6) ? li[0] : T(1) - li[0];
            const T xb = (k == 2 || k == 3 || k == 6 || k == 7) ? li[1] : T(1) - li[1];
            const T xc = (k >= 4) ? li[2] : T(1) - li[2];
            v = xa * xb * xc;
        }
        up[k] = v;
    }
    if constexpr (!tensor) {
        if (side == dim) up[0] = T(0);   // the diagonal side does not contain corner 0
    }
    convLen = best * vnorm;
    return true;
}

// Upwind shapes and convection length of SCVF 'ip' for IP velocity 'vel'.
// Returns false if a skewed / LPS ray finds no side.
template <int ROID, typename T>
__device__ __forceinline__ bool upwind_shapes(const int type, const Elem<ROID, T>& E, const IpGeo<T>& G, const int ip,
                                              const T* vel, const T vnorm, const bool down, const T (&wref)[3],
                                              T (&up)[Ref<ROID>::nsh], T& convLen) {
    using R = Ref<ROID>;
    constexpr int dim = R::dim, nsh = R::nsh;
    if (type == UPW_NO) {
#pragma unroll
        for (int k = 0; k < nsh; ++k) up[k] = ipN<ROID, T>(ip, k);
        convLen = T(1);
        return true;
    }
    if (type == UPW_FULL) {
        T flux = T(0);
#pragma unroll
        for (int d = 0; d < dim; ++d) flux += G.n[d] * vel[d];
        const bool f = flux > T(0);
        const int co = f ? G.from : G.to;
#pragma unroll
        for (int k = 0; k < nsh; ++k) up[k] = (k == co) ? T(1) : T(0);
        convLen = dist<T, dim>(G.gip, f ? G.xf : G.xt);
        return true;
    }
    // skewed / LPS
    if (vnorm < T(1e-14)) {
#pragma unroll
        for (int k = 0; k < nsh; ++k) up[k] = T(0);
        convLen = T(1);
        return true;
    }
    // (prisms are never affine here, so they always take the general ray test)
    if constexpr (ROID != ROID_PRISM) {
        if (type == UPW_LPS && E.affine) return lps_affine<ROID, T>(tab<ROID, T>(), wref, ip, down, vnorm, up, convLen);
    }
    return ray_upwind<ROID, T>(E, G.gip, vel, type == UPW_LPS, up, convLen);
}

// ---------------------------------------------------------------------------
// Diffusion length 1/L^2 of one SCVF (RAW / FIVEPOINT; COR uses element-wide
// minima, passed in).
// ---------------------------------------------------------------------------
template <int ROID, typename T>
__device__ __forceinline__ T diff_len_sq_inv(const int type, const Elem<ROID, T>& E, const IpGeo<T>& G,
                                            const T corMinN, const T corMinD, const T corAvgN) {
    using R = Ref<ROID>;
    constexpr int dim = R::dim, nsh = R::nsh;
    T nn = T(0);
#pragma unroll
    for (int d = 0; d < dim; ++d) nn += G.n[d] * G.n[d];
    T vf = E.vol[0], vt = E.vol[0];
#pragma unroll
    for (int k = 1; k < nsh; ++k) { vf = (k == G.from) ? E.vol[k] : vf; vt = (k == G.to) ? E.vol[k] : vt; }
    T area = T(0.5) * (vf + vt);
    area *= area;
    if (type == DL_COR) {
        if constexpr (dim == 2) return T(2.0) * corMinN / area + T(8.0) / (T(3.0) * corAvgN);
        else return T(2.0) * corMinN / area + T(8.0) * corMinD / (T(3.0) * corAvgN);
    }
    T ds = T(0);
    if constexpr (dim == 3) {
#pragma unroll
        for (int d = 0; d < 3; ++d) { const T x = G.em[d] - E.cen[d]; ds += x * x; }
    }
    // one division each: 2 nn/A + 8 ds/nn = (2 nn^2 + 8 ds A) / (A nn)   (2D: ds -> 1) and
    // 1 / (0.5 A/nn + 3 ds/8) = nn / (0.5 A + 0.375 ds nn)               (2D: ds -> nn)
    if (type == DL_FIVEPOINT) {
        if constexpr (dim == 2) return (T(2.0) * nn * nn + T(8.0) * area) / (area * nn);
        else return (T(2.0) * nn * nn + T(8.0) * ds * area) / (area * nn);
    }
    if constexpr (dim == 2) ds = nn;
    return nn / (T(0.5) * area + T(0.375) * ds * nn);
}

template <int ROID, typename T>
__device__ __forceinline__ void cor_data(const Elem<ROID, T>& E, T& minN, T& minD, T& avgN) {
    using R = Ref<ROID>;
    minN = T(3.0e38); minD = T(3.0e38); avgN = T(0);
#pragma unroll 1
    for (int ip = 0; ip < R::nip; ++ip) {
        IpGeo<T> G;
        ip_geom<ROID, T>(E, ip, G);
        T nn = T(0);
#pragma unroll
        for (int d = 0; d < R::dim; ++d) nn += G.n[d] * G.n[d];
        minN = nn < minN ? nn : minN;
        avgN += nn;
        if constexpr (R::dim == 3) {
            T ds = T(0);
#pragma unroll
            for (int d = 0; d < 3; ++d) { const T x = G.em[d] - E.cen[d]; ds += x * x; }
            minD = ds < minD ? ds : minD;
        }
    }
    avgN = avgN / T(R::nip);
}

// ---------------------------------------------------------------------------
// Per-SCVF state shared by the defect and the Jacobian
// ---------------------------------------------------------------------------
template <int ROID, typename T>
struct IpState {
    static constexpr int nsh = Ref<ROID>::nsh;
    T StdVel[3];
    T upC[nsh];         // convection upwind shapes
    T upS[nsh];         // stabilisation upwind shapes
    T dnS[nsh];         // stabilisation downwind shapes (FLOW)
    T nuL;              // nu / L_diff^2
    T nsvcl, nsvdl;     // |v| / L_up ; |v| / (L_down + L_up)
    T diag, idiag;      // the stabilisation's diagonal and its inverse (0 without stabilisation)
    bool ok;
};

// Upwind / stabilisation coefficients of one SCVF.
template <int ROID, typename T>
__device__ __forceinline__ void ip_state(const DiscParams& P, const Elem<ROID, T>& E, const IpGeo<T>& G, const int ip,
                                         const T (&u)[Ref<ROID>::b][Ref<ROID>::nsh], const T corMinN, const T corMinD, const T corAvgN,
                                         const T nuEl, IpState<ROID, T>& S) {
    using R = Ref<ROID>;
    constexpr int dim = R::dim, nsh = R::nsh;
    S.ok = true;
#pragma unroll
    for (int d = 0; d < 3; ++d) S.StdVel[d] = T(0);
#pragma unroll
    for (int sh = 0; sh < nsh; ++sh) {
        const T N = ipN<ROID, T>(ip, sh);
#pragma unroll
        for (int d = 0; d < dim; ++d) S.StdVel[d] += u[d][sh] * N;
    }
    const bool stokes = P.stokes != 0;
    T vv = T(0);
#pragma unroll
    for (int d = 0; d < dim; ++d) vv += S.StdVel[d] * S.StdVel[d];
    const T norm = Num<T>::sqrt_(vv);   // |StdVel|, also the norm of the negated (downwind) velocity
    T Lup = T(1), Ldown = T(1);
#pragma unroll
    for (int k = 0; k < nsh; ++k) { S.upS[k] = T(0); S.dnS[k] = T(0); S.upC[k] = T(0); }
    // J^-1 StdVel (reference-coordinate velocity) for the affine LPS exits
    T wref[3] = {T(0), T(0), T(0)};
    if (!stokes && E.affine && (P.stabUpwind == UPW_LPS || P.convUpwind == UPW_LPS)) {
#pragma unroll
        for (int a = 0; a < dim; ++a) {
            T s = T(0);
#pragma unroll
            for (int r = 0; r < dim; ++r) s += E.JtInv[r][a] * S.StdVel[r];
            wref[a] = s;
        }
    }
    if (!stokes) {
        // the stabilisation's upwind (and downwind for FLOW) first, then the
        // convection's own upwind when it is a different object
        const int nUp = (P.stab == STAB_FLOW ? 2 : 1) + (P.sameUpwind ? 0 : 1);
#pragma unroll 1
        for (int w = 0; w < nUp; ++w) {
            const bool isDown = (w == 1 && P.stab == STAB_FLOW);
            const bool isConv = (w == nUp - 1 && !P.sameUpwind);
            T vel[3];
#pragma unroll
            for (int d = 0; d < 3; ++d) vel[d] = isDown ? S.StdVel[d] * T(-1) : S.StdVel[d];
            T sh[nsh], L;
            S.ok &= upwind_shapes<ROID, T>(isConv ? P.convUpwind : P.stabUpwind, E, G, ip, vel, norm, isDown, wref, sh, L);
#pragma unroll
            for (int k = 0; k < nsh; ++k) {
                if (isConv) S.upC[k] = sh[k];
                else if (isDown) S.dnS[k] = sh[k];
                else S.upS[k] = sh[k];
            }
            if (!isConv) { if (isDown) Ldown = L; else Lup = L; }
        }
        if (P.sameUpwind) {
#pragma unroll
            for (int k = 0; k < nsh; ++k) S.upC[k] = S.upS[k];
        }
    }
    S.nuL = T(0); S.nsvcl = T(0); S.nsvdl = T(0); S.diag = T(1); S.idiag = T(0);
    if (P.stab == STAB_WITHOUT) return;
    const T Linv = diff_len_sq_inv<ROID, T>(P.diffLen, E, G, corMinN, corMinD, corAvgN);
    S.nuL = nuEl * Linv;
    if (!stokes) {
        S.nsvcl = norm / Lup;
        if (P.stab == STAB_FLOW) S.nsvdl = norm / (Ldown + Lup);
    }
    S.diag = S.nuL;
    if (P.transient) S.diag += T(1) / T(P.dt);
    if (!stokes) S.diag += S.nsvcl;
    S.idiag = T(1) / S.diag;
}

// peclet_blend weight (navier_stokes_fv1.cpp:871-892); blends UpwindVel in place
template <int ROID, typename T>
__device__ __forceinline__ T peclet_blend(const IpGeo<T>& G, const T* StdVel, T nu, T* UpwindVel) {
    constexpr int dim = Ref<ROID>::dim;
    T vn = T(0), nn = T(0);
#pragma unroll
    for (int d = 0; d < dim; ++d) { vn += StdVel[d] * G.n[d]; nn += G.n[d] * G.n[d]; }
    const T Pe = vn / nn * dist<T, dim>(G.xt, G.xf) / nu;
    const T Pe2 = Pe * Pe;
    const T w = Pe2 / (T(5.0) + Pe2);
#pragma unroll
    for (int d = 0; d < dim; ++d) UpwindVel[d] = w * UpwindVel[d] + (T(1) - w) * StdVel[d];
    return w;
}

// ---------------------------------------------------------------------------
// Local stiffness defect of one element: every SCVF flux is handed to the sink
// with sink.add(corner, fct, value) (+ at from, - at to).
// uo is read only when P.transient (pass any array otherwise).
// Returns false if an upwind ray found no side.
// ---------------------------------------------------------------------------
// velocity and pressure gradients at the integration point of SCVF ip: local
// gradients first, then one J^-T (grad_k = J^-T lgrad_k, so
// sum_k u_k grad_k = J^-T sum_k u_k lgrad_k)
template <int ROID, typename T>
__device__ __forceinline__ void ip_gradients(const IpGeo<T>& G, const int ip, const T (&u)[Ref<ROID>::b][Ref<ROID>::nsh],
                                             T (&gradVel)[3][3], T (&gradP)[3]) {
    using R = Ref<ROID>;
    constexpr int dim = R::dim, nsh = R::nsh;
    const auto& tb = tab<ROID, T>();
    T gl[4][3];
#pragma unroll
    for (int f = 0; f <= dim; ++f)
#pragma unroll
        for (int c = 0; c < dim; ++c) {
            T acc = T(0);
#pragma unroll
            for (int sh = 0; sh < nsh; ++sh) acc += u[f][sh] * T(tb.ipLGrad[ip][sh][c]);
            gl[f][c] = acc;
        }
#pragma unroll
    for (int f = 0; f <= dim; ++f)
#pragma unroll
        for (int d2 = 0; d2 < dim; ++d2) {
            T acc = T(0);
#pragma unroll
            for (int c = 0; c < dim; ++c) acc += G.JtInv[d2][c] * gl[f][c];
            if (f < dim) gradVel[f][d2] = acc;
            else gradP[d2] = acc;
        }
}

// The stabilised velocity of SCVF ip (stab_vel of the diagonal FIELDS / FLOW
// update, stabilization.cpp:163-241, 486-588; the interpolated velocity without
// stabilisation, :805-850). upShared: the stabilisation's upwind velocity
// sum_k upS_k u_k when already known (the convection shares the upwind), else null.
template <int ROID, typename T>
__device__ __forceinline__ void stab_velocity(const DiscParams& P, const IpState<ROID, T>& S, const int ip,
                                              const T (&u)[Ref<ROID>::b][Ref<ROID>::nsh], const T (&uo)[Ref<ROID>::dim][Ref<ROID>::nsh],
                                              const T (&gradVel)[3][3], const T (&gradP)[3], const T rho, const T* upShared,
                                              T (&stabVel)[3]) {
    using R = Ref<ROID>;
    constexpr int dim = R::dim, nsh = R::nsh;
    if (P.stab == STAB_WITHOUT) {
#pragma unroll
        for (int d = 0; d < dim; ++d) stabVel[d] = S.StdVel[d];
        return;
    }
    T trace = T(0);
#pragma unroll
    for (int d = 0; d < dim; ++d) trace += gradVel[d][d];
    const T idiag = S.idiag, irho = T(1) / rho;
#pragma unroll
    for (int d = 0; d < dim; ++d) {
        T rhs = T(0);
        if (P.hasSource) rhs = T(P.src[d]);
        if (P.transient) {
            T oldIPVel = T(0);
#pragma unroll
            for (int sh = 0; sh < nsh; ++sh) oldIPVel += ipN<ROID, T>(ip, sh) * uo[d][sh];
            rhs += oldIPVel / T(P.dt);
        }
        rhs += S.nuL * S.StdVel[d];
        if (!P.stokes) {
            T UpS = T(0), DnS = T(0);
            if (upShared) UpS = upShared[d];
#pragma unroll
            for (int sh = 0; sh < nsh; ++sh) {
                if (!upShared) UpS += S.upS[sh] * u[d][sh];
                if (P.stab == STAB_FLOW) DnS += S.dnS[sh] * u[d][sh];
            }
            rhs += S.nsvcl * UpS;
            if (P.stab == STAB_FLOW) rhs += S.nsvdl * (DnS - UpS);
        }
        if (P.stab == STAB_FLOW) {
            T cross = T(0);
#pragma unroll
            for (int d2 = 0; d2 < dim; ++d2)
                if (d2 != d) cross += S.StdVel[d2] * gradVel[d][d2];
            rhs += S.StdVel[d] * (trace - gradVel[d][d]) - cross;
        }
        rhs -= gradP[d] * irho;
        stabVel[d] = rhs * idiag;
    }
}

template <int ROID, typename T, class DSink>
__device__ __forceinline__ void scvf_def_A(const DiscParams& P, const Elem<ROID, T>& E, const IpGeo<T>& G, const IpState<ROID, T>& S,
                                           const int ip, const T (&u)[Ref<ROID>::b][Ref<ROID>::nsh],
                                           const T (&uo)[Ref<ROID>::dim][Ref<ROID>::nsh], DSink& sink, const T nu) {
    using R = Ref<ROID>;
    constexpr int dim = R::dim, nsh = R::nsh, Pc = dim;
    const T rho = T(P.rho);
    T gradVel[3][3], gradP[3];
    ip_gradients<ROID, T>(G, ip, u, gradVel, gradP);
    // diffusion
    T flux[3];
#pragma unroll
    for (int d1 = 0; d1 < dim; ++d1) {
        T s = T(0);
#pragma unroll
        for (int d2 = 0; d2 < dim; ++d2) s += gradVel[d1][d2] * G.n[d2];
        if (!P.laplace) {
#pragma unroll
            for (int d2 = 0; d2 < dim; ++d2) s += gradVel[d2][d1] * G.n[d2];
        }
        flux[d1] = s * (T(-1.0) * nu * rho);
    }
    // the convection's upwind velocity (before blending); with a shared upwind object
    // it is also the stabilisation's
    T UpConv[3] = {T(0), T(0), T(0)};
    const bool upwindConv = !P.stokes && !P.pac;
    if (upwindConv) {
#pragma unroll
        for (int d = 0; d < dim; ++d) {
            T s = T(0);
#pragma unroll
            for (int sh = 0; sh < nsh; ++sh) s += S.upC[sh] * u[d][sh];
            UpConv[d] = s;
        }
    }
    T stabVel[3];
    stab_velocity<ROID, T>(P, S, ip, u, uo, gradVel, gradP, rho, (upwindConv && P.sameUpwind) ? UpConv : nullptr, stabVel);
    // convection: the upwind velocity, or the stabilised velocity with PAC
    // (navier_stokes_fv1.cpp:707-712)
    if (!P.stokes) {
        T UpwindVel[3];
#pragma unroll
        for (int d = 0; d < dim; ++d) UpwindVel[d] = P.pac ? stabVel[d] : UpConv[d];
        if (P.peclet) peclet_blend<ROID, T>(G, S.StdVel, nu, UpwindVel);
        T prod = T(0);
#pragma unroll
        for (int d = 0; d < dim; ++d) prod += S.StdVel[d] * G.n[d];
        prod *= rho;
#pragma unroll
        for (int d1 = 0; d1 < dim; ++d1) flux[d1] += UpwindVel[d1] * prod;
    }
    // pressure
    T pressure = T(0);
#pragma unroll
    for (int sh = 0; sh < nsh; ++sh) pressure += ipN<ROID, T>(ip, sh) * u[Pc][sh];
#pragma unroll
    for (int d1 = 0; d1 < dim; ++d1) flux[d1] += pressure * G.n[d1];
    // continuity with the stabilised velocity
    T contFlux = T(0);
#pragma unroll
    for (int d = 0; d < dim; ++d) contFlux += stabVel[d] * G.n[d];
    contFlux *= rho;
#pragma unroll
    for (int d1 = 0; d1 < dim; ++d1) { sink.add(G.from, d1, flux[d1]); sink.add(G.to, d1, flip_sign(flux[d1])); }
    sink.add(G.from, Pc, contFlux);
    sink.add(G.to, Pc, flip_sign(contFlux));
}

template <int ROID, typename T, class DSink>
__device__ __forceinline__ bool elem_def_A(const DiscParams& P, const Elem<ROID, T>& E, const T (&u)[Ref<ROID>::b][Ref<ROID>::nsh],
                                           const T (&uo)[Ref<ROID>::dim][Ref<ROID>::nsh], DSink& sink, const T nu) {
    using R = Ref<ROID>;
    T corMinN = T(0), corMinD = T(0), corAvgN = T(1);
    if (P.stab != STAB_WITHOUT && P.diffLen == DL_COR) cor_data<ROID, T>(E, corMinN, corMinD, corAvgN);
    bool ok = true;
#pragma unroll 1
    for (int ip = 0; ip < R::nip; ++ip) {
        IpGeo<T> G;
        ip_geom<ROID, T>(E, ip, G);
        IpState<ROID, T> S;
        ip_state<ROID, T>(P, E, G, ip, u, corMinN, corMinD, corAvgN, nu, S);
        ok &= S.ok;
        scvf_def_A<ROID, T>(P, E, G, S, ip, u, uo, sink, nu);
    }
    return ok;
}

// ---------------------------------------------------------------------------
// Local stiffness Jacobian: for every SCVF ip and column corner k the b x b
// block B is added to row corner 'from' and subtracted from row corner 'to'
// through the sink (sink.add(i, k, B, plus)); 'scale' multiplies B (dt for the
// implicit-Euler Jacobian M + dt dA/du).
// ---------------------------------------------------------------------------
// PAC: compile the stabilisation-as-upwind branches (set_pac_upwind); without it
// those branches cost registers in every configuration
// Per-SCVF factors of the Jacobian blocks (everything the block of one column
// corner needs besides the reference-element tables).
template <int ROID, typename T>
struct JacIp {
    static constexpr int nsh = Ref<ROID>::nsh;
    int from, to;
    T n[3], JtInv[3][3], StdVel[3], UpwindVel[3];
    T upC[nsh], upS[nsh], dnS[nsh];
    T nuL, nsvcl, nsvdl, idiag;
    T pw, ppe, w, riVn;
};

template <int ROID, typename T, bool PAC>
__device__ __forceinline__ void jac_ip_factors(const DiscParams& P, const IpGeo<T>& G, const IpState<ROID, T>& S, const int ip,
                                               const T (&u)[Ref<ROID>::b][Ref<ROID>::nsh],
                                               const T (&uo)[Ref<ROID>::dim][Ref<ROID>::nsh], const T nu, JacIp<ROID, T>& J) {
    using R = Ref<ROID>;
    constexpr int dim = R::dim, nsh = R::nsh;
    const T rho = T(P.rho);
    T w = T(1), prod = T(0), Vn = T(0);
#pragma unroll
    for (int d = 0; d < 3; ++d) J.UpwindVel[d] = T(0);
#pragma unroll
    for (int d = 0; d < dim; ++d) Vn += S.StdVel[d] * G.n[d];
    const bool pac = PAC && !P.stokes && P.pac;
    const bool fullNewton = !P.stokes && P.fullNewton != 0.0;
    if (!P.stokes) {
        if (pac) {
            // the stabilised velocity is the upwind velocity (navier_stokes_fv1.cpp:382-384); the
            // Jacobian needs it only for the exact-Jacobian terms
            if (fullNewton) {
                T gradVel[3][3], gradP[3];
                ip_gradients<ROID, T>(G, ip, u, gradVel, gradP);
                stab_velocity<ROID, T>(P, S, ip, u, uo, gradVel, gradP, rho, nullptr, J.UpwindVel);
            }
        } else {
#pragma unroll
            for (int d = 0; d < dim; ++d) {
                T s = T(0);
#pragma unroll
                for (int sh = 0; sh < nsh; ++sh) s += S.upC[sh] * u[d][sh];
                J.UpwindVel[d] = s;
            }
        }
        if (P.peclet) w = peclet_blend<ROID, T>(G, S.StdVel, nu, J.UpwindVel);
        prod = Vn * rho;
    }
    J.from = G.from; J.to = G.to;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        J.n[d] = G.n[d]; J.StdVel[d] = S.StdVel[d];
#pragma unroll
        for (int c = 0; c < 3; ++c) J.JtInv[d][c] = G.JtInv[d][c];
    }
#pragma unroll
    for (int k = 0; k < nsh; ++k) { J.upC[k] = S.upC[k]; J.upS[k] = S.upS[k]; J.dnS[k] = S.dnS[k]; }
    J.nuL = S.nuL; J.nsvcl = S.nsvcl; J.nsvdl = S.nsvdl; J.idiag = S.idiag;
    J.pw = prod * w; J.ppe = prod * (T(1) - w); J.w = w;
    J.riVn = rho * S.idiag * Vn;
}

// The b x b block of one SCVF and one column corner k (added to row 'from',
// subtracted from row 'to' by the caller), from the SCVF's factors Jf (JacIp or
// any type with its scalar members) and the column's inputs: lg = the reference
// gradient and N the value of shape k at the SCVF's ip, upCk / upSk / dnSk its
// convection-upwind, stabilisation-upwind and downwind shapes.
template <int ROID, typename T, bool PAC, class F>
__device__ __forceinline__ void jac_block_col(const DiscParams& P, const F& Jf, const T (&lg)[3], const T N, const T upCk,
                                              const T upSk, const T dnSk, const T nu, T (&B)[Ref<ROID>::b][Ref<ROID>::b]) {
    using R = Ref<ROID>;
    constexpr int dim = R::dim, Pc = dim;
    const T rho = T(P.rho), irho = T(1) / rho;
    const T mnr = T(-1.0) * nu * rho;
    const bool pac = PAC && !P.stokes && P.pac;
    const bool fullNewton = !P.stokes && P.fullNewton != 0.0;
    const T idiag = Jf.idiag, ri = rho * idiag, riVn = Jf.riVn, pw = Jf.pw, ppe = Jf.ppe, w = Jf.w, ppr = -ri * irho;
    const T fr = T(P.fullNewton) * rho;
    T mn[3], rin[3], nrho[3];
#pragma unroll
    for (int d = 0; d < dim; ++d) { mn[d] = mnr * Jf.n[d]; rin[d] = ri * Jf.n[d]; nrho[d] = Jf.n[d] * rho; }
    const auto& S = Jf;
    const T (&UpwindVel)[3] = Jf.UpwindVel;
    struct { const T (&n)[3]; const T (&JtInv)[3][3]; } G{Jf.n, Jf.JtInv};
    {
        {
            T g[3];
#pragma unroll
            for (int r = 0; r < dim; ++r) {
                T sacc = T(0);
#pragma unroll
                for (int c = 0; c < dim; ++c) sacc += G.JtInv[r][c] * lg[c];
                g[r] = sacc;
            }
            T gn = T(0), Vg = T(0);
#pragma unroll
            for (int d = 0; d < dim; ++d) { gn += g[d] * G.n[d]; Vg += S.StdVel[d] * g[d]; }
            // diffusion: -nu rho ((g.n) I + g (x) n)
            T dd = mnr * gn;
            // convection (fixpoint part) on the diagonal: the upwind shape, the Peclet blend
            if (!P.stokes) {
                if (!pac) dd += upCk * pw;
                if (P.peclet) dd += ppe * N;
            }
#pragma unroll
            for (int d1 = 0; d1 < dim; ++d1)
#pragma unroll
                for (int d2 = 0; d2 < dim; ++d2) {
                    T v = P.laplace ? T(0) : g[d1] * mn[d2];
                    if (d1 == d2) v += dd;
                    B[d1][d2] = v;
                }
            if (fullNewton) {
#pragma unroll
                for (int d2 = 0; d2 < dim; ++d2) {
                    // upwind used as upwind (:521-534, the factor is not applied there) and the Peclet blend
                    T pv = pac ? T(0) : w * upCk * nrho[d2];
                    if (P.peclet) pv += (T(1) - w) * N * nrho[d2];
#pragma unroll
                    for (int d1 = 0; d1 < dim; ++d1) B[d1][d2] += pv * UpwindVel[d1];
                }
            }
            // pressure
#pragma unroll
            for (int d1 = 0; d1 < dim; ++d1) B[d1][Pc] = N * G.n[d1];
            // continuity: the stabilised-velocity shapes of corner k (diagonal branch)
            T Sk = T(0);
            if (P.stab == STAB_WITHOUT) {
#pragma unroll
                for (int d1 = 0; d1 < dim; ++d1) B[Pc][d1] = N * nrho[d1];
                B[Pc][Pc] = T(0);
            } else {
                Sk = S.nuL * N;
                if (!P.stokes) {
                    Sk += S.nsvcl * upSk;
                    if (P.stab == STAB_FLOW) Sk += S.nsvdl * (dnSk - upSk);
                }
                if (P.stab == STAB_FLOW) {
                    const T sv = Sk - Vg;
#pragma unroll
                    for (int d1 = 0; d1 < dim; ++d1) B[Pc][d1] = sv * rin[d1] + riVn * g[d1];
                } else {
#pragma unroll
                    for (int d1 = 0; d1 < dim; ++d1) B[Pc][d1] = Sk * rin[d1];
                }
                B[Pc][Pc] = gn * ppr;
            }
            if (pac) {
                // the stabilisation's shapes stab_shape_vel(ip, a, c, k) = V[a][c] and
                // stab_shape_p(ip, a, k) = Q[a] (diagonal branch; without stabilisation the
                // interpolation shape)
                T V[3][3], Q[3];
                const bool flow = P.stab == STAB_FLOW, without = P.stab == STAB_WITHOUT;
#pragma unroll
                for (int a = 0; a < dim; ++a) {
#pragma unroll
                    for (int c = 0; c < dim; ++c) {
                        T v;
                        if (without) v = (a == c) ? N : T(0);
                        else if (flow) v = ((a == c) ? (Sk - Vg + S.StdVel[a] * g[a]) : S.StdVel[a] * g[c]) * idiag;
                        else v = (a == c) ? Sk * idiag : T(0);
                        V[a][c] = v;
                    }
                    Q[a] = without ? T(0) : T(-1) * g[a] * irho * idiag;
                }
                // stabilisation used as upwind, fixpoint part (navier_stokes_fv1.cpp:398-427)
#pragma unroll
                for (int d1 = 0; d1 < dim; ++d1) {
#pragma unroll
                    for (int d2 = 0; d2 < dim; ++d2)
                        if (flow || d1 == d2) B[d1][d2] += pw * V[d1][d2];
                    B[d1][Pc] += pw * Q[d1];
                }
                if (fullNewton) {
                    // exact-Jacobian part (:477-518); without connected velocity components the
                    // (d1, d1) shape serves every column d2 and the blend weight is not applied
                    T pp = T(0);
#pragma unroll
                    for (int q = 0; q < dim; ++q) pp += Q[q] * G.n[q];
#pragma unroll
                    for (int d1 = 0; d1 < dim; ++d1) {
#pragma unroll
                        for (int d2 = 0; d2 < dim; ++d2) {
                            T pv = T(0);
                            if (flow) {
#pragma unroll
                                for (int q = 0; q < dim; ++q) pv += w * V[q][d2] * G.n[q];
                            } else {
                                pv = V[d1][d1] * G.n[d1];
                            }
                            B[d1][d2] += pv * fr * UpwindVel[d1];
                        }
                        B[d1][Pc] += pp * fr * UpwindVel[d1];
                    }
                }
            }
        }
    }
}

// The block of SCVF ip and column corner k from the SCVF's JacIp and the
// reference-element tables.
template <int ROID, typename T, bool PAC>
__device__ __forceinline__ void jac_block(const DiscParams& P, const JacIp<ROID, T>& Jf, const int ip, const int k, const T nu,
                                          T (&B)[Ref<ROID>::b][Ref<ROID>::b]) {
    const auto& tb = tab<ROID, T>();
    const T lg[3] = {T(tb.ipLGrad[ip][k][0]), T(tb.ipLGrad[ip][k][1]), Ref<ROID>::dim == 3 ? T(tb.ipLGrad[ip][k][2]) : T(0)};
    jac_block_col<ROID, T, PAC>(P, Jf, lg, ipN<ROID, T>(ip, k), Jf.upC[k], Jf.upS[k], Jf.dnS[k], nu, B);
}

template <int ROID, typename T, bool PAC, class Sink>
__device__ __forceinline__ void scvf_jac_A(const DiscParams& P, const IpGeo<T>& G, const IpState<ROID, T>& S,
                                           const int ip, const T (&u)[Ref<ROID>::b][Ref<ROID>::nsh],
                                           const T (&uo)[Ref<ROID>::dim][Ref<ROID>::nsh], const T scale, Sink& sink, const T nu) {
    using R = Ref<ROID>;
    constexpr int nsh = R::nsh, b = R::b;
    JacIp<ROID, T> Jf;
    jac_ip_factors<ROID, T, PAC>(P, G, S, ip, u, uo, nu, Jf);
#pragma unroll
    for (int k = 0; k < nsh; ++k) {
        T B[b][b];
        jac_block<ROID, T, PAC>(P, Jf, ip, k, nu, B);
        if (scale != T(1)) {
#pragma unroll
            for (int r = 0; r < b; ++r)
#pragma unroll
                for (int c = 0; c < b; ++c) B[r][c] *= scale;
        }
        sink.add(Jf.from, k, B, true);
        sink.add(Jf.to, k, B, false);
    }
}

template <int ROID, typename T, bool PAC, class Sink>
__device__ __forceinline__ bool elem_jac_A(const DiscParams& P, const Elem<ROID, T>& E, const T (&u)[Ref<ROID>::b][Ref<ROID>::nsh],
                                           const T (&uo)[Ref<ROID>::dim][Ref<ROID>::nsh], const T scale, Sink& sink, const T nu) {
    using R = Ref<ROID>;
    T corMinN = T(0), corMinD = T(0), corAvgN = T(1);
    if (P.stab != STAB_WITHOUT && P.diffLen == DL_COR) cor_data<ROID, T>(E, corMinN, corMinD, corAvgN);
    bool ok = true;
#pragma unroll 1
    for (int ip = 0; ip < R::nip; ++ip) {
        IpGeo<T> G;
        ip_geom<ROID, T>(E, ip, G);
        IpState<ROID, T> S;
        ip_state<ROID, T>(P, E, G, ip, u, corMinN, corMinD, corAvgN, nu, S);
        ok &= S.ok;
        scvf_jac_A<ROID, T, PAC>(P, G, S, ip, u, uo, scale, sink, nu);
    }
    return ok;
}

// Defect and Jacobian of one element at the same state in one pass: the
// geometry, upwind shapes and stabilisation of every SCVF are computed once and
// feed both (the reference evaluates them separately in add_def_A_elem and
// add_jac_A_elem, navier_stokes_fv1.cpp:296-309, 645-659). 'jscale' multiplies
// the Jacobian blocks (dt for the implicit-Euler Jacobian); the defect sink
// applies its own scaling.
template <int ROID, typename T, bool PAC, class DSink, class JSink>
__device__ __forceinline__ bool elem_def_jac_A(const DiscParams& P, const Elem<ROID, T>& E, const T (&u)[Ref<ROID>::b][Ref<ROID>::nsh],
                                               const T (&uo)[Ref<ROID>::dim][Ref<ROID>::nsh], DSink& dsink, const T jscale,
                                               JSink& jsink, const T nu) {
    using R = Ref<ROID>;
    T corMinN = T(0), corMinD = T(0), corAvgN = T(1);
    if (P.stab != STAB_WITHOUT && P.diffLen == DL_COR) cor_data<ROID, T>(E, corMinN, corMinD, corAvgN);
    bool ok = true;
#pragma unroll 1
    for (int ip = 0; ip < R::nip; ++ip) {
        IpGeo<T> G;
        ip_geom<ROID, T>(E, ip, G);
        IpState<ROID, T> S;
        ip_state<ROID, T>(P, E, G, ip, u, corMinN, corMinD, corAvgN, nu, S);
        ok &= S.ok;
        scvf_def_A<ROID, T>(P, E, G, S, ip, u, uo, dsink, nu);
        scvf_jac_A<ROID, T, PAC>(P, G, S, ip, u, uo, jscale, jsink, nu);
    }
    return ok;
}

}  // namespace nsfv1
