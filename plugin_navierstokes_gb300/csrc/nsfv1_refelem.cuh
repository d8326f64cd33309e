// Reference-element tables of the FV1 elements of this path, as compile-time
// constants for the sm_103a kernels (all loops over corners / SCVFs / sides
// are unrolled, so every lookup below folds to an immediate).
//
// Numbering follows ugcore's ReferenceObjectID and reference elements
// (triangle, quadrilateral, tetrahedron, hexahedron; corners of the unit
// simplex / unit cube, edges and sides in reference order). SCVF i belongs to
// edge i with from = edge corner 0 and to = edge corner 1, as used by
// navier_stokes_fv1.cpp:342-343 (J(d1, scvf.from(), ...) / scvf.to()).
// 3D SCVF corners are {edge midpoint, centre of face F1, element centre,
// centre of face F2}; the face pair is ordered so that the SCVF normal
// 0.5 (c2 - c0) x (c3 - c1) points from -> to (global_corner(0) = edge
// midpoint and global_corner(2) = element centre, diffusion_length.h:79-82).
#pragma once
#include "nsfv1_params.h"

#define NSFV1_HD __host__ __device__ __forceinline__

namespace nsfv1 {

template <int ROID> struct Ref;

template <> struct Ref<ROID_TRIANGLE> {
    static constexpr int dim = 2, nsh = 3, nip = 3, nside = 3, b = 3;
    NSFV1_HD static constexpr double co(int c, int d) {
        return c == 1 ? (d == 0 ? 1.0 : 0.0) : c == 2 ? (d == 1 ? 1.0 : 0.0) : 0.0;
    }
    NSFV1_HD static constexpr int edge(int e, int k) { return k == 0 ? e : (e + 1) % 3; }
    NSFV1_HD static constexpr int side_nco(int) { return 2; }
    NSFV1_HD static constexpr int side(int s, int j) { return edge(s, j); }
    NSFV1_HD static constexpr int edge_face(int, int) { return 0; }
    NSFV1_HD static constexpr int scv_tab(int, int) { return 0; }
};

template <> struct Ref<ROID_QUADRILATERAL> {
    static constexpr int dim = 2, nsh = 4, nip = 4, nside = 4, b = 3;
    NSFV1_HD static constexpr double co(int c, int d) {
        return d == 0 ? ((c == 1 || c == 2) ? 1.0 : 0.0) : ((c == 2 || c == 3) ? 1.0 : 0.0);
    }
    NSFV1_HD static constexpr int edge(int e, int k) { return k == 0 ? e : (e + 1) % 4; }
    NSFV1_HD static constexpr int side_nco(int) { return 2; }
    NSFV1_HD static constexpr int side(int s, int j) { return edge(s, j); }
    NSFV1_HD static constexpr int edge_face(int, int) { return 0; }
    NSFV1_HD static constexpr int scv_tab(int, int) { return 0; }
};

template <> struct Ref<ROID_TETRAHEDRON> {
    static constexpr int dim = 3, nsh = 4, nip = 6, nside = 4, b = 4;
    NSFV1_HD static constexpr double co(int c, int d) { return (c >= 1 && c - 1 == d) ? 1.0 : 0.0; }
    NSFV1_HD static constexpr int edge(int e, int k) {
        return e == 0 ? (k ? 1 : 0) : e == 1 ? (k ? 2 : 1) : e == 2 ? (k ? 0 : 2)
             : e == 3 ? (k ? 3 : 0) : e == 4 ? (k ? 3 : 1) : (k ? 3 : 2);
    }
    NSFV1_HD static constexpr int side_nco(int) { return 3; }
    NSFV1_HD static constexpr int side(int s, int j) {
        // {0,2,1}, {0,1,3}, {1,2,3}, {0,3,2}
        return s == 0 ? (j == 0 ? 0 : j == 1 ? 2 : 1) : s == 1 ? (j == 0 ? 0 : j == 1 ? 1 : 3)
             : s == 2 ? (j == 0 ? 1 : j == 1 ? 2 : 3) : (j == 0 ? 0 : j == 1 ? 3 : 2);
    }
    NSFV1_HD static constexpr int edge_face(int e, int k) {
        // (0,1) (0,2) (0,3) (1,3) (2,1) (3,2)
        return e == 0 ? (k ? 1 : 0) : e == 1 ? (k ? 2 : 0) : e == 2 ? (k ? 3 : 0)
             : e == 3 ? (k ? 3 : 1) : e == 4 ? (k ? 1 : 2) : (k ? 2 : 3);
    }
    // per corner a: {edge to nb0, face(a,nb0,nb1), edge to nb1, edge to nb2, face(a,nb0,nb2), face(a,nb1,nb2)}
    NSFV1_HD static constexpr int scv_tab(int a, int k) {
        constexpr int t[4][6] = {{0, 0, 2, 3, 1, 3}, {0, 0, 1, 4, 1, 2}, {1, 0, 2, 5, 2, 3}, {3, 1, 4, 5, 3, 2}};
        return t[a][k];
    }
};

template <> struct Ref<ROID_HEXAHEDRON> {
    static constexpr int dim = 3, nsh = 8, nip = 12, nside = 6, b = 4;
    NSFV1_HD static constexpr double co(int c, int d) {
        return d == 0 ? ((c == 1 || c == 2 || c == 5 || c == 6) ? 1.0 : 0.0)
             : d == 1 ? ((c == 2 || c == 3 || c == 6 || c == 7) ? 1.0 : 0.0)
                      : (c >= 4 ? 1.0 : 0.0);
    }
    NSFV1_HD static constexpr int edge(int e, int k) {
        constexpr int t[12][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}, {0, 4}, {1, 5}, {2, 6}, {3, 7}, {4, 5}, {5, 6}, {6, 7}, {7, 4}};
        return t[e][k];
    }
    NSFV1_HD static constexpr int side_nco(int) { return 4; }
    NSFV1_HD static constexpr int side(int s, int j) {
        constexpr int t[6][4] = {{0, 3, 2, 1}, {0, 1, 5, 4}, {1, 2, 6, 5}, {2, 3, 7, 6}, {0, 4, 7, 3}, {4, 5, 6, 7}};
        return t[s][j];
    }
    NSFV1_HD static constexpr int edge_face(int e, int k) {
        constexpr int t[12][2] = {{0, 1}, {0, 2}, {0, 3}, {0, 4}, {1, 4}, {2, 1}, {3, 2}, {4, 3}, {1, 5}, {2, 5}, {3, 5}, {4, 5}};
        return t[e][k];
    }
    NSFV1_HD static constexpr int scv_tab(int a, int k) {
        constexpr int t[8][6] = {{0, 0, 3, 4, 1, 4}, {0, 0, 1, 5, 1, 2}, {1, 0, 2, 6, 2, 3}, {2, 0, 3, 7, 3, 4},
                                 {4, 1, 8, 11, 4, 5}, {5, 1, 8, 9, 2, 5}, {6, 2, 9, 10, 3, 5}, {7, 3, 10, 11, 4, 5}};
        return t[a][k];
    }
};

// Prism: triangle (0, 1, 2) at z = 0 extruded to (3, 4, 5) at z = 1; sides 0 and 4
// are the triangles, 1..3 the quadrilaterals (outward corner order as the others).
template <> struct Ref<ROID_PRISM> {
    static constexpr int dim = 3, nsh = 6, nip = 9, nside = 5, b = 4;
    NSFV1_HD static constexpr double co(int c, int d) {
        return d == 0 ? ((c == 1 || c == 4) ? 1.0 : 0.0) : d == 1 ? ((c == 2 || c == 5) ? 1.0 : 0.0) : (c >= 3 ? 1.0 : 0.0);
    }
    NSFV1_HD static constexpr int edge(int e, int k) {
        constexpr int t[9][2] = {{0, 1}, {1, 2}, {2, 0}, {0, 3}, {1, 4}, {2, 5}, {3, 4}, {4, 5}, {5, 3}};
        return t[e][k];
    }
    NSFV1_HD static constexpr int side_nco(int s) { return (s == 0 || s == 4) ? 3 : 4; }
    NSFV1_HD static constexpr int side(int s, int j) {
        constexpr int t[5][4] = {{0, 2, 1, 0}, {0, 1, 4, 3}, {1, 2, 5, 4}, {2, 0, 3, 5}, {3, 4, 5, 3}};
        return t[s][j];
    }
    NSFV1_HD static constexpr int edge_face(int e, int k) {
        constexpr int t[9][2] = {{0, 1}, {0, 2}, {0, 3}, {1, 3}, {2, 1}, {3, 2}, {1, 4}, {2, 4}, {3, 4}};
        return t[e][k];
    }
    NSFV1_HD static constexpr int scv_tab(int a, int k) {
        constexpr int t[6][6] = {{0, 0, 2, 3, 1, 3}, {0, 0, 1, 4, 1, 2}, {1, 0, 2, 5, 2, 3},
                                 {3, 1, 6, 8, 3, 4}, {4, 1, 6, 7, 2, 4}, {5, 2, 7, 8, 3, 4}};
        return t[a][k];
    }
};

// ---- derived compile-time quantities --------------------------------------

// local (reference) coordinates of the element centre, face centres, edge mids,
// computed as the mean of the reference corners (same formula as the geometry)
template <class R> NSFV1_HD constexpr double loc_center(int d) {
    double s = 0.0;
    for (int c = 0; c < R::nsh; ++c) s += R::co(c, d);
    return s * (1.0 / R::nsh);
}
template <class R> NSFV1_HD constexpr double loc_face(int f, int d) {
    double s = 0.0;
    for (int j = 0; j < R::side_nco(f); ++j) s += R::co(R::side(f, j), d);
    return s * (1.0 / R::side_nco(f));
}
template <class R> NSFV1_HD constexpr double loc_edge(int e, int d) {
    return 0.5 * (R::co(R::edge(e, 0), d) + R::co(R::edge(e, 1), d));
}
// local SCVF integration point = mean of the local SCVF corners
template <class R> NSFV1_HD constexpr double loc_ip(int ip, int d) {
    if (R::dim == 2) return (loc_edge<R>(ip, d) + loc_center<R>(d)) * 0.5;
    return (loc_edge<R>(ip, d) + loc_face<R>(R::edge_face(ip, 0), d) + loc_center<R>(d) + loc_face<R>(R::edge_face(ip, 1), d)) * 0.25;
}

// P1 Lagrange shapes and local gradients at a local point
template <int ROID> NSFV1_HD constexpr double p1_shape(int k, double a, double b, double c) {
    if (ROID == ROID_TRIANGLE) return k == 0 ? 1.0 - a - b : k == 1 ? a : b;
    if (ROID == ROID_QUADRILATERAL)
        return k == 0 ? (1.0 - a) * (1.0 - b) : k == 1 ? a * (1.0 - b) : k == 2 ? a * b : (1.0 - a) * b;
    if (ROID == ROID_TETRAHEDRON) return k == 0 ? 1.0 - a - b - c : k == 1 ? a : k == 2 ? b : c;
    if (ROID == ROID_PRISM) {
        const double t = k == 0 || k == 3 ? 1.0 - a - b : (k == 1 || k == 4) ? a : b;
        return t * (k >= 3 ? c : 1.0 - c);
    }
    // hexahedron
    return k == 0 ? (1.0 - a) * (1.0 - b) * (1.0 - c) : k == 1 ? a * (1.0 - b) * (1.0 - c)
         : k == 2 ? a * b * (1.0 - c) : k == 3 ? (1.0 - a) * b * (1.0 - c)
         : k == 4 ? (1.0 - a) * (1.0 - b) * c : k == 5 ? a * (1.0 - b) * c
         : k == 6 ? a * b * c : (1.0 - a) * b * c;
}
template <int ROID> NSFV1_HD constexpr double p1_grad(int k, int d, double a, double b, double c) {
    if (ROID == ROID_TRIANGLE) return k == 0 ? -1.0 : (k == 1 ? (d == 0 ? 1.0 : 0.0) : (d == 1 ? 1.0 : 0.0));
    if (ROID == ROID_QUADRILATERAL) {
        if (d == 0) return k == 0 ? -(1.0 - b) : k == 1 ? (1.0 - b) : k == 2 ? b : -b;
        return k == 0 ? -(1.0 - a) : k == 1 ? -a : k == 2 ? a : (1.0 - a);
    }
    if (ROID == ROID_TETRAHEDRON) return k == 0 ? -1.0 : (k - 1 == d ? 1.0 : 0.0);
    if (ROID == ROID_PRISM) {
        const double t = k == 0 || k == 3 ? 1.0 - a - b : (k == 1 || k == 4) ? a : b;
        const double dt = k == 0 || k == 3 ? -1.0 : ((k == 1 || k == 4) ? (d == 0 ? 1.0 : 0.0) : (d == 1 ? 1.0 : 0.0));
        const double z = k >= 3 ? c : 1.0 - c;
        return d == 2 ? (k >= 3 ? t : -t) : dt * z;
    }
    const double xa = (k == 1 || k == 2 || k == 5 || k == 6) ? a : 1.0 - a;
    const double xb = (k == 2 || k == 3 || k == 6 || k == 7) ? b : 1.0 - b;
    const double xc = (k >= 4) ? c : 1.0 - c;
    const double sa = (k == 1 || k == 2 || k == 5 || k == 6) ? 1.0 : -1.0;
    const double sb = (k == 2 || k == 3 || k == 6 || k == 7) ? 1.0 : -1.0;
    const double sc = (k >= 4) ? 1.0 : -1.0;
    return d == 0 ? sa * xb * xc : d == 1 ? xa * sb * xc : xa * xb * sc;
}
template <int ROID> NSFV1_HD constexpr double ip_shape(int ip, int k) {
    using R = Ref<ROID>;
    return p1_shape<ROID>(k, loc_ip<R>(ip, 0), loc_ip<R>(ip, 1), R::dim == 3 ? loc_ip<R>(ip, 2) : 0.0);
}
template <int ROID> NSFV1_HD constexpr double ip_lgrad(int ip, int k, int d) {
    using R = Ref<ROID>;
    return p1_grad<ROID>(k, d, loc_ip<R>(ip, 0), loc_ip<R>(ip, 1), R::dim == 3 ? loc_ip<R>(ip, 2) : 0.0);
}

}  // namespace nsfv1
