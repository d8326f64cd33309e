/*
 * nsfv1_oracle.cpp -- CPU restatement (FP64, scalar C++) of the incompressible
 * FV1 Navier-Stokes element assembly of UG4 plugin_NavierStokes, plus the
 * small pieces of ugcore that the path needs (FV1 dual-mesh geometry, element
 * side ray intersection, block-CSR global assembly, Dirichlet rows, Newton,
 * BiCGStab with point-block Jacobi).
 *
 * THIS IS TEST INFRASTRUCTURE. It is the checker: only tests/, the smoke()
 * entry of __graft_entry__.py and the cpu_baseline / reference leg of
 * bench.py load it. The product library (plugin_navierstokes_gb300) never
 * links, loads or calls it.
 *
 * Parity status: PINNED to the reference's own plugin code. The reference
 * ships no tests, fixtures or golden vectors for this path, and every file
 * includes ugcore (UG4's core library, not in the reference tree). Its FV1
 * sources (navier_stokes_fv1.cpp, stabilization.cpp, upwind.cpp,
 * upwind_interface.cpp, the NavierStokes base classes) are therefore compiled
 * unmodified against a ugcore stand-in (oracle/ugshim, oracle/ref_driver.cpp,
 * make -C oracle ref), and this restatement matches their element callbacks
 * to about 2e-14 relative on every element type and discretisation case
 * (tests/test_reference_pin.py, fixtures tests/golden/reference_elements.npz).
 * The plugin-level algorithm is restated line by line below, each function
 * citing the lines it follows. The ugcore pieces (FV1Geometry,
 * ElementSideRayIntersection, Newton, Krylov) are restated from the box-method
 * definition and documented where they are defined; the stand-in restates the
 * same ugcore pieces independently, so they are cross-checked, not pinned.
 *
 * Layouts (shared with the product's C ABI):
 *   element-local vector  u[fct * nsh + sh]                (fct-major, as
 *                          LocalVector u(fct, sh), navier_stokes_fv1.h:128-140)
 *   element-local matrix  J[((f1 * nsh + s1) * b + f2) * nsh + s2]
 *   global vector         U[node * b + fct]                 (point blocks)
 *   global matrix         block CSR, b x b row-major blocks, rows sorted
 */
#include <cmath>
#include <cstdint>
#include <cstring>
#include <cstdio>
#include <string>
#include <vector>
#include <algorithm>
#include <stdexcept>
#include <cctype>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace nsora {

typedef double number;
enum { MAXCO = 8, MAXEDGE = 12, MAXSIDE = 6, MAXSCVF = 12 };

// ReferenceObjectID numbering of ugcore (elements of this path only).
enum { ROID_TRIANGLE = 2, ROID_QUADRILATERAL = 3, ROID_TETRAHEDRON = 4, ROID_PRISM = 6, ROID_HEXAHEDRON = 8 };

// upwind / stabilisation / diffusion-length ids
enum { UPW_NONE = -1, UPW_NO = 0, UPW_FULL = 1, UPW_SKEWED = 2, UPW_LPS = 3, UPW_POS = 4 };
enum { STAB_NONE = -1, STAB_FIELDS = 0, STAB_FLOW = 1, STAB_WITHOUT = 2 };
enum { DL_RAW = 0, DL_FIVEPOINT = 1, DL_COR = 2 };

static const number SMALL_TOL = 1e-12;

/* ------------------------------------------------------------------------ */
/* Reference elements (the ugcore reference-element tables, restated)       */
/* ------------------------------------------------------------------------ */
struct RefElem {
    int roid, dim, nco, nedge, nside;
    number co[MAXCO][3];
    int edge[MAXEDGE][2];
    int side_nco[MAXSIDE];
    int side[MAXSIDE][4];
    int edge_face[MAXEDGE][2];   // 3D: the two faces at an edge, ordered so that the
                                 // SCVF normal points from edge corner 0 to corner 1
};

static void set_co(RefElem& r, int i, number x, number y, number z) { r.co[i][0] = x; r.co[i][1] = y; r.co[i][2] = z; }

static void cross3(const number* a, const number* b, number* c) {
    c[0] = a[1] * b[2] - a[2] * b[1];
    c[1] = a[2] * b[0] - a[0] * b[2];
    c[2] = a[0] * b[1] - a[1] * b[0];
}

static RefElem make_ref(int roid) {
    RefElem r;
    std::memset(&r, 0, sizeof(r));
    r.roid = roid;
    if (roid == ROID_TRIANGLE) {
        r.dim = 2; r.nco = 3; r.nedge = 3; r.nside = 3;
        set_co(r, 0, 0, 0, 0); set_co(r, 1, 1, 0, 0); set_co(r, 2, 0, 1, 0);
        int e[3][2] = {{0, 1}, {1, 2}, {2, 0}};
        for (int i = 0; i < 3; ++i) { r.edge[i][0] = e[i][0]; r.edge[i][1] = e[i][1]; r.side_nco[i] = 2; r.side[i][0] = e[i][0]; r.side[i][1] = e[i][1]; }
    } else if (roid == ROID_QUADRILATERAL) {
        r.dim = 2; r.nco = 4; r.nedge = 4; r.nside = 4;
        set_co(r, 0, 0, 0, 0); set_co(r, 1, 1, 0, 0); set_co(r, 2, 1, 1, 0); set_co(r, 3, 0, 1, 0);
        int e[4][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}};
        for (int i = 0; i < 4; ++i) { r.edge[i][0] = e[i][0]; r.edge[i][1] = e[i][1]; r.side_nco[i] = 2; r.side[i][0] = e[i][0]; r.side[i][1] = e[i][1]; }
    } else if (roid == ROID_TETRAHEDRON) {
        r.dim = 3; r.nco = 4; r.nedge = 6; r.nside = 4;
        set_co(r, 0, 0, 0, 0); set_co(r, 1, 1, 0, 0); set_co(r, 2, 0, 1, 0); set_co(r, 3, 0, 0, 1);
        int e[6][2] = {{0, 1}, {1, 2}, {2, 0}, {0, 3}, {1, 3}, {2, 3}};
        int f[4][3] = {{0, 2, 1}, {0, 1, 3}, {1, 2, 3}, {0, 3, 2}};
        for (int i = 0; i < 6; ++i) { r.edge[i][0] = e[i][0]; r.edge[i][1] = e[i][1]; }
        for (int i = 0; i < 4; ++i) { r.side_nco[i] = 3; for (int j = 0; j < 3; ++j) r.side[i][j] = f[i][j]; }
    } else if (roid == ROID_PRISM) {
        // the triangle (0, 1, 2) at z = 0 extruded to (3, 4, 5); sides 0 and 4 triangles
        r.dim = 3; r.nco = 6; r.nedge = 9; r.nside = 5;
        set_co(r, 0, 0, 0, 0); set_co(r, 1, 1, 0, 0); set_co(r, 2, 0, 1, 0);
        set_co(r, 3, 0, 0, 1); set_co(r, 4, 1, 0, 1); set_co(r, 5, 0, 1, 1);
        int e[9][2] = {{0, 1}, {1, 2}, {2, 0}, {0, 3}, {1, 4}, {2, 5}, {3, 4}, {4, 5}, {5, 3}};
        int f[5][4] = {{0, 2, 1, -1}, {0, 1, 4, 3}, {1, 2, 5, 4}, {2, 0, 3, 5}, {3, 4, 5, -1}};
        for (int i = 0; i < 9; ++i) { r.edge[i][0] = e[i][0]; r.edge[i][1] = e[i][1]; }
        for (int i = 0; i < 5; ++i) { r.side_nco[i] = (i == 0 || i == 4) ? 3 : 4; for (int j = 0; j < r.side_nco[i]; ++j) r.side[i][j] = f[i][j]; }
    } else if (roid == ROID_HEXAHEDRON) {
        r.dim = 3; r.nco = 8; r.nedge = 12; r.nside = 6;
        set_co(r, 0, 0, 0, 0); set_co(r, 1, 1, 0, 0); set_co(r, 2, 1, 1, 0); set_co(r, 3, 0, 1, 0);
        set_co(r, 4, 0, 0, 1); set_co(r, 5, 1, 0, 1); set_co(r, 6, 1, 1, 1); set_co(r, 7, 0, 1, 1);
        int e[12][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}, {0, 4}, {1, 5}, {2, 6}, {3, 7}, {4, 5}, {5, 6}, {6, 7}, {7, 4}};
        int f[6][4] = {{0, 3, 2, 1}, {0, 1, 5, 4}, {1, 2, 6, 5}, {2, 3, 7, 6}, {0, 4, 7, 3}, {4, 5, 6, 7}};
        for (int i = 0; i < 12; ++i) { r.edge[i][0] = e[i][0]; r.edge[i][1] = e[i][1]; }
        for (int i = 0; i < 6; ++i) { r.side_nco[i] = 4; for (int j = 0; j < 4; ++j) r.side[i][j] = f[i][j]; }
    } else {
        throw std::runtime_error("unsupported reference element");
    }
    if (r.dim == 3) {
        // faces adjacent to each edge, oriented such that
        // 0.5 * (center - edgeMid) x (faceMid[F2] - faceMid[F1]) points from edge corner 0 to 1
        number cen[3] = {0, 0, 0};
        for (int c = 0; c < r.nco; ++c) for (int d = 0; d < 3; ++d) cen[d] += r.co[c][d];
        for (int d = 0; d < 3; ++d) cen[d] /= r.nco;
        for (int e = 0; e < r.nedge; ++e) {
            int a = r.edge[e][0], b = r.edge[e][1], nf = 0, fs[2] = {-1, -1};
            for (int s = 0; s < r.nside; ++s) {
                bool ha = false, hb = false;
                for (int j = 0; j < r.side_nco[s]; ++j) { ha |= (r.side[s][j] == a); hb |= (r.side[s][j] == b); }
                if (ha && hb && nf < 2) fs[nf++] = s;
            }
            if (nf != 2) throw std::runtime_error("edge-face table");
            number fm[2][3];
            for (int k = 0; k < 2; ++k) {
                for (int d = 0; d < 3; ++d) fm[k][d] = 0;
                for (int j = 0; j < r.side_nco[fs[k]]; ++j) for (int d = 0; d < 3; ++d) fm[k][d] += r.co[r.side[fs[k]][j]][d];
                for (int d = 0; d < 3; ++d) fm[k][d] /= r.side_nco[fs[k]];
            }
            number em[3], u[3], v[3], n[3];
            for (int d = 0; d < 3; ++d) { em[d] = 0.5 * (r.co[a][d] + r.co[b][d]); u[d] = cen[d] - em[d]; v[d] = fm[1][d] - fm[0][d]; }
            cross3(u, v, n);
            number dot = 0;
            for (int d = 0; d < 3; ++d) dot += n[d] * (r.co[b][d] - r.co[a][d]);
            if (dot > 0) { r.edge_face[e][0] = fs[0]; r.edge_face[e][1] = fs[1]; }
            else { r.edge_face[e][0] = fs[1]; r.edge_face[e][1] = fs[0]; }
        }
    }
    return r;
}

static const RefElem& ref_elem(int roid) {
    static const RefElem tri = make_ref(ROID_TRIANGLE);
    static const RefElem quad = make_ref(ROID_QUADRILATERAL);
    static const RefElem tet = make_ref(ROID_TETRAHEDRON);
    static const RefElem prism = make_ref(ROID_PRISM);
    static const RefElem hex = make_ref(ROID_HEXAHEDRON);
    switch (roid) {
        case ROID_TRIANGLE: return tri;
        case ROID_QUADRILATERAL: return quad;
        case ROID_TETRAHEDRON: return tet;
        case ROID_PRISM: return prism;
        case ROID_HEXAHEDRON: return hex;
    }
    throw std::runtime_error("unsupported element type");
}

/* P1 Lagrange trial space (linear on simplices, multilinear on quad/hex). */
static void p1_shapes(int roid, const number* x, number* N) {
    switch (roid) {
        case ROID_TRIANGLE: N[0] = 1.0 - x[0] - x[1]; N[1] = x[0]; N[2] = x[1]; return;
        case ROID_QUADRILATERAL:
            N[0] = (1.0 - x[0]) * (1.0 - x[1]); N[1] = x[0] * (1.0 - x[1]);
            N[2] = x[0] * x[1]; N[3] = (1.0 - x[0]) * x[1]; return;
        case ROID_TETRAHEDRON: N[0] = 1.0 - x[0] - x[1] - x[2]; N[1] = x[0]; N[2] = x[1]; N[3] = x[2]; return;
        case ROID_PRISM: {
            const number t[3] = {1.0 - x[0] - x[1], x[0], x[1]};
            for (int k = 0; k < 6; ++k) N[k] = t[k % 3] * (k >= 3 ? x[2] : 1.0 - x[2]);
            return;
        }
        case ROID_HEXAHEDRON: {
            const number a = x[0], b = x[1], c = x[2];
            N[0] = (1.0 - a) * (1.0 - b) * (1.0 - c); N[1] = a * (1.0 - b) * (1.0 - c);
            N[2] = a * b * (1.0 - c); N[3] = (1.0 - a) * b * (1.0 - c);
            N[4] = (1.0 - a) * (1.0 - b) * c; N[5] = a * (1.0 - b) * c;
            N[6] = a * b * c; N[7] = (1.0 - a) * b * c; return;
        }
    }
}

static void p1_grads(int roid, const number* x, number G[][3]) {
    switch (roid) {
        case ROID_TRIANGLE:
            G[0][0] = -1; G[0][1] = -1; G[1][0] = 1; G[1][1] = 0; G[2][0] = 0; G[2][1] = 1; return;
        case ROID_QUADRILATERAL:
            G[0][0] = -(1.0 - x[1]); G[0][1] = -(1.0 - x[0]);
            G[1][0] = (1.0 - x[1]);  G[1][1] = -x[0];
            G[2][0] = x[1];          G[2][1] = x[0];
            G[3][0] = -x[1];         G[3][1] = (1.0 - x[0]); return;
        case ROID_TETRAHEDRON:
            G[0][0] = -1; G[0][1] = -1; G[0][2] = -1;
            G[1][0] = 1; G[1][1] = 0; G[1][2] = 0;
            G[2][0] = 0; G[2][1] = 1; G[2][2] = 0;
            G[3][0] = 0; G[3][1] = 0; G[3][2] = 1; return;
        case ROID_PRISM: {
            const number t[3] = {1.0 - x[0] - x[1], x[0], x[1]};
            const number dt[3][2] = {{-1.0, -1.0}, {1.0, 0.0}, {0.0, 1.0}};
            for (int k = 0; k < 6; ++k) {
                const number z = k >= 3 ? x[2] : 1.0 - x[2], dz = k >= 3 ? 1.0 : -1.0;
                G[k][0] = dt[k % 3][0] * z; G[k][1] = dt[k % 3][1] * z; G[k][2] = t[k % 3] * dz;
            }
            return;
        }
        case ROID_HEXAHEDRON: {
            const number a = x[0], b = x[1], c = x[2];
            G[0][0] = -(1.0 - b) * (1.0 - c); G[0][1] = -(1.0 - a) * (1.0 - c); G[0][2] = -(1.0 - a) * (1.0 - b);
            G[1][0] = (1.0 - b) * (1.0 - c);  G[1][1] = -a * (1.0 - c);         G[1][2] = -a * (1.0 - b);
            G[2][0] = b * (1.0 - c);          G[2][1] = a * (1.0 - c);          G[2][2] = -a * b;
            G[3][0] = -b * (1.0 - c);         G[3][1] = (1.0 - a) * (1.0 - c);  G[3][2] = -(1.0 - a) * b;
            G[4][0] = -(1.0 - b) * c;         G[4][1] = -(1.0 - a) * c;         G[4][2] = (1.0 - a) * (1.0 - b);
            G[5][0] = (1.0 - b) * c;          G[5][1] = -a * c;                 G[5][2] = a * (1.0 - b);
            G[6][0] = b * c;                  G[6][1] = a * c;                  G[6][2] = a * b;
            G[7][0] = -b * c;                 G[7][1] = (1.0 - a) * c;          G[7][2] = (1.0 - a) * b; return;
        }
    }
}

/* ------------------------------------------------------------------------ */
/* FV1 geometry (ugcore FV1Geometry::update, restated from the box method).  */
/* SCVF i belongs to edge i (from = edge corner 0, to = edge corner 1).      */
/* 2D SCVF corners: {edge midpoint, element centre}; normal = the segment    */
/*   normal (d_y, -d_x) of d = centre - edgeMid, pointing from -> to.        */
/* 3D SCVF corners: {edge midpoint, face centre F1, element centre, face     */
/*   centre F2}; normal = 0.5 (c2 - c0) x (c3 - c1), pointing from -> to.    */
/* ip = mean of the SCVF corners (global and local alike); shapes and local  */
/* gradients at the local ip; global grad = J^-T(local ip) * local grad.     */
/* SCV of corner a: 2D quad {a, mid(next edge), centre, mid(prev edge)};     */
/* 3D hex {a, mids of the 3 edges at a, centres of the 3 faces at a,         */
/* centre}; volume = |sum of 6 tetrahedra around the a-centre diagonal|.     */
/* ------------------------------------------------------------------------ */
struct SCVF {
    int from, to, numCo;
    number gloPos[4][3], locPos[4][3];
    number globalIP[3], localIP[3], normal[3];
    number shape[MAXCO];
    number localGrad[MAXCO][3];
    number globalGrad[MAXCO][3];
    number detJ;
};
struct SCV {
    int nodeId;
    number vol;
    number globalIP[3];
};

struct FV1Geometry {
    int roid, dim, nsh, nscvf, nscv;
    number corners[MAXCO][3];
    SCVF scvf[MAXSCVF];
    SCV scv[MAXCO];
    void update(int roid_, const number* vCornerCoords);
};

static number det_and_jtinv(int dim, const number J[3][3], number JtInv[3][3]) {
    // J[i][j] = d x_i / d xi_j ; JtInv = (J^T)^{-1}
    if (dim == 2) {
        const number det = J[0][0] * J[1][1] - J[0][1] * J[1][0];
        const number id = 1.0 / det;
        // (J^T)^-1 = (J^-1)^T ; J^-1 = id * [[J11, -J01], [-J10, J00]]
        JtInv[0][0] = J[1][1] * id;  JtInv[0][1] = -J[1][0] * id;
        JtInv[1][0] = -J[0][1] * id; JtInv[1][1] = J[0][0] * id;
        return det;
    }
    // cofactor matrix C of J: J^-1 = C^T / det ; (J^-1)^T = C / det
    number C[3][3];
    C[0][0] = J[1][1] * J[2][2] - J[1][2] * J[2][1];
    C[0][1] = J[1][2] * J[2][0] - J[1][0] * J[2][2];
    C[0][2] = J[1][0] * J[2][1] - J[1][1] * J[2][0];
    C[1][0] = J[0][2] * J[2][1] - J[0][1] * J[2][2];
    C[1][1] = J[0][0] * J[2][2] - J[0][2] * J[2][0];
    C[1][2] = J[0][1] * J[2][0] - J[0][0] * J[2][1];
    C[2][0] = J[0][1] * J[1][2] - J[0][2] * J[1][1];
    C[2][1] = J[0][2] * J[1][0] - J[0][0] * J[1][2];
    C[2][2] = J[0][0] * J[1][1] - J[0][1] * J[1][0];
    const number det = J[0][0] * C[0][0] + J[0][1] * C[0][1] + J[0][2] * C[0][2];
    const number id = 1.0 / det;
    for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) JtInv[i][j] = C[i][j] * id;
    return det;
}

static number tet_signed6(const number* a, const number* b, const number* c, const number* d) {
    number u[3], v[3], w[3], x[3];
    for (int k = 0; k < 3; ++k) { u[k] = b[k] - a[k]; v[k] = c[k] - a[k]; w[k] = d[k] - a[k]; }
    cross3(v, w, x);
    return u[0] * x[0] + u[1] * x[1] + u[2] * x[2];
}

void FV1Geometry::update(int roid_, const number* vCornerCoords) {
    const RefElem& R = ref_elem(roid_);
    roid = roid_; dim = R.dim; nsh = R.nco; nscvf = R.nedge; nscv = R.nco;
    for (int c = 0; c < nsh; ++c) for (int d = 0; d < 3; ++d) corners[c][d] = (d < dim) ? vCornerCoords[c * dim + d] : 0.0;

    // midpoints: edges, faces (3D), element centre -- global and local
    number gEdge[MAXEDGE][3], lEdge[MAXEDGE][3], gFace[MAXSIDE][3], lFace[MAXSIDE][3], gCen[3], lCen[3];
    for (int e = 0; e < R.nedge; ++e) {
        const int a = R.edge[e][0], b = R.edge[e][1];
        for (int d = 0; d < 3; ++d) {
            gEdge[e][d] = 0.5 * (corners[a][d] + corners[b][d]);
            lEdge[e][d] = 0.5 * (R.co[a][d] + R.co[b][d]);
        }
    }
    if (dim == 3) {
        for (int s = 0; s < R.nside; ++s) {
            const number w = 1.0 / R.side_nco[s];
            for (int d = 0; d < 3; ++d) {
                number g = 0, l = 0;
                for (int j = 0; j < R.side_nco[s]; ++j) { g += corners[R.side[s][j]][d]; l += R.co[R.side[s][j]][d]; }
                gFace[s][d] = g * w; lFace[s][d] = l * w;
            }
        }
    }
    {
        const number w = 1.0 / nsh;
        for (int d = 0; d < 3; ++d) {
            number g = 0, l = 0;
            for (int c = 0; c < nsh; ++c) { g += corners[c][d]; l += R.co[c][d]; }
            gCen[d] = g * w; lCen[d] = l * w;
        }
    }

    for (int i = 0; i < nscvf; ++i) {
        SCVF& f = scvf[i];
        f.from = R.edge[i][0]; f.to = R.edge[i][1];
        if (dim == 2) {
            f.numCo = 2;
            for (int d = 0; d < 3; ++d) {
                f.gloPos[0][d] = gEdge[i][d]; f.gloPos[1][d] = gCen[d];
                f.locPos[0][d] = lEdge[i][d]; f.locPos[1][d] = lCen[d];
            }
            const number dx = f.gloPos[1][0] - f.gloPos[0][0], dy = f.gloPos[1][1] - f.gloPos[0][1];
            f.normal[0] = dy; f.normal[1] = -dx; f.normal[2] = 0;
        } else {
            f.numCo = 4;
            const int F1 = R.edge_face[i][0], F2 = R.edge_face[i][1];
            for (int d = 0; d < 3; ++d) {
                f.gloPos[0][d] = gEdge[i][d]; f.gloPos[1][d] = gFace[F1][d];
                f.gloPos[2][d] = gCen[d];     f.gloPos[3][d] = gFace[F2][d];
                f.locPos[0][d] = lEdge[i][d]; f.locPos[1][d] = lFace[F1][d];
                f.locPos[2][d] = lCen[d];     f.locPos[3][d] = lFace[F2][d];
            }
            number a[3], b[3], n[3];
            for (int d = 0; d < 3; ++d) { a[d] = f.gloPos[2][d] - f.gloPos[0][d]; b[d] = f.gloPos[3][d] - f.gloPos[1][d]; }
            cross3(a, b, n);
            for (int d = 0; d < 3; ++d) f.normal[d] = 0.5 * n[d];
        }
        const number w = 1.0 / f.numCo;
        for (int d = 0; d < 3; ++d) {
            number g = 0, l = 0;
            for (int k = 0; k < f.numCo; ++k) { g += f.gloPos[k][d]; l += f.locPos[k][d]; }
            f.globalIP[d] = g * w; f.localIP[d] = l * w;
        }
        p1_shapes(roid, f.localIP, f.shape);
        p1_grads(roid, f.localIP, f.localGrad);
        number J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, JtInv[3][3];
        for (int r = 0; r < dim; ++r)
            for (int c = 0; c < dim; ++c) {
                number s = 0;
                for (int k = 0; k < nsh; ++k) s += corners[k][r] * f.localGrad[k][c];
                J[r][c] = s;
            }
        f.detJ = det_and_jtinv(dim, J, JtInv);
        for (int k = 0; k < nsh; ++k) {
            for (int r = 0; r < 3; ++r) f.globalGrad[k][r] = 0;
            for (int r = 0; r < dim; ++r) {
                number s = 0;
                for (int c = 0; c < dim; ++c) s += JtInv[r][c] * f.localGrad[k][c];
                f.globalGrad[k][r] = s;
            }
        }
    }

    for (int a = 0; a < nscv; ++a) {
        SCV& v = scv[a];
        v.nodeId = a;
        for (int d = 0; d < 3; ++d) v.globalIP[d] = corners[a][d];
        if (dim == 2) {
            int next = -1, prev = -1;
            for (int e = 0; e < R.nedge; ++e) { if (R.edge[e][0] == a) next = e; if (R.edge[e][1] == a) prev = e; }
            const number* p0 = corners[a];
            const number* p1 = gEdge[next];
            const number* p2 = gCen;
            const number* p3 = gEdge[prev];
            const number cr = (p2[0] - p0[0]) * (p3[1] - p1[1]) - (p2[1] - p0[1]) * (p3[0] - p1[0]);
            v.vol = 0.5 * std::fabs(cr);
        } else {
            int nb[3], eid[3], n = 0;
            for (int e = 0; e < R.nedge && n < 3; ++e) {
                if (R.edge[e][0] == a) { nb[n] = R.edge[e][1]; eid[n++] = e; }
                else if (R.edge[e][1] == a) { nb[n] = R.edge[e][0]; eid[n++] = e; }
            }
            auto face_of = [&](int x, int y) -> int {
                for (int s = 0; s < R.nside; ++s) {
                    bool ha = false, hx = false, hy = false;
                    for (int j = 0; j < R.side_nco[s]; ++j) { ha |= R.side[s][j] == a; hx |= R.side[s][j] == x; hy |= R.side[s][j] == y; }
                    if (ha && hx && hy) return s;
                }
                throw std::runtime_error("scv face");
            };
            const number* q[8];
            q[0] = corners[a];
            q[1] = gEdge[eid[0]];
            q[2] = gFace[face_of(nb[0], nb[1])];
            q[3] = gEdge[eid[1]];
            q[4] = gEdge[eid[2]];
            q[5] = gFace[face_of(nb[0], nb[2])];
            q[6] = gCen;
            q[7] = gFace[face_of(nb[1], nb[2])];
            number s6 = tet_signed6(q[0], q[1], q[2], q[6]) + tet_signed6(q[0], q[2], q[3], q[6])
                      + tet_signed6(q[0], q[3], q[7], q[6]) + tet_signed6(q[0], q[7], q[4], q[6])
                      + tet_signed6(q[0], q[4], q[5], q[6]) + tet_signed6(q[0], q[5], q[1], q[6]);
            v.vol = std::fabs(s6) / 6.0;
        }
    }
}

/* ------------------------------------------------------------------------ */
/* ElementSideRayIntersection (ugcore lib_disc/common/geometry_util.h, absent), */
/* restated: sides are tested in reference order, a quadrilateral face as the */
/* two triangles (0,1,2) and (0,2,3); the first side hit with t <= 0 (upwind  */
/* search) or t >= 0 (downstream search) is taken. Local intersection = the  */
/* same barycentric combination of the side's reference corners.            */
/* ------------------------------------------------------------------------ */
static bool ray_side_intersection(const RefElem& R, const number corners[][3], const number* from, const number* dir,
                                  bool positive, int& sideOut, number* gInt, number* lInt) {
    if (R.dim == 2) {
        for (int s = 0; s < R.nside; ++s) {
            const int i0 = R.side[s][0], i1 = R.side[s][1];
            const number* p0 = corners[i0];
            const number* p1 = corners[i1];
            // p0 + bc (p1 - p0) = from + t dir
            const number a00 = p1[0] - p0[0], a01 = -dir[0];
            const number a10 = p1[1] - p0[1], a11 = -dir[1];
            const number det = a00 * a11 - a01 * a10;
            if (det == 0.0) continue;
            const number r0 = from[0] - p0[0], r1 = from[1] - p0[1];
            const number bc = (r0 * a11 - a01 * r1) / det;
            const number t = (a00 * r1 - r0 * a10) / det;
            if (bc < -SMALL_TOL || bc > 1.0 + SMALL_TOL) continue;
            if ((positive && t >= 0.0) || (!positive && t <= 0.0)) {
                sideOut = s;
                for (int d = 0; d < 3; ++d) {
                    gInt[d] = (d < 2) ? p0[d] + bc * (p1[d] - p0[d]) : 0.0;
                    lInt[d] = R.co[i0][d] + bc * (R.co[i1][d] - R.co[i0][d]);
                }
                return true;
            }
        }
        return false;
    }
    for (int s = 0; s < R.nside; ++s) {
        const int ntri = (R.side_nco[s] == 4) ? 2 : 1;
        for (int tr = 0; tr < ntri; ++tr) {
            const int i0 = R.side[s][0];
            const int i1 = R.side[s][tr == 0 ? 1 : 2];
            const int i2 = R.side[s][tr == 0 ? 2 : 3];
            const number* q0 = corners[i0];
            const number* q1 = corners[i1];
            const number* q2 = corners[i2];
            number e1[3], e2[3], nd[3], r[3], c[3];
            for (int d = 0; d < 3; ++d) { e1[d] = q1[d] - q0[d]; e2[d] = q2[d] - q0[d]; nd[d] = -dir[d]; r[d] = from[d] - q0[d]; }
            // [e1 e2 -dir] (a, b, t)^T = r   (Cramer's rule)
            cross3(e2, nd, c);
            const number det = e1[0] * c[0] + e1[1] * c[1] + e1[2] * c[2];
            if (det == 0.0) continue;
            const number a = (r[0] * c[0] + r[1] * c[1] + r[2] * c[2]) / det;
            number c2[3];
            cross3(r, nd, c2);
            const number b = (e1[0] * c2[0] + e1[1] * c2[1] + e1[2] * c2[2]) / det;
            number c3[3];
            cross3(e2, r, c3);
            const number t = (e1[0] * c3[0] + e1[1] * c3[1] + e1[2] * c3[2]) / det;
            if (a < -SMALL_TOL || b < -SMALL_TOL || a + b > 1.0 + SMALL_TOL) continue;
            if ((positive && t >= 0.0) || (!positive && t <= 0.0)) {
                sideOut = s;
                for (int d = 0; d < 3; ++d) {
                    gInt[d] = q0[d] + a * e1[d] + b * e2[d];
                    lInt[d] = R.co[i0][d] + a * (R.co[i1][d] - R.co[i0][d]) + b * (R.co[i2][d] - R.co[i0][d]);
                }
                return true;
            }
        }
    }
    return false;
}

static number vdist(int dim, const number* a, const number* b) {
    number s = 0;
    for (int d = 0; d < dim; ++d) { const number x = a[d] - b[d]; s += x * x; }
    return std::sqrt(s);
}
static number vnorm(int dim, const number* a) {
    number s = 0;
    for (int d = 0; d < dim; ++d) s += a[d] * a[d];
    return std::sqrt(s);
}

/* ------------------------------------------------------------------------ */
/* Upwinds (upwind.cpp / upwind_interface.h)                                */
/* ------------------------------------------------------------------------ */
struct Upwind {
    int type = UPW_NONE;
    number upShapeSh[MAXSCVF][MAXCO], downShapeSh[MAXSCVF][MAXCO];
    number upShapeIp[MAXSCVF][MAXSCVF], downShapeIp[MAXSCVF][MAXSCVF];
    number upConvLength[MAXSCVF], downConvLength[MAXSCVF];

    // set_shape_ip_flag of the constructors (upwind.h:69-295): only the positive
    // (and regular) upwinds take values at other integration points
    bool non_zero_shape_ip() const { return type == UPW_POS; }

    // NavierStokesPositiveUpwind::compute<FV1> (upwind.cpp:643-786): per SCV, every
    // outflow face takes the SCV's inflow faces (weighted by their share of the
    // larger of total in- and outflow) as ip shapes and the corner the rest
    void positive(const FV1Geometry& geo, const number vIPVel[][3], number vUpShapeSh[][MAXCO], number vUpShapeIp[][MAXSCVF],
                  number vConvLength[]) const {
        const int dim = geo.dim, nip = geo.nscvf;
        number massFlux[MAXSCVF];
        bool hasFlux[MAXSCVF];
        const number eps = std::numeric_limits<number>::epsilon() * 10;
        int numNoFlux = 0;
        for (int ip = 0; ip < nip; ++ip) {
            const SCVF& scvf = geo.scvf[ip];
            massFlux[ip] = 0.0;
            hasFlux[ip] = true;
            for (int sh = 0; sh < geo.nsh; ++sh) vUpShapeSh[ip][sh] = 0.0;
            for (int j = 0; j < nip; ++j) vUpShapeIp[ip][j] = 0.0;
            number normSq = 0;
            for (int d = 0; d < dim; ++d) normSq += vIPVel[ip][d] * vIPVel[ip][d];
            if (std::fabs(normSq) <= eps) {
                vUpShapeSh[ip][scvf.from] = 0.5;
                vUpShapeSh[ip][scvf.to] = 0.5;
                hasFlux[ip] = false;
                ++numNoFlux;
                continue;
            }
            number mf = 0;
            for (int d = 0; d < dim; ++d) mf += vIPVel[ip][d] * scvf.normal[d];
            massFlux[ip] = mf;
            const number vel = std::sqrt(normSq);
            const number len = vnorm(dim, scvf.normal);
            if (std::fabs(massFlux[ip] / std::sqrt(vel * len)) <= eps) {
                vUpShapeSh[ip][scvf.from] = 0.5;
                vUpShapeSh[ip][scvf.to] = 0.5;
                hasFlux[ip] = false;
                ++numNoFlux;
                continue;
            }
        }
        if (numNoFlux != nip) {
            for (int sh = 0; sh < geo.nsh; ++sh) {
                number mIn = 0, mOut = 0;
                int ips[MAXSCVF], n = 0;
                number flux[MAXSCVF];
                for (int ip = 0; ip < nip; ++ip) {
                    if (!hasFlux[ip]) continue;
                    const SCVF& scvf = geo.scvf[ip];
                    if (scvf.from == sh) {
                        ips[n] = ip; flux[n] = massFlux[ip]; ++n;
                        mIn += -1.0 * std::min(massFlux[ip], 0.0);
                        mOut += std::max(massFlux[ip], 0.0);
                    } else if (scvf.to == sh) {
                        ips[n] = ip; flux[n] = -1.0 * massFlux[ip]; ++n;
                        mIn += -1.0 * std::min(-1.0 * massFlux[ip], 0.0);
                        mOut += std::max(-1.0 * massFlux[ip], 0.0);
                    }
                }
                const number F = std::max(mIn, mOut);
                for (int i = 0; i < n; ++i) {
                    if (flux[i] > 0) {
                        number sum = 0.0;
                        for (int j = 0; j < n; ++j)
                            if (flux[j] < 0) sum += vUpShapeIp[ips[i]][ips[j]] = -1.0 * flux[j] / F;
                        vUpShapeSh[ips[i]][sh] = 1.0 - sum;
                    }
                }
            }
        }
        // convection length: distance of the ip from the upwind point the shapes interpolate
        for (int ip = 0; ip < nip; ++ip) {
            number up[3] = {0, 0, 0};
            for (int sh = 0; sh < geo.nsh; ++sh)
                for (int d = 0; d < dim; ++d) up[d] += vUpShapeSh[ip][sh] * geo.corners[sh][d];
            for (int j = 0; j < nip; ++j)
                for (int d = 0; d < dim; ++d) up[d] += vUpShapeIp[ip][j] * geo.scvf[j].globalIP[d];
            vConvLength[ip] = vdist(dim, geo.scvf[ip].globalIP, up);
        }
    }

    // INavierStokesUpwind::compute dispatch (upwind_interface.h:243-250)
    void compute(const FV1Geometry& geo, const number vIPVel[][3], number vUpShapeSh[][MAXCO], number vUpShapeIp[][MAXSCVF],
                 number vConvLength[]) const {
        const RefElem& R = ref_elem(geo.roid);
        const int dim = geo.dim;
        if (type == UPW_POS) { positive(geo, vIPVel, vUpShapeSh, vUpShapeIp, vConvLength); return; }
        for (int ip = 0; ip < geo.nscvf; ++ip) {
            const SCVF& scvf = geo.scvf[ip];
            if (type == UPW_NO) {
                // NavierStokesNoUpwind::compute<FV1> (upwind.cpp:52-80)
                for (int sh = 0; sh < geo.nsh; ++sh) vUpShapeSh[ip][sh] = scvf.shape[sh];
                vConvLength[ip] = 1.0;
            } else if (type == UPW_FULL) {
                // NavierStokesFullUpwind::compute<FV1> (upwind.cpp:133-172)
                for (int sh = 0; sh < geo.nsh; ++sh) vUpShapeSh[ip][sh] = 0.0;
                number flux = 0;
                for (int d = 0; d < dim; ++d) flux += scvf.normal[d] * vIPVel[ip][d];
                if (flux > 0.0) {
                    vUpShapeSh[ip][scvf.from] = 1.0;
                    vConvLength[ip] = vdist(dim, scvf.globalIP, geo.corners[scvf.from]);
                } else {
                    vUpShapeSh[ip][scvf.to] = 1.0;
                    vConvLength[ip] = vdist(dim, scvf.globalIP, geo.corners[scvf.to]);
                }
            } else if (type == UPW_SKEWED || type == UPW_LPS) {
                // NavierStokesSkewedUpwind::compute<FV1> (upwind.cpp:381-430)
                // NavierStokesLinearProfileSkewedUpwind::compute<FV1> (upwind.cpp:505-575)
                for (int sh = 0; sh < geo.nsh; ++sh) vUpShapeSh[ip][sh] = 0.0;
                if (vnorm(dim, vIPVel[ip]) < 1e-14) { vConvLength[ip] = 1.0; continue; }
                int side = 0;
                number gInt[3], lInt[3];
                if (!ray_side_intersection(R, geo.corners, scvf.globalIP, vIPVel[ip], false, side, gInt, lInt))
                    throw std::runtime_error("upwind: cannot find cut side");
                if (type == UPW_LPS) {
                    number N[MAXCO];
                    p1_shapes(geo.roid, lInt, N);
                    for (int j = 0; j < R.side_nco[side]; ++j) {
                        const int co = R.side[side][j];
                        vUpShapeSh[ip][co] = N[co];
                    }
                    vConvLength[ip] = vdist(dim, scvf.globalIP, gInt);
                } else {
                    // GetNodeNextToCut (upwind.cpp:338-379)
                    number mn = 1e300;
                    int coOut = R.side[side][0];
                    for (int j = 0; j < R.side_nco[side]; ++j) {
                        const int co = R.side[side][j];
                        number dist = 0;
                        for (int d = 0; d < dim; ++d) { const number x = gInt[d] - geo.corners[co][d]; dist += x * x; }
                        if (dist < mn) { mn = dist; coOut = co; }
                    }
                    vUpShapeSh[ip][coOut] = 1.0;
                    vConvLength[ip] = vdist(dim, scvf.globalIP, geo.corners[coOut]);
                }
            } else {
                throw std::runtime_error("upwind type not set");
            }
        }
    }
    // update_upwind / update_downwind (upwind_interface.h:150-165)
    void update_upwind(const FV1Geometry& geo, const number vStdVel[][3]) { compute(geo, vStdVel, upShapeSh, upShapeIp, upConvLength); }
    void update_downwind(const FV1Geometry& geo, const number vStdVel[][3]) {
        number vDown[MAXSCVF][3];
        for (int ip = 0; ip < geo.nscvf; ++ip) for (int d = 0; d < 3; ++d) vDown[ip][d] = vStdVel[ip][d] * -1.0;
        compute(geo, vDown, downShapeSh, downShapeIp, downConvLength);
    }
    // upwind_vel (upwind_interface.h:333-358): corner shapes, plus the ip shapes times
    // the ip velocities where the upwind has them
    void upwind_vel(const FV1Geometry& geo, int scvf, const number* u, const number vStdVel[][3], number* vel) const {
        for (int d = 0; d < 3; ++d) vel[d] = 0.0;
        for (int sh = 0; sh < geo.nsh; ++sh)
            for (int d = 0; d < geo.dim; ++d) vel[d] += upShapeSh[scvf][sh] * u[d * geo.nsh + sh];
        if (!non_zero_shape_ip()) return;
        for (int j = 0; j < geo.nscvf; ++j)
            for (int d = 0; d < geo.dim; ++d) vel[d] += upShapeIp[scvf][j] * vStdVel[j][d];
    }
};

/* ------------------------------------------------------------------------ */
/* Diffusion lengths (incompressible/fv1/diffusion_length.h)                */
/* ------------------------------------------------------------------------ */
static void diff_length(int type, const FV1Geometry& geo, number* out) {
    const int dim = geo.dim;
    if (type == DL_COR) {
        // NSDiffLengthCor (diffusion_length.h:135-199)
        number minNormSq = 1.79769313486231570e308, minDistSq = 1.79769313486231570e308, avgNormSq = 0.0;
        for (int i = 0; i < geo.nscvf; ++i) {
            const SCVF& f = geo.scvf[i];
            number nn = 0;
            for (int d = 0; d < dim; ++d) nn += f.normal[d] * f.normal[d];
            if (nn < minNormSq) minNormSq = nn;
            avgNormSq += nn;
            if (dim == 3) {
                number ds = 0;
                for (int d = 0; d < 3; ++d) { const number x = f.gloPos[0][d] - f.gloPos[2][d]; ds += x * x; }
                if (ds < minDistSq) minDistSq = ds;
            }
        }
        avgNormSq /= geo.nscvf;
        for (int i = 0; i < geo.nscvf; ++i) {
            const SCVF& f = geo.scvf[i];
            number area = 0.5 * (geo.scv[f.from].vol + geo.scv[f.to].vol);
            area *= area;
            if (dim == 2) out[i] = 2.0 * minNormSq / area + 8.0 / (3.0 * avgNormSq);
            else out[i] = 2.0 * minNormSq / area + 8.0 * minDistSq / (3.0 * avgNormSq);
        }
        return;
    }
    for (int i = 0; i < geo.nscvf; ++i) {
        const SCVF& f = geo.scvf[i];
        number nn = 0;
        for (int d = 0; d < dim; ++d) nn += f.normal[d] * f.normal[d];
        number area = 0.5 * (geo.scv[f.from].vol + geo.scv[f.to].vol);
        area *= area;
        number ds = 0;
        if (dim == 3) for (int d = 0; d < 3; ++d) { const number x = f.gloPos[0][d] - f.gloPos[2][d]; ds += x * x; }
        if (type == DL_FIVEPOINT) {
            // NSDiffLengthFivePoint (diffusion_length.h:48-89)
            if (dim == 2) out[i] = 2.0 * nn / area + 8.0 / nn;
            else out[i] = 2.0 * nn / area + 8.0 * ds / nn;
        } else {
            // NSDiffLengthRaw (diffusion_length.h:91-133)
            if (dim == 2) out[i] = 1. / (0.5 * area / nn + 3.0 * nn / 8.);
            else out[i] = 1. / (0.5 * area / nn + 3.0 * ds / 8.);
        }
    }
}

/* ------------------------------------------------------------------------ */
/* Stabilisations (incompressible/fv1/stabilization.{h,cpp}): the diagonal    */
/* branch (upwinds without ip shapes: no, full, skewed, LPS) and the         */
/* non-diagonal one (positive upwind), whose ip-ip system is inverted.      */
/* ------------------------------------------------------------------------ */

// inverse of the n x n matrix A (row-major, leading dimension MAXSCVF) by
// Gauss-Jordan elimination with partial pivoting; false if a pivot is zero
static bool dense_inverse(int n, const number A[][MAXSCVF], number inv[][MAXSCVF]) {
    number w[MAXSCVF][2 * MAXSCVF];
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) { w[i][j] = A[i][j]; w[i][n + j] = (i == j) ? 1.0 : 0.0; }
    for (int c = 0; c < n; ++c) {
        int p = c;
        for (int q = c + 1; q < n; ++q) if (std::fabs(w[q][c]) > std::fabs(w[p][c])) p = q;
        if (w[p][c] == 0.0) return false;
        if (p != c) for (int j = 0; j < 2 * n; ++j) std::swap(w[p][j], w[c][j]);
        const number piv = 1.0 / w[c][c];
        for (int j = 0; j < 2 * n; ++j) w[c][j] *= piv;
        for (int q = 0; q < n; ++q) {
            if (q == c) continue;
            const number f = w[q][c];
            if (f == 0.0) continue;
            for (int j = 0; j < 2 * n; ++j) w[q][j] -= f * w[c][j];
        }
    }
    for (int i = 0; i < n; ++i) for (int j = 0; j < n; ++j) inv[i][j] = w[i][n + j];
    return true;
}

// y = inv x over n entries (the summation order of a dense matrix-vector product)
static void inv_apply(int n, const number inv[][MAXSCVF], const number* x, number* y) {
    for (int i = 0; i < n; ++i) {
        number acc = 0;
        for (int j = 0; j < n; ++j) acc += inv[i][j] * x[j];
        y[i] = 1.0 * acc;
    }
}

struct Stab {
    int type = STAB_NONE;
    int diffLengthType = DL_RAW;
    Upwind* upwind = nullptr;   // shared with the convection upwind when set by name
    number stabVel[MAXSCVF][3];
    number stabShapeVel[MAXSCVF][3][3][MAXCO];
    number stabShapeP[MAXSCVF][3][MAXCO];
    number diffLenSqInv[MAXSCVF];
    bool vel_comp_connected() const { return type == STAB_FLOW; }   // stabilization.h:462,544,612

    // FIELDS, non-diagonal branch (stabilization.cpp:244-403): one ip-ip matrix (time,
    // diffusion, convection with the upwind's ip shapes), inverted once and applied per
    // velocity component to the corner contributions and to the right-hand side
    void nondiag_fields(const FV1Geometry& geo, const number* u, number density, const number* pSource, const number* uOld,
                        number dt, const number* visc, const number* nsvcl) {
        const int dim = geo.dim, nsh = geo.nsh, P = dim, N = geo.nscvf;
        number mat[MAXSCVF][MAXSCVF], inv[MAXSCVF][MAXSCVF];
        for (int i = 0; i < N; ++i) for (int j = 0; j < N; ++j) mat[i][j] = 0.0;
        for (int ip = 0; ip < N; ++ip) {
            if (uOld != nullptr) mat[ip][ip] += 1. / dt;
            mat[ip][ip] += visc[ip];
            const number scale = nsvcl[ip];
            mat[ip][ip] += scale;
            for (int ip2 = 0; ip2 < N; ++ip2) mat[ip][ip2] -= upwind->upShapeIp[ip][ip2] * scale;
        }
        if (!dense_inverse(N, mat, inv)) throw std::runtime_error("Could not compute inverse.");
        for (int d = 0; d < dim; ++d) {
            number contVel[MAXCO][MAXSCVF], contP[MAXCO][MAXSCVF], x[MAXSCVF];
            for (int ip = 0; ip < N; ++ip) {
                const SCVF& scvf = geo.scvf[ip];
                for (int k = 0; k < nsh; ++k) {
                    contVel[k][ip] = visc[ip] * scvf.shape[k];
                    contVel[k][ip] += nsvcl[ip] * upwind->upShapeSh[ip][k];
                    contP[k][ip] = -1.0 * scvf.globalGrad[k][d] / density;
                }
            }
            for (int k = 0; k < nsh; ++k) {
                inv_apply(N, inv, contVel[k], x);
                for (int ip = 0; ip < N; ++ip) stabShapeVel[ip][d][d][k] = x[ip];
                inv_apply(N, inv, contP[k], x);
                for (int ip = 0; ip < N; ++ip) stabShapeP[ip][d][k] = x[ip];
            }
            number f[MAXSCVF];
            for (int ip = 0; ip < N; ++ip) {
                const SCVF& scvf = geo.scvf[ip];
                f[ip] = 0.0;
                if (pSource != nullptr) f[ip] = pSource[d];
                if (uOld != nullptr) {
                    number oldIPVel = 0.0;
                    for (int sh = 0; sh < nsh; ++sh) oldIPVel += scvf.shape[sh] * uOld[d * nsh + sh];
                    f[ip] += oldIPVel / dt;
                }
            }
            for (int k = 0; k < nsh; ++k) {
                for (int ip = 0; ip < N; ++ip) f[ip] = 1.0 * f[ip] + u[d * nsh + k] * contVel[k][ip];
                for (int ip = 0; ip < N; ++ip) f[ip] = 1.0 * f[ip] + u[P * nsh + k] * contP[k][ip];
            }
            inv_apply(N, inv, f, x);
            for (int ip = 0; ip < N; ++ip) stabVel[ip][d] = x[ip];
        }
    }

    // FLOW, non-diagonal branch (stabilization.cpp:589-771): the ip-ip matrix adds the
    // divergence correction with the upwind and downwind ip shapes; the velocity
    // components stay coupled through the ip velocities and the shape gradients
    void nondiag_flow(const FV1Geometry& geo, const number* u, const number vStdVel[][3], number density, const number* pSource,
                      const number* uOld, number dt, const number* visc, const number* nsvcl, const number* nsvdl) {
        const int dim = geo.dim, nsh = geo.nsh, P = dim, N = geo.nscvf;
        number mat[MAXSCVF][MAXSCVF], inv[MAXSCVF][MAXSCVF];
        for (int i = 0; i < N; ++i) for (int j = 0; j < N; ++j) mat[i][j] = 0.0;
        for (int ip = 0; ip < N; ++ip) {
            if (uOld != nullptr) mat[ip][ip] += 1. / dt;
            mat[ip][ip] += visc[ip];
            mat[ip][ip] += nsvcl[ip];
            for (int ip2 = 0; ip2 < N; ++ip2) {
                mat[ip][ip2] -= upwind->upShapeIp[ip][ip2] * nsvcl[ip];
                mat[ip][ip2] += nsvdl[ip] * (upwind->upShapeIp[ip][ip2] - upwind->downShapeIp[ip][ip2]);
            }
        }
        if (!dense_inverse(N, mat, inv)) throw std::runtime_error("Could not compute inverse.");
        // contributions per (velocity component, corner); every pass over d rewrites all of them
        number contVel[3][MAXCO][MAXSCVF], contP[MAXCO][MAXSCVF], x[MAXSCVF];
        for (int d = 0; d < dim; ++d) {
            for (int ip = 0; ip < N; ++ip) {
                const SCVF& scvf = geo.scvf[ip];
                for (int k = 0; k < nsh; ++k) {
                    contP[k][ip] = -1.0 * scvf.globalGrad[k][d] / density;
                    contVel[d][k][ip] = visc[ip] * scvf.shape[k];
                    contVel[d][k][ip] += nsvcl[ip] * upwind->upShapeSh[ip][k];
                    contVel[d][k][ip] += nsvdl[ip] * (upwind->downShapeSh[ip][k] - upwind->upShapeSh[ip][k]);
                    for (int d2 = 0; d2 < dim; ++d2) {
                        if (d2 == d) continue;
                        contVel[d][k][ip] -= vStdVel[ip][d2] * scvf.globalGrad[k][d2];
                        contVel[d2][k][ip] = vStdVel[ip][d] * scvf.globalGrad[k][d2];
                    }
                }
            }
            for (int k = 0; k < nsh; ++k) {
                inv_apply(N, inv, contP[k], x);
                for (int ip = 0; ip < N; ++ip) stabShapeP[ip][d][k] = x[ip];
                for (int d2 = 0; d2 < dim; ++d2) {
                    inv_apply(N, inv, contVel[d2][k], x);
                    for (int ip = 0; ip < N; ++ip) stabShapeVel[ip][d][d2][k] = x[ip];
                }
            }
            number f[MAXSCVF];
            for (int ip = 0; ip < N; ++ip) f[ip] = 0.0;
            for (int k = 0; k < nsh; ++k) {
                for (int d2 = 0; d2 < dim; ++d2)
                    for (int ip = 0; ip < N; ++ip) f[ip] = 1.0 * f[ip] + u[d2 * nsh + k] * contVel[d2][k][ip];
                for (int ip = 0; ip < N; ++ip) f[ip] = 1.0 * f[ip] + u[P * nsh + k] * contP[k][ip];
            }
            for (int ip = 0; ip < N; ++ip) {
                const SCVF& scvf = geo.scvf[ip];
                if (pSource != nullptr) f[ip] += pSource[d];
                if (uOld != nullptr) {
                    number oldIPVel = 0.0;
                    for (int sh = 0; sh < nsh; ++sh) oldIPVel += scvf.shape[sh] * uOld[d * nsh + sh];
                    f[ip] += oldIPVel / dt;
                }
            }
            inv_apply(N, inv, f, x);
            for (int ip = 0; ip < N; ++ip) stabVel[ip][d] = x[ip];
        }
    }

    void update(const FV1Geometry& geo, const number* u, const number vStdVel[][3], bool bStokes,
                number kinVisco, number density, const number* pSource, const number* uOld, number dt) {
        const int dim = geo.dim, nsh = geo.nsh, P = dim, numIp = geo.nscvf;
        if (type == STAB_WITHOUT) {
            // NavierStokesFV1WithoutStabilization::update (stabilization.cpp:805-850)
            if (!bStokes) { if (!upwind) throw std::runtime_error("no upwind object"); upwind->update_upwind(geo, vStdVel); }
            for (int ip = 0; ip < numIp; ++ip)
                for (int i = 0; i < dim; ++i)
                    for (int sh = 0; sh < nsh; ++sh) stabShapeP[ip][i][sh] = 0;
            for (int ip = 0; ip < numIp; ++ip) {
                const SCVF& scvf = geo.scvf[ip];
                for (int sh = 0; sh < nsh; ++sh) {
                    const number val = scvf.shape[sh];
                    for (int i = 0; i < dim; ++i) {
                        for (int j = 0; j < dim; ++j) stabShapeVel[ip][i][j][sh] = 0;
                        stabShapeVel[ip][i][i][sh] = val;
                    }
                }
                for (int d = 0; d < 3; ++d) stabVel[ip][d] = vStdVel[ip][d];
            }
            return;
        }
        const bool flow = (type == STAB_FLOW);
        // compute_upwind / compute_downwind (stabilization.cpp:143, 457-461)
        if (!bStokes) {
            if (!upwind) throw std::runtime_error("no upwind object");
            upwind->update_upwind(geo, vStdVel);
            if (flow) upwind->update_downwind(geo, vStdVel);
        }
        diff_length(diffLengthType, geo, diffLenSqInv);   // compute_diff_length (stabilization.cpp:102-116)

        number vViscoPerDiffLenSq[MAXSCVF], vNormStdVelPerConvLen[MAXSCVF], vNormStdVelPerDownLen[MAXSCVF];
        for (int ip = 0; ip < numIp; ++ip) vViscoPerDiffLenSq[ip] = kinVisco * diffLenSqInv[ip];
        if (!bStokes)
            for (int ip = 0; ip < numIp; ++ip) {
                const number norm = vnorm(dim, vStdVel[ip]);
                vNormStdVelPerConvLen[ip] = norm / upwind->upConvLength[ip];
                if (flow) vNormStdVelPerDownLen[ip] = norm / (upwind->downConvLength[ip] + upwind->upConvLength[ip]);
            }

        if (!bStokes && upwind->non_zero_shape_ip()) {
            if (flow) nondiag_flow(geo, u, vStdVel, density, pSource, uOld, dt, vViscoPerDiffLenSq, vNormStdVelPerConvLen, vNormStdVelPerDownLen);
            else nondiag_fields(geo, u, density, pSource, uOld, dt, vViscoPerDiffLenSq, vNormStdVelPerConvLen);
            return;
        }
        for (int ip = 0; ip < numIp; ++ip) {
            const SCVF& scvf = geo.scvf[ip];
            number diag = vViscoPerDiffLenSq[ip];
            if (uOld != nullptr) diag += 1. / dt;
            if (!bStokes) diag += vNormStdVelPerConvLen[ip];
            for (int d = 0; d < dim; ++d) {
                number rhs = 0.0;
                if (pSource != nullptr) rhs = pSource[d];
                if (uOld != nullptr) {
                    number oldIPVel = 0.0;
                    for (int sh = 0; sh < nsh; ++sh) oldIPVel += scvf.shape[sh] * uOld[d * nsh + sh];
                    rhs += oldIPVel / dt;
                }
                for (int k = 0; k < nsh; ++k) {
                    number sumVel = vViscoPerDiffLenSq[ip] * scvf.shape[k];
                    if (!bStokes) {
                        sumVel += vNormStdVelPerConvLen[ip] * upwind->upShapeSh[ip][k];
                        if (flow)
                            sumVel += vNormStdVelPerDownLen[ip] * (upwind->downShapeSh[ip][k] - upwind->upShapeSh[ip][k]);
                    }
                    if (flow)
                        for (int d2 = 0; d2 < dim; ++d2) {
                            if (d2 == d) continue;
                            sumVel -= vStdVel[ip][d2] * scvf.globalGrad[k][d2];
                        }
                    rhs += sumVel * u[d * nsh + k];
                    stabShapeVel[ip][d][d][k] = sumVel / diag;
                    if (flow)
                        for (int d2 = 0; d2 < dim; ++d2) {
                            if (d2 == d) continue;
                            const number sumVel2 = vStdVel[ip][d] * scvf.globalGrad[k][d2];
                            rhs += sumVel2 * u[d2 * nsh + k];
                            stabShapeVel[ip][d][d2][k] = sumVel2 / diag;
                        }
                    const number sumP = -1.0 * scvf.globalGrad[k][d] / density;
                    rhs += sumP * u[P * nsh + k];
                    stabShapeP[ip][d][k] = sumP / diag;
                }
                stabVel[ip][d] = rhs / diag;
            }
        }
    }
};

/* ------------------------------------------------------------------------ */
/* NavierStokesFV1 element disc (incompressible/fv1/navier_stokes_fv1.cpp)  */
/* ------------------------------------------------------------------------ */
struct Disc {
    int dim;
    number kinVisco = 0.0;
    bool viscoSet = false;
    number density = 1.0;          // init() sets density 1 (navier_stokes_fv1.cpp:82)
    bool hasSource = false;
    number source[3] = {0, 0, 0};
    number fullNewtonFactor = 0.0; // navier_stokes_base.cpp:57
    bool bStokes = false, bLaplace = false, bPecletBlend = false;   // incompressible_navier_stokes_base.cpp:57-59
    Stab stab;
    bool stabSet = false;
    Upwind convUpwind;
    bool convUpwindSet = false;
    Upwind ownStabUpwind;          // used when the stabilisation's upwind differs from the convection upwind
    bool stabHasOwnUpwind = false;
    bool pac = false;              // the stabilisation is the convective upwind (set_pac_upwind)

    explicit Disc(int d) : dim(d) {}

    // set_pac_upwind(true) (navier_stokes_fv1.h:217-225): the stabilisation takes the
    // convection's upwind object and becomes the convective upwind itself
    // (m_spConvStab = m_spStab, m_spConvUpwind = SPNULL); false changes nothing
    void set_pac_upwind(bool on) {
        if (!on) return;
        if (!convUpwindSet) throw std::runtime_error("Upwind must be specified previously.");
        if (!stabSet) throw std::runtime_error("Stabilization must be specified previously.");
        stab.upwind = &convUpwind;
        stabHasOwnUpwind = false;
        pac = true;
    }

    // set_upwind(name) (navier_stokes_fv1.h:213-215); upwind shared with the stabilisation
    void set_upwind(int t) {
        pac = false;   // set_upwind(name) clears m_spConvStab
        // a new upwind object: a stabilisation that shared the previous one keeps it
        if (stab.upwind == &convUpwind) { ownStabUpwind = convUpwind; stabHasOwnUpwind = true; stab.upwind = &ownStabUpwind; }
        convUpwind.type = t; convUpwindSet = true;
        if (stabSet && stab.upwind == nullptr) stab.upwind = &convUpwind;
    }
    // set_stabilization(name[, diffLength]) (navier_stokes_fv1.h:190-199)
    void set_stabilization(int t, int dl) {
        stab = Stab();
        stab.type = t; stab.diffLengthType = dl; stabSet = true; stabHasOwnUpwind = false;
        if (convUpwindSet) stab.upwind = &convUpwind;
    }
    // INavierStokesFV1Stabilization::set_upwind with an upwind object of its own (stabilization.h:91-95)
    void set_stabilization_upwind(int t) {
        ownStabUpwind.type = t; stabHasOwnUpwind = true; stab.upwind = &ownStabUpwind;
    }

    // prep_elem_loop checks (navier_stokes_fv1.cpp:136-199)
    void check() const {
        if (!stabSet) throw std::runtime_error("Stabilization has not been set.");
        if (!bStokes && !convUpwindSet) throw std::runtime_error("Upwinding for convective Term in Momentum eq. not set.");
        if (!viscoSet) throw std::runtime_error("Kinematic Viscosity has not been set, but is required.");
    }

    void std_vel(const FV1Geometry& geo, const number* u, number StdVel[][3]) const {
        for (int ip = 0; ip < geo.nscvf; ++ip) {
            const SCVF& scvf = geo.scvf[ip];
            for (int d = 0; d < 3; ++d) StdVel[ip][d] = 0.0;
            for (int sh = 0; sh < geo.nsh; ++sh)
                for (int d1 = 0; d1 < dim; ++d1) StdVel[ip][d1] += u[d1 * geo.nsh + sh] * scvf.shape[sh];
        }
    }

    void update_stab_and_upwind(const FV1Geometry& geo, const number* u, const number StdVel[][3], const number* uOld, number dt) {
        stab.update(geo, u, StdVel, bStokes, kinVisco, density, hasSource ? source : nullptr, uOld, dt);
        if (!bStokes)
            if (stab.upwind != &convUpwind) convUpwind.update_upwind(geo, StdVel);
    }

    // peclet_blend (navier_stokes_fv1.cpp:871-892)
    number peclet_blend(number* UpwindVel, const FV1Geometry& geo, int ip, const number* StdVel, number kv) const {
        const SCVF& scvf = geo.scvf[ip];
        number vn = 0, nn = 0;
        for (int d = 0; d < dim; ++d) { vn += StdVel[d] * scvf.normal[d]; nn += scvf.normal[d] * scvf.normal[d]; }
        const number Pe = vn / nn * vdist(dim, geo.corners[scvf.to], geo.corners[scvf.from]) / kv;
        const number Pe2 = Pe * Pe;
        const number w = Pe2 / (5.0 + Pe2);
        for (int d = 0; d < dim; ++d) UpwindVel[d] = w * UpwindVel[d] + (1.0 - w) * StdVel[d];
        return w;
    }

    // add_def_A_elem (navier_stokes_fv1.cpp:597-778)
    void add_def_A_elem(number* dloc, const FV1Geometry& geo, const number* u, const number* uOld, number dt) {
        const int nsh = geo.nsh, P = dim;
        number StdVel[MAXSCVF][3];
        std_vel(geo, u, StdVel);
        update_stab_and_upwind(geo, u, StdVel, uOld, dt);
        const number nu = kinVisco, rho = density;
        for (int ip = 0; ip < geo.nscvf; ++ip) {
            const SCVF& scvf = geo.scvf[ip];
            const int from = scvf.from, to = scvf.to;
            number gradVel[3][3];
            for (int d1 = 0; d1 < dim; ++d1)
                for (int d2 = 0; d2 < dim; ++d2) {
                    gradVel[d1][d2] = 0.0;
                    for (int sh = 0; sh < nsh; ++sh) gradVel[d1][d2] += scvf.globalGrad[sh][d2] * u[d1 * nsh + sh];
                }
            number diffFlux[3];
            for (int d1 = 0; d1 < dim; ++d1) {
                diffFlux[d1] = 0.0;
                for (int d2 = 0; d2 < dim; ++d2) diffFlux[d1] += gradVel[d1][d2] * scvf.normal[d2];
            }
            if (!bLaplace)
                for (int d1 = 0; d1 < dim; ++d1)
                    for (int d2 = 0; d2 < dim; ++d2) diffFlux[d1] += gradVel[d2][d1] * scvf.normal[d2];
            for (int d1 = 0; d1 < dim; ++d1) diffFlux[d1] *= (-1.0) * nu * rho;
            for (int d1 = 0; d1 < dim; ++d1) {
                dloc[d1 * nsh + from] += diffFlux[d1];
                dloc[d1 * nsh + to] -= diffFlux[d1];
            }
            if (!bStokes) {
                number UpwindVel[3];
                // PAC: the stabilised velocity is the upwind velocity (navier_stokes_fv1.cpp:707-712)
                if (pac) for (int d = 0; d < 3; ++d) UpwindVel[d] = stab.stabVel[ip][d];
                else convUpwind.upwind_vel(geo, ip, u, StdVel, UpwindVel);
                if (bPecletBlend) peclet_blend(UpwindVel, geo, ip, StdVel[ip], nu);
                number prod = 0;
                for (int d = 0; d < dim; ++d) prod += StdVel[ip][d] * scvf.normal[d];
                prod *= rho;
                for (int d1 = 0; d1 < dim; ++d1) {
                    dloc[d1 * nsh + from] += UpwindVel[d1] * prod;
                    dloc[d1 * nsh + to] -= UpwindVel[d1] * prod;
                }
            }
            number pressure = 0.0;
            for (int sh = 0; sh < nsh; ++sh) pressure += scvf.shape[sh] * u[P * nsh + sh];
            for (int d1 = 0; d1 < dim; ++d1) {
                dloc[d1 * nsh + from] += pressure * scvf.normal[d1];
                dloc[d1 * nsh + to] -= pressure * scvf.normal[d1];
            }
            number contFlux = 0;
            for (int d = 0; d < dim; ++d) contFlux += stab.stabVel[ip][d] * scvf.normal[d];
            contFlux *= rho;
            dloc[P * nsh + from] += contFlux;
            dloc[P * nsh + to] -= contFlux;
        }
    }

    // add_jac_A_elem (navier_stokes_fv1.cpp:250-595), upwind (not PAC) branches
    void add_jac_A_elem(number* J, const FV1Geometry& geo, const number* u, const number* uOld, number dt) {
        const int nsh = geo.nsh, P = dim, b = dim + 1;
        auto Jx = [&](int f1, int s1, int f2, int s2) -> number& { return J[((f1 * nsh + s1) * b + f2) * nsh + s2]; };
        number StdVel[MAXSCVF][3];
        std_vel(geo, u, StdVel);
        update_stab_and_upwind(geo, u, StdVel, uOld, dt);
        const number nu = kinVisco, rho = density;
        for (int ip = 0; ip < geo.nscvf; ++ip) {
            const SCVF& scvf = geo.scvf[ip];
            const int from = scvf.from, to = scvf.to;
            for (int sh = 0; sh < nsh; ++sh) {
                // diffusion (:336-356)
                number gn = 0;
                for (int d = 0; d < dim; ++d) gn += scvf.globalGrad[sh][d] * scvf.normal[d];
                const number flux_sh = -1.0 * nu * rho * gn;
                for (int d1 = 0; d1 < dim; ++d1) { Jx(d1, from, d1, sh) += flux_sh; Jx(d1, to, d1, sh) -= flux_sh; }
                if (!bLaplace)
                    for (int d1 = 0; d1 < dim; ++d1)
                        for (int d2 = 0; d2 < dim; ++d2) {
                            const number flux2_sh = -1.0 * nu * rho * scvf.globalGrad[sh][d1] * scvf.normal[d2];
                            Jx(d1, from, d2, sh) += flux2_sh;
                            Jx(d1, to, d2, sh) -= flux2_sh;
                        }
                // pressure (:362-368)
                for (int d1 = 0; d1 < dim; ++d1) {
                    const number fl = scvf.shape[sh] * scvf.normal[d1];
                    Jx(d1, from, P, sh) += fl;
                    Jx(d1, to, P, sh) -= fl;
                }
                // convection (:377-552)
                if (!bStokes) {
                    number UpwindVel[3];
                    if (pac) for (int d = 0; d < 3; ++d) UpwindVel[d] = stab.stabVel[ip][d];
                    else convUpwind.upwind_vel(geo, ip, u, StdVel, UpwindVel);
                    number w = 1.0;
                    if (bPecletBlend) w = peclet_blend(UpwindVel, geo, ip, StdVel[ip], nu);
                    number prod = 0;
                    for (int d = 0; d < dim; ++d) prod += StdVel[ip][d] * scvf.normal[d];
                    prod *= rho;
                    if (pac) {
                        // stabilisation used as upwind, fixpoint part (:398-427)
                        if (stab.vel_comp_connected())
                            for (int d1 = 0; d1 < dim; ++d1)
                                for (int d2 = 0; d2 < dim; ++d2) {
                                    const number cf = prod * w * stab.stabShapeVel[ip][d1][d2][sh];
                                    Jx(d1, from, d2, sh) += cf;
                                    Jx(d1, to, d2, sh) -= cf;
                                }
                        else
                            for (int d1 = 0; d1 < dim; ++d1) {
                                const number cf = prod * w * stab.stabShapeVel[ip][d1][d1][sh];
                                Jx(d1, from, d1, sh) += cf;
                                Jx(d1, to, d1, sh) -= cf;
                            }
                        for (int d1 = 0; d1 < dim; ++d1) {
                            const number cfp = prod * w * stab.stabShapeP[ip][d1][sh];
                            Jx(d1, from, P, sh) += cfp;
                            Jx(d1, to, P, sh) -= cfp;
                        }
                    } else {
                        number convFlux_vel = convUpwind.upShapeSh[ip][sh];
                        // ip shapes: the ip velocities interpolated from the corners (:431-447)
                        if (convUpwind.non_zero_shape_ip())
                            for (int ip2 = 0; ip2 < geo.nscvf; ++ip2) convFlux_vel += geo.scvf[ip2].shape[sh] * convUpwind.upShapeIp[ip][ip2];
                        convFlux_vel *= prod * w;
                        for (int d1 = 0; d1 < dim; ++d1) { Jx(d1, from, d1, sh) += convFlux_vel; Jx(d1, to, d1, sh) -= convFlux_vel; }
                    }
                    if (bPecletBlend) {
                        const number convFluxPe = prod * (1.0 - w) * scvf.shape[sh];
                        for (int d1 = 0; d1 < dim; ++d1) { Jx(d1, from, d1, sh) += convFluxPe; Jx(d1, to, d1, sh) -= convFluxPe; }
                    }
                    if (fullNewtonFactor != 0.0 && pac) {
                        // stabilisation used as upwind (:477-518): the non-connected branch takes the
                        // (d1, d1) shape for every column d2 and no blending weight, as the reference does
                        for (int d1 = 0; d1 < dim; ++d1) {
                            for (int d2 = 0; d2 < dim; ++d2) {
                                number prod_vel = 0.0;
                                if (stab.vel_comp_connected())
                                    for (int k = 0; k < dim; ++k) prod_vel += w * stab.stabShapeVel[ip][k][d2][sh] * scvf.normal[k];
                                else
                                    prod_vel = stab.stabShapeVel[ip][d1][d1][sh] * scvf.normal[d1];
                                prod_vel *= fullNewtonFactor * rho;
                                Jx(d1, from, d2, sh) += prod_vel * UpwindVel[d1];
                                Jx(d1, to, d2, sh) -= prod_vel * UpwindVel[d1];
                            }
                            number prod_p = 0.0;
                            for (int k = 0; k < dim; ++k) prod_p += stab.stabShapeP[ip][k][sh] * scvf.normal[k];
                            prod_p *= fullNewtonFactor * rho;
                            Jx(d1, from, P, sh) += prod_p * UpwindVel[d1];
                            Jx(d1, to, P, sh) -= prod_p * UpwindVel[d1];
                        }
                    }
                    if (fullNewtonFactor != 0.0) {
                        // upwind branch (:521-534): the factor itself is not applied here
                        if (!pac)
                        for (int d1 = 0; d1 < dim; ++d1)
                            for (int d2 = 0; d2 < dim; ++d2) {
                                const number prod_vel = w * convUpwind.upShapeSh[ip][sh] * scvf.normal[d2] * rho;
                                Jx(d1, from, d2, sh) += prod_vel * UpwindVel[d1];
                                Jx(d1, to, d2, sh) -= prod_vel * UpwindVel[d1];
                            }
                        if (bPecletBlend)
                            for (int d1 = 0; d1 < dim; ++d1)
                                for (int d2 = 0; d2 < dim; ++d2) {
                                    const number convFluxPe = UpwindVel[d1] * (1.0 - w) * scvf.shape[sh] * scvf.normal[d2] * rho;
                                    Jx(d1, from, d2, sh) += convFluxPe;
                                    Jx(d1, to, d2, sh) -= convFluxPe;
                                }
                    }
                }
                // continuity (:560-592)
                if (stab.vel_comp_connected()) {
                    for (int d1 = 0; d1 < dim; ++d1) {
                        number contFlux_vel = 0.0;
                        for (int d2 = 0; d2 < dim; ++d2) contFlux_vel += stab.stabShapeVel[ip][d2][d1][sh] * scvf.normal[d2] * rho;
                        Jx(P, from, d1, sh) += contFlux_vel;
                        Jx(P, to, d1, sh) -= contFlux_vel;
                    }
                } else {
                    for (int d1 = 0; d1 < dim; ++d1) {
                        const number contFlux_vel = stab.stabShapeVel[ip][d1][d1][sh] * scvf.normal[d1] * rho;
                        Jx(P, from, d1, sh) += contFlux_vel;
                        Jx(P, to, d1, sh) -= contFlux_vel;
                    }
                }
                number contFlux_p = 0.0;
                for (int d1 = 0; d1 < dim; ++d1) contFlux_p += stab.stabShapeP[ip][d1][sh] * scvf.normal[d1] * rho;
                Jx(P, from, P, sh) += contFlux_p;
                Jx(P, to, P, sh) -= contFlux_p;
            }
        }
    }

    // add_jac_M_elem (:781-808)
    void add_jac_M_elem(number* J, const FV1Geometry& geo) const {
        const int nsh = geo.nsh, b = dim + 1;
        for (int ip = 0; ip < geo.nscv; ++ip) {
            const int sh = geo.scv[ip].nodeId;
            for (int d1 = 0; d1 < dim; ++d1) J[((d1 * nsh + sh) * b + d1) * nsh + sh] += geo.scv[ip].vol * density;
        }
    }
    // add_def_M_elem (:811-838)
    void add_def_M_elem(number* dloc, const FV1Geometry& geo, const number* u) const {
        const int nsh = geo.nsh;
        for (int ip = 0; ip < geo.nscv; ++ip) {
            const int sh = geo.scv[ip].nodeId;
            for (int d1 = 0; d1 < dim; ++d1) dloc[d1 * nsh + sh] += u[d1 * nsh + sh] * geo.scv[ip].vol * density;
        }
    }
    // add_rhs_elem (:841-869)
    void add_rhs_elem(number* dloc, const FV1Geometry& geo) const {
        if (!hasSource) return;
        const int nsh = geo.nsh;
        for (int ip = 0; ip < geo.nscv; ++ip) {
            const int sh = geo.scv[ip].nodeId;
            for (int d1 = 0; d1 < dim; ++d1) dloc[d1 * nsh + sh] += source[d1] * geo.scv[ip].vol * density;
        }
    }
};

/* ------------------------------------------------------------------------ */
/* Global assembly (the ugcore element loop, restated): block-CSR pattern,    */
/* greedy element colouring, defect/Jacobian, Dirichlet rows.               */
/* Stationary:  d = A(u) - F,                     J = dA/du                  */
/* Transient (implicit Euler, theta = 1):                                   */
/*              d = M(u) - M(u_old) + dt (A(u) - F), J = M + dt dA/du          */
/* ------------------------------------------------------------------------ */
struct Mesh {
    int roid = 0, dim = 0, nsh = 0;
    int64_t nNodes = 0, nElems = 0;
    std::vector<number> coords;       // nNodes * dim
    std::vector<int32_t> conn;        // nElems * nsh
    std::vector<int32_t> rowPtr, colIdx;
    std::vector<int64_t> elemBlk;     // nElems * nsh * nsh block positions
    std::vector<int32_t> color;
    int nColors = 0;
    std::vector<int32_t> colorPtr, colorElems;
};

static void build_pattern(Mesh& m) {
    const int nsh = m.nsh;
    std::vector<std::vector<int32_t>> rows(m.nNodes);
    for (int64_t e = 0; e < m.nElems; ++e)
        for (int i = 0; i < nsh; ++i)
            for (int j = 0; j < nsh; ++j) rows[m.conn[e * nsh + i]].push_back(m.conn[e * nsh + j]);
    m.rowPtr.assign(m.nNodes + 1, 0);
    for (int64_t r = 0; r < m.nNodes; ++r) {
        auto& v = rows[r];
        std::sort(v.begin(), v.end());
        v.erase(std::unique(v.begin(), v.end()), v.end());
        m.rowPtr[r + 1] = m.rowPtr[r] + (int32_t)v.size();
    }
    m.colIdx.resize(m.rowPtr[m.nNodes]);
    for (int64_t r = 0; r < m.nNodes; ++r) std::copy(rows[r].begin(), rows[r].end(), m.colIdx.begin() + m.rowPtr[r]);
    m.elemBlk.resize(m.nElems * nsh * nsh);
    for (int64_t e = 0; e < m.nElems; ++e)
        for (int i = 0; i < nsh; ++i) {
            const int32_t r = m.conn[e * nsh + i];
            const int32_t* b = m.colIdx.data() + m.rowPtr[r];
            const int32_t* en = m.colIdx.data() + m.rowPtr[r + 1];
            for (int j = 0; j < nsh; ++j) {
                const int32_t c = m.conn[e * nsh + j];
                m.elemBlk[(e * nsh + i) * nsh + j] = (int64_t)(std::lower_bound(b, en, c) - m.colIdx.data());
            }
        }
}

// greedy colouring in element order: smallest colour not used by an earlier element sharing a node
static void build_coloring(Mesh& m) {
    const int nsh = m.nsh;
    std::vector<int32_t> nptr(m.nNodes + 1, 0), nel;
    for (int64_t k = 0; k < m.nElems * nsh; ++k) nptr[m.conn[k] + 1]++;
    for (int64_t r = 0; r < m.nNodes; ++r) nptr[r + 1] += nptr[r];
    nel.resize(nptr[m.nNodes]);
    std::vector<int32_t> fill(nptr.begin(), nptr.end() - 1);
    for (int64_t e = 0; e < m.nElems; ++e)
        for (int i = 0; i < nsh; ++i) nel[fill[m.conn[e * nsh + i]]++] = (int32_t)e;
    m.color.assign(m.nElems, -1);
    std::vector<int64_t> mark(256, -1);
    int nc = 0;
    for (int64_t e = 0; e < m.nElems; ++e) {
        for (int i = 0; i < nsh; ++i) {
            const int32_t n = m.conn[e * nsh + i];
            for (int32_t k = nptr[n]; k < nptr[n + 1]; ++k) {
                const int32_t o = nel[k];
                if (o < e && m.color[o] >= 0) mark[m.color[o]] = e;
            }
        }
        int c = 0;
        while (mark[c] == e) ++c;
        m.color[e] = c;
        if (c + 1 > nc) nc = c + 1;
        if (nc >= 255) throw std::runtime_error("too many colours");
    }
    m.nColors = nc;
    m.colorPtr.assign(nc + 1, 0);
    for (int64_t e = 0; e < m.nElems; ++e) m.colorPtr[m.color[e] + 1]++;
    for (int c = 0; c < nc; ++c) m.colorPtr[c + 1] += m.colorPtr[c];
    m.colorElems.resize(m.nElems);
    std::vector<int32_t> f(m.colorPtr.begin(), m.colorPtr.end() - 1);
    for (int64_t e = 0; e < m.nElems; ++e) m.colorElems[f[m.color[e]]++] = (int32_t)e;
}

// one boundary face of an outflow side (NavierStokesNoNormalStressOutflowFV1): the
// part of the side belonging to one of its corners
struct OutflowBF {
    int64_t elem;      // the element the side belongs to
    int local;         // the corner's index in the element
    number xi[3];      // local coordinates of the face's integration point
    number n[3];       // outward area-weighted normal
};

struct Problem {
    Disc disc;
    Mesh mesh;
    std::vector<int32_t> dirRow;   // node * b + fct
    std::vector<number> dirVal;
    std::vector<number> bndFlux;   // continuity right-hand side of inflow boundaries, per node
    std::vector<OutflowBF> outflow;
    std::string lastError;
    explicit Problem(int dim) : disc(dim) {}
};

/* ------------------------------------------------------------------------ */
/* Boundary element discs (incompressible/bnd/wall_impl.h:57-69,            */
/* incompressible/fv1/bnd/inflow_fv1_impl.h:57-82) with ugcore's            */
/* DirichletBoundary and NeumannBoundaryFV1 (absent) restated:              */
/*  - Dirichlet rows: defect u - g, Jacobian identity row; a later value for */
/*    the same unknown replaces an earlier one;                             */
/*  - NeumannBoundaryFV1 with vector data j on the pressure function: the    */
/*    right-hand side of the continuity row of every boundary corner gets    */
/*    -(j . n_bf), n_bf the outward normal of the corner's boundary face     */
/*    (the part {corner, side-edge midpoints, side centre} of the side), so  */
/*    the defect d = A(u) - F gets + j . n_bf (dt-scaled when transient).    */
/* ------------------------------------------------------------------------ */
static void merge_dirichlet(Problem& P, const std::vector<int32_t>& rows, const std::vector<number>& vals) {
    std::vector<std::pair<int32_t, number>> all;
    for (size_t k = 0; k < P.dirRow.size(); ++k) all.emplace_back(P.dirRow[k], P.dirVal[k]);
    for (size_t k = 0; k < rows.size(); ++k) all.emplace_back(rows[k], vals[k]);
    std::stable_sort(all.begin(), all.end(), [](const std::pair<int32_t, number>& a, const std::pair<int32_t, number>& c) { return a.first < c.first; });
    P.dirRow.clear();
    P.dirVal.clear();
    for (auto& x : all) {
        if (!P.dirRow.empty() && P.dirRow.back() == x.first) P.dirVal.back() = x.second;
        else { P.dirRow.push_back(x.first); P.dirVal.push_back(x.second); }
    }
}

// outward area-weighted normal of the boundary face of side corner j
static void boundary_face_normal(int dim, int nco, const number x[][3], int j, const number* elemCen, number* n) {
    number sc[3] = {0, 0, 0};
    for (int k = 0; k < nco; ++k) for (int d = 0; d < 3; ++d) sc[d] += x[k][d];
    for (int d = 0; d < 3; ++d) sc[d] /= nco;
    if (dim == 2) {
        // the half side from corner j to the side midpoint
        const number* a = x[j];
        const number* o = x[1 - j];
        number t[2] = {0.5 * (o[0] - a[0]), 0.5 * (o[1] - a[1])};
        n[0] = t[1]; n[1] = -t[0]; n[2] = 0.0;
    } else {
        // quadrilateral {a, mid(a, next), side centre, mid(prev, a)}: half the cross product of its diagonals
        const number* a = x[j];
        const number* nx = x[(j + 1) % nco];
        const number* pv = x[(j + nco - 1) % nco];
        number d1[3], d2[3];
        for (int d = 0; d < 3; ++d) { d1[d] = sc[d] - a[d]; d2[d] = 0.5 * (pv[d] + a[d]) - 0.5 * (a[d] + nx[d]); }
        cross3(d1, d2, n);
        for (int d = 0; d < 3; ++d) n[d] *= 0.5;
    }
    number dot = 0;
    for (int d = 0; d < dim; ++d) dot += n[d] * (sc[d] - elemCen[d]);
    if (dot < 0) for (int d = 0; d < 3; ++d) n[d] = -n[d];
}

static void gather_elem(const Mesh& m, int64_t e, const number* U, number* corners, number* uloc, int b) {
    const int nsh = m.nsh, dim = m.dim;
    for (int i = 0; i < nsh; ++i) {
        const int32_t n = m.conn[e * nsh + i];
        for (int d = 0; d < dim; ++d) corners[i * dim + d] = m.coords[n * dim + d];
        if (U) for (int f = 0; f < b; ++f) uloc[f * nsh + i] = U[(int64_t)n * b + f];
    }
}

// one element: the full local defect / Jacobian of the time discretisation above
static void elem_local(Disc& disc, FV1Geometry& geo, const number* corners, int roid, const number* uloc, const number* uoldloc,
                       number dt, bool transient, number* dloc, number* Jloc) {
    const int nsh = ref_elem(roid).nco, b = disc.dim + 1, n = b * nsh;
    geo.update(roid, corners);   // prep_elem (navier_stokes_fv1.cpp:208-248)
    if (dloc) {
        number dA[4 * MAXCO], dM[4 * MAXCO], dMo[4 * MAXCO], f[4 * MAXCO];
        std::fill(dA, dA + n, 0.0); std::fill(f, f + n, 0.0);
        disc.add_def_A_elem(dA, geo, uloc, transient ? uoldloc : nullptr, dt);
        disc.add_rhs_elem(f, geo);
        if (transient) {
            std::fill(dM, dM + n, 0.0); std::fill(dMo, dMo + n, 0.0);
            disc.add_def_M_elem(dM, geo, uloc);
            disc.add_def_M_elem(dMo, geo, uoldloc);
            for (int k = 0; k < n; ++k) dloc[k] = (dM[k] - dMo[k]) + dt * (dA[k] - f[k]);
        } else {
            for (int k = 0; k < n; ++k) dloc[k] = dA[k] - f[k];
        }
    }
    if (Jloc) {
        std::vector<number> JA(n * n, 0.0);
        disc.add_jac_A_elem(JA.data(), geo, uloc, transient ? uoldloc : nullptr, dt);
        if (transient) {
            std::vector<number> JM(n * n, 0.0);
            disc.add_jac_M_elem(JM.data(), geo);
            for (int k = 0; k < n * n; ++k) Jloc[k] = JM[k] + dt * JA[k];
        } else {
            for (int k = 0; k < n * n; ++k) Jloc[k] = JA[k];
        }
    }
}

/* NavierStokesNoNormalStressOutflowFV1 (no_normal_stress_outflow_fv1.cpp:343-504) on one
 * boundary face, into the element-local defect / Jacobian (row bf.local), scaled by sc:
 * momentum: the viscous flux -nu rho ((grad u + grad u^T) n) minus its part along the
 * area-weighted n (v + (-(v.n)) n, as the reference writes it), the outgoing convective
 * flux max(rho u.n, 0) u; continuity rho u.n; the Jacobian of the viscous and continuity
 * terms and of the convective one with the flux frozen. */
static void outflow_face_terms(const Disc& disc, int roid, const number* corners, const number* uloc, const OutflowBF& bf, number sc,
                               number* dloc, number* Jloc) {
    const RefElem& R = ref_elem(roid);
    const int dim = R.dim, nsh = R.nco, b = dim + 1, Pc = dim, node = bf.local;
    number N[MAXCO], LG[MAXCO][3], J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, JtInv[3][3], G[MAXCO][3];
    p1_shapes(roid, bf.xi, N);
    p1_grads(roid, bf.xi, LG);
    for (int k = 0; k < nsh; ++k)
        for (int r = 0; r < dim; ++r)
            for (int c = 0; c < dim; ++c) J[r][c] += corners[k * dim + r] * LG[k][c];
    det_and_jtinv(dim, J, JtInv);
    for (int k = 0; k < nsh; ++k)
        for (int r = 0; r < 3; ++r) {
            G[k][r] = 0;
            if (r < dim) for (int c = 0; c < dim; ++c) G[k][r] += JtInv[r][c] * LG[k][c];
        }
    const number* nn = bf.n;
    const number nu = disc.kinVisco, rho = disc.density;
    number stdVel[3] = {0, 0, 0};
    for (int d1 = 0; d1 < dim; ++d1)
        for (int sh = 0; sh < nsh; ++sh) stdVel[d1] += uloc[d1 * nsh + sh] * N[sh];
    number vn = 0;
    for (int d = 0; d < dim; ++d) vn += stdVel[d] * nn[d];
    auto Jx = [&](int f1, int s1, int f2, int s2) -> number& { return Jloc[((f1 * nsh + s1) * b + f2) * nsh + s2]; };
    if (dloc) {
        number gradVel[3][3], df[3] = {0, 0, 0};
        for (int d1 = 0; d1 < dim; ++d1)
            for (int d2 = 0; d2 < dim; ++d2) {
                gradVel[d1][d2] = 0.0;
                for (int sh = 0; sh < nsh; ++sh) gradVel[d1][d2] += G[sh][d2] * uloc[d1 * nsh + sh];
            }
        for (int d1 = 0; d1 < dim; ++d1) for (int d2 = 0; d2 < dim; ++d2) df[d1] += gradVel[d1][d2] * nn[d2];
        if (!disc.bLaplace)
            for (int d1 = 0; d1 < dim; ++d1) for (int d2 = 0; d2 < dim; ++d2) df[d1] += gradVel[d2][d1] * nn[d2];
        number dot = 0;
        for (int d = 0; d < dim; ++d) dot += df[d] * nn[d];
        for (int d = 0; d < dim; ++d) df[d] += -dot * nn[d];
        for (int d = 0; d < dim; ++d) df[d] *= -nu * rho;
        for (int d1 = 0; d1 < dim; ++d1) dloc[d1 * nsh + node] += sc * df[d1];
        if (!disc.bStokes) {
            number flux = vn * rho;
            if (flux < 0) flux = 0;
            for (int d1 = 0; d1 < dim; ++d1) dloc[d1 * nsh + node] += sc * (flux * stdVel[d1]);
        }
        dloc[Pc * nsh + node] += sc * (vn * rho);
    }
    if (Jloc) {
        for (int sh = 0; sh < nsh; ++sh) {
            number M[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, ns[3] = {0, 0, 0}, gn = 0;
            for (int d = 0; d < dim; ++d) gn += G[sh][d] * nn[d];
            for (int d = 0; d < dim; ++d) M[d][d] = gn;
            if (!disc.bLaplace)
                for (int d1 = 0; d1 < dim; ++d1) for (int d2 = 0; d2 < dim; ++d2) M[d1][d2] += G[sh][d1] * nn[d2];
            for (int d2 = 0; d2 < dim; ++d2) for (int d1 = 0; d1 < dim; ++d1) ns[d2] += M[d1][d2] * nn[d1];
            for (int d1 = 0; d1 < dim; ++d1)
                for (int d2 = 0; d2 < dim; ++d2) Jx(d1, node, d2, sh) += sc * ((M[d1][d2] - nn[d1] * ns[d2]) * (-nu * rho));
        }
        if (!disc.bStokes) {
            number old = vn * rho;
            if (old < 0) old = 0;
            for (int sh = 0; sh < nsh; ++sh)
                for (int d1 = 0; d1 < dim; ++d1) Jx(d1, node, d1, sh) += sc * (old * N[sh]);
        }
        for (int sh = 0; sh < nsh; ++sh)
            for (int d2 = 0; d2 < dim; ++d2) Jx(Pc, node, d2, sh) += sc * (N[sh] * nn[d2] * rho);
    }
}

/* The boundary faces of one element side given by its element-local corners loc[nco]
 * (cyclic order): per corner the face {corner, side-edge midpoints, side centre} (2D:
 * {corner, side midpoint}), its integration point at the mean of those points in local
 * coordinates and its outward area-weighted normal. */
static void side_outflow_faces(int roid, const number* corners, const int* loc, int nco, int64_t elem, std::vector<OutflowBF>& out) {
    const RefElem& R = ref_elem(roid);
    const int dim = R.dim, nsh = R.nco;
    number x[4][3] = {{0}}, cen[3] = {0, 0, 0}, lx[4][3] = {{0}}, lsc[3] = {0, 0, 0};
    for (int j = 0; j < nco; ++j)
        for (int d = 0; d < dim; ++d) {
            x[j][d] = corners[loc[j] * dim + d];
            lx[j][d] = R.co[loc[j]][d];
            lsc[d] += lx[j][d] / nco;
        }
    for (int i = 0; i < nsh; ++i) for (int d = 0; d < dim; ++d) cen[d] += corners[i * dim + d] / nsh;
    for (int j = 0; j < nco; ++j) {
        OutflowBF bf;
        bf.elem = elem;
        bf.local = loc[j];
        boundary_face_normal(dim, nco, x, j, cen, bf.n);
        for (int d = 0; d < 3; ++d) bf.xi[d] = 0.0;
        if (dim == 2) {
            const int o = 1 - j;
            for (int d = 0; d < 2; ++d) bf.xi[d] = 0.5 * (lx[j][d] + 0.5 * (lx[j][d] + lx[o][d]));
        } else {
            const int nx = (j + 1) % nco, pv = (j + nco - 1) % nco;
            for (int d = 0; d < 3; ++d) bf.xi[d] = 0.25 * (lx[j][d] + 0.5 * (lx[j][d] + lx[nx][d]) + lsc[d] + 0.5 * (lx[pv][d] + lx[j][d]));
        }
        out.push_back(bf);
    }
}

static void assemble(Problem& P, const number* U, const number* Uold, number dt, number* D, number* JV, int nthreads) {
    Mesh& m = P.mesh;
    P.disc.check();
    const int nsh = m.nsh, b = m.dim + 1, n = b * nsh;
    const bool transient = (Uold != nullptr);
    if (D) std::fill(D, D + m.nNodes * b, 0.0);
    if (JV) std::fill(JV, JV + (int64_t)m.colIdx.size() * b * b, 0.0);
    auto do_elem = [&](Disc& disc, int64_t e) {
        FV1Geometry geo;
        number corners[MAXCO * 3], uloc[4 * MAXCO], uold[4 * MAXCO], dloc[4 * MAXCO];
        std::vector<number> Jloc(JV ? n * n : 0);
        gather_elem(m, e, U, corners, uloc, b);
        if (transient) gather_elem(m, e, Uold, corners, uold, b);
        elem_local(disc, geo, corners, m.roid, uloc, uold, dt, transient, D ? dloc : nullptr, JV ? Jloc.data() : nullptr);
        for (int i = 0; i < nsh; ++i) {
            const int64_t row = m.conn[e * nsh + i];
            if (D) for (int f = 0; f < b; ++f) D[row * b + f] += dloc[f * nsh + i];
            if (JV)
                for (int j = 0; j < nsh; ++j) {
                    number* blk = JV + m.elemBlk[(e * nsh + i) * nsh + j] * b * b;
                    for (int f1 = 0; f1 < b; ++f1)
                        for (int f2 = 0; f2 < b; ++f2) blk[f1 * b + f2] += Jloc[((f1 * nsh + i) * b + f2) * nsh + j];
                }
        }
    };
    if (nthreads <= 1) {
        for (int64_t e = 0; e < m.nElems; ++e) do_elem(P.disc, e);
    } else {
        // colour by colour, elements of one colour in parallel (no shared nodes)
        for (int c = 0; c < m.nColors; ++c) {
#ifdef _OPENMP
#pragma omp parallel num_threads(nthreads)
#endif
            {
                Disc local = P.disc;   // per-thread scratch (the reference's disc is not re-entrant)
                if (local.stab.upwind == &P.disc.convUpwind) local.stab.upwind = &local.convUpwind;
                else if (local.stab.upwind == &P.disc.ownStabUpwind) local.stab.upwind = &local.ownStabUpwind;
#ifdef _OPENMP
#pragma omp for schedule(static)
#endif
                for (int32_t k = m.colorPtr[c]; k < m.colorPtr[c + 1]; ++k) do_elem(local, m.colorElems[k]);
            }
        }
    }
    // outflow boundaries without normal stress (no_normal_stress_outflow_fv1.cpp:343-504),
    // dt-scaled when transient like the other stiffness terms
    if (!P.outflow.empty()) {
        const number sc = transient ? dt : 1.0;
        std::vector<number> dl(n), Jl(n * n);
        for (const OutflowBF& bf : P.outflow) {
            number corners[MAXCO * 3], uloc[4 * MAXCO];
            gather_elem(m, bf.elem, U, corners, uloc, b);
            std::fill(dl.begin(), dl.end(), 0.0);
            std::fill(Jl.begin(), Jl.end(), 0.0);
            outflow_face_terms(P.disc, m.roid, corners, uloc, bf, sc, D ? dl.data() : nullptr, JV ? Jl.data() : nullptr);
            const int i = bf.local;
            const int64_t row = m.conn[bf.elem * nsh + i];
            if (D) for (int f = 0; f < b; ++f) D[row * b + f] += dl[f * nsh + i];
            if (JV)
                for (int j = 0; j < nsh; ++j) {
                    number* blk = JV + m.elemBlk[(bf.elem * nsh + i) * nsh + j] * b * b;
                    for (int f1 = 0; f1 < b; ++f1)
                        for (int f2 = 0; f2 < b; ++f2) blk[f1 * b + f2] += Jl[((f1 * nsh + i) * b + f2) * nsh + j];
                }
        }
    }
    // inflow boundaries: the continuity rows' Neumann flux (a right-hand side: dt-scaled when transient)
    if (D && !P.bndFlux.empty())
        for (int64_t r = 0; r < m.nNodes; ++r) D[r * b + (b - 1)] += (transient ? dt : 1.0) * P.bndFlux[r];
    // Dirichlet rows: defect = u - g, Jacobian row = identity (off-diagonal blocks kept in the pattern)
    for (size_t k = 0; k < P.dirRow.size(); ++k) {
        const int64_t row = P.dirRow[k] / b;
        const int f = P.dirRow[k] % b;
        if (D) D[P.dirRow[k]] = U[P.dirRow[k]] - P.dirVal[k];
        if (JV)
            for (int32_t q = m.rowPtr[row]; q < m.rowPtr[row + 1]; ++q) {
                number* blk = JV + (int64_t)q * b * b;
                for (int f2 = 0; f2 < b; ++f2) blk[f * b + f2] = (m.colIdx[q] == row && f2 == f) ? 1.0 : 0.0;
            }
    }
}

/* ------------------------------------------------------------------------ */
/* Plain method (ugcore Newton + BiCGStab + point-block Jacobi, restated)   */
/* ------------------------------------------------------------------------ */
static void bsr_mv(const Mesh& m, int b, const number* V, const number* x, number* y) {
    for (int64_t r = 0; r < m.nNodes; ++r) {
        number acc[4] = {0, 0, 0, 0};
        for (int32_t q = m.rowPtr[r]; q < m.rowPtr[r + 1]; ++q) {
            const number* blk = V + (int64_t)q * b * b;
            const number* xc = x + (int64_t)m.colIdx[q] * b;
            for (int i = 0; i < b; ++i) for (int j = 0; j < b; ++j) acc[i] += blk[i * b + j] * xc[j];
        }
        for (int i = 0; i < b; ++i) y[r * b + i] = acc[i];
    }
}

static bool invert_block(int b, const number* A, number* Ainv) {
    // Gauss-Jordan with partial pivoting
    number M[4][8];
    for (int i = 0; i < b; ++i) for (int j = 0; j < b; ++j) { M[i][j] = A[i * b + j]; M[i][b + j] = (i == j) ? 1.0 : 0.0; }
    for (int c = 0; c < b; ++c) {
        int p = c;
        for (int r = c + 1; r < b; ++r) if (std::fabs(M[r][c]) > std::fabs(M[p][c])) p = r;
        if (M[p][c] == 0.0) return false;
        if (p != c) for (int j = 0; j < 2 * b; ++j) std::swap(M[p][j], M[c][j]);
        const number piv = 1.0 / M[c][c];
        for (int j = 0; j < 2 * b; ++j) M[c][j] *= piv;
        for (int r = 0; r < b; ++r) {
            if (r == c) continue;
            const number f = M[r][c];
            if (f != 0.0) for (int j = 0; j < 2 * b; ++j) M[r][j] -= f * M[c][j];
        }
    }
    for (int i = 0; i < b; ++i) for (int j = 0; j < b; ++j) Ainv[i * b + j] = M[i][b + j];
    return true;
}

static number dot(int64_t n, const number* a, const number* c) { number s = 0; for (int64_t i = 0; i < n; ++i) s += a[i] * c[i]; return s; }

// right-preconditioned BiCGStab; returns iterations (or -1 on breakdown)
static int bicgstab(const Mesh& m, int b, const number* V, const number* Dinv, const number* rhs, number* x,
                    number rtol, int maxit, number* relres) {
    const int64_t n = m.nNodes * b;
    std::vector<number> r(n), r0(n), p(n), v(n), s(n), t(n), ph(n), sh(n);
    auto prec = [&](const number* in, number* out) {
        for (int64_t k = 0; k < m.nNodes; ++k)
            for (int i = 0; i < b; ++i) {
                number a = 0;
                for (int j = 0; j < b; ++j) a += Dinv[k * b * b + i * b + j] * in[k * b + j];
                out[k * b + i] = a;
            }
    };
    std::fill(x, x + n, 0.0);
    std::copy(rhs, rhs + n, r.begin());
    const number nr0 = std::sqrt(dot(n, r.data(), r.data()));
    *relres = 1.0;
    if (nr0 == 0.0) return 0;
    r0 = r;
    number rho = 1, alpha = 1, omega = 1;
    std::fill(p.begin(), p.end(), 0.0); std::fill(v.begin(), v.end(), 0.0);
    // breakdowns (rho = 0, (r0, v) = 0, (t, t) = 0, omega = 0) stop the iteration
    // with the last finite iterate; only a non-finite residual is a failure
    for (int it = 1; it <= maxit; ++it) {
        const number rho1 = dot(n, r0.data(), r.data());
        if (rho1 == 0.0) return it - 1;
        const number beta = (rho1 / rho) * (alpha / omega);
        for (int64_t k = 0; k < n; ++k) p[k] = r[k] + beta * (p[k] - omega * v[k]);
        prec(p.data(), ph.data());
        bsr_mv(m, b, V, ph.data(), v.data());
        const number r0v = dot(n, r0.data(), v.data());
        if (r0v == 0.0) return it - 1;
        alpha = rho1 / r0v;
        for (int64_t k = 0; k < n; ++k) s[k] = r[k] - alpha * v[k];
        const number ns = std::sqrt(dot(n, s.data(), s.data()));
        if (ns / nr0 < rtol) {
            for (int64_t k = 0; k < n; ++k) x[k] += alpha * ph[k];
            *relres = ns / nr0;
            return it;
        }
        prec(s.data(), sh.data());
        bsr_mv(m, b, V, sh.data(), t.data());
        const number tt = dot(n, t.data(), t.data());
        if (tt == 0.0) { for (int64_t k = 0; k < n; ++k) x[k] += alpha * ph[k]; return it; }
        omega = dot(n, t.data(), s.data()) / tt;
        for (int64_t k = 0; k < n; ++k) { x[k] += alpha * ph[k] + omega * sh[k]; r[k] = s[k] - omega * t[k]; }
        rho = rho1;
        const number nr = std::sqrt(dot(n, r.data(), r.data()));
        *relres = nr / nr0;
        if (!std::isfinite(nr)) return -1;
        if (*relres < rtol) return it;
        if (omega == 0.0) return it;
    }
    return maxit;
}

}  // namespace nsora

/* ======================================================================== */
/* C ABI for the Python test harness (ctypes)                               */
/* ======================================================================== */
using namespace nsora;

static std::string lower_trim(const char* s) {
    std::string n = s ? s : "";
    size_t a = n.find_first_not_of(" \t\n\r"), z = n.find_last_not_of(" \t\n\r");
    n = (a == std::string::npos) ? std::string() : n.substr(a, z - a + 1);
    std::transform(n.begin(), n.end(), n.begin(), [](unsigned char c) { return (char)std::tolower(c); });
    return n;
}

extern "C" {

int ora_upwind_id(const char* name) {
    // CreateNavierStokesUpwind (upwind_interface.cpp:43-62), FV1 upwinds of this path
    const std::string n = lower_trim(name);
    if (n == "no") return UPW_NO;
    if (n == "full") return UPW_FULL;
    if (n == "skewed") return UPW_SKEWED;
    if (n == "linearprofileskewed" || n == "lps") return UPW_LPS;
    if (n == "positive" || n == "pos") return UPW_POS;
    return -1;
}
int ora_stab_id(const char* name) {
    // CreateNavierStokesStabilization (stabilization.cpp:46-57), plus the stabilisation-free variant
    const std::string n = lower_trim(name);
    if (n == "fields") return STAB_FIELDS;
    if (n == "flow") return STAB_FLOW;
    if (n == "without" || n == "none") return STAB_WITHOUT;
    return -1;
}
int ora_difflen_id(const char* name) {
    // set_diffusion_length (stabilization.cpp:86-100)
    const std::string n = lower_trim(name);
    if (n == "raw") return DL_RAW;
    if (n == "fivepoint") return DL_FIVEPOINT;
    if (n == "cor") return DL_COR;
    return -1;
}

void* ora_create(int dim) {
    if (dim != 2 && dim != 3) return nullptr;
    return new Problem(dim);
}
void ora_destroy(void* h) { delete static_cast<Problem*>(h); }
const char* ora_last_error(void* h) { return static_cast<Problem*>(h)->lastError.c_str(); }

int ora_set_kinematic_viscosity(void* h, double v) { auto* P = static_cast<Problem*>(h); P->disc.kinVisco = v; P->disc.viscoSet = true; return 0; }
int ora_set_density(void* h, double v) { static_cast<Problem*>(h)->disc.density = v; return 0; }
int ora_set_source(void* h, const double* f, int n) {
    auto* P = static_cast<Problem*>(h);
    if (n != P->disc.dim) return 1;
    P->disc.hasSource = true;
    for (int d = 0; d < n; ++d) P->disc.source[d] = f[d];
    return 0;
}
int ora_set_exact_jacobian(void* h, double factor) { static_cast<Problem*>(h)->disc.fullNewtonFactor = factor; return 0; }
int ora_set_stokes(void* h, int v) { static_cast<Problem*>(h)->disc.bStokes = v != 0; return 0; }
int ora_set_laplace(void* h, int v) { static_cast<Problem*>(h)->disc.bLaplace = v != 0; return 0; }
int ora_set_peclet_blend(void* h, int v) { static_cast<Problem*>(h)->disc.bPecletBlend = v != 0; return 0; }
int ora_set_upwind(void* h, const char* name) {
    const int t = ora_upwind_id(name);
    if (t < 0) return 1;
    static_cast<Problem*>(h)->disc.set_upwind(t);
    return 0;
}
int ora_set_stabilization(void* h, const char* name, const char* diffLength) {
    const int t = ora_stab_id(name);
    const int dl = diffLength ? ora_difflen_id(diffLength) : DL_RAW;
    if (t < 0 || dl < 0) return 1;
    static_cast<Problem*>(h)->disc.set_stabilization(t, dl);
    return 0;
}
int ora_set_pac_upwind(void* h, int on) {
    auto* P = static_cast<Problem*>(h);
    try { P->disc.set_pac_upwind(on != 0); } catch (std::exception& e) { P->lastError = e.what(); return 1; }
    return 0;
}
int ora_set_stabilization_upwind(void* h, const char* name) {
    const int t = ora_upwind_id(name);
    if (t < 0) return 1;
    static_cast<Problem*>(h)->disc.set_stabilization_upwind(t);
    return 0;
}

/* FV1 geometry dump of one element (for unit tests).
 * out layout per SCVF: from, to, ip[3], normal[3], shape[8], grad[8][3]  (40 doubles)
 * then per SCV: vol (1 double). */
int ora_geometry(int roid, const double* corners, double* out) {
    try {
        FV1Geometry g;
        g.update(roid, corners);
        double* o = out;
        for (int i = 0; i < g.nscvf; ++i) {
            const SCVF& f = g.scvf[i];
            *o++ = f.from; *o++ = f.to;
            for (int d = 0; d < 3; ++d) *o++ = f.globalIP[d];
            for (int d = 0; d < 3; ++d) *o++ = f.normal[d];
            for (int k = 0; k < MAXCO; ++k) *o++ = (k < g.nsh) ? f.shape[k] : 0.0;
            for (int k = 0; k < MAXCO; ++k) for (int d = 0; d < 3; ++d) *o++ = (k < g.nsh) ? f.globalGrad[k][d] : 0.0;
        }
        for (int a = 0; a < g.nscv; ++a) *o++ = g.scv[a].vol;
        return 0;
    } catch (...) { return 1; }
}

/* Reference-element tables (for the product-table consistency test). */
int ora_ref_tables(int roid, int* nco, int* nedge, int* edges, int* nside, int* side_nco, int* sides, int* edge_face) {
    try {
        const RefElem& R = ref_elem(roid);
        *nco = R.nco; *nedge = R.nedge; *nside = R.nside;
        for (int e = 0; e < R.nedge; ++e) { edges[2 * e] = R.edge[e][0]; edges[2 * e + 1] = R.edge[e][1];
            edge_face[2 * e] = R.edge_face[e][0]; edge_face[2 * e + 1] = R.edge_face[e][1]; }
        for (int s = 0; s < R.nside; ++s) { side_nco[s] = R.side_nco[s]; for (int j = 0; j < 4; ++j) sides[4 * s + j] = R.side[s][j]; }
        return 0;
    } catch (...) { return 1; }
}

/* Batched element-local callbacks: for each element the local
 * add_def_A_elem / add_jac_A_elem / add_def_M_elem / add_jac_M_elem / add_rhs_elem
 * results (each output may be NULL). u_old may be NULL (stationary); when given,
 * the stabilisation sees the old time level and dt as in the reference. */
int ora_elem_batch(void* h, int roid, int64_t nelem, const double* corners, const double* u, const double* u_old, double dt,
                   double* defA, double* jacA, double* defM, double* jacM, double* rhs) {
    auto* P = static_cast<Problem*>(h);
    try {
        P->disc.check();
        const RefElem& R = ref_elem(roid);
        if (R.dim != P->disc.dim) throw std::runtime_error("element dimension does not match the disc");
        const int nsh = R.nco, b = R.dim + 1, n = b * nsh;
        FV1Geometry geo;
        for (int64_t e = 0; e < nelem; ++e) {
            const double* c = corners + e * nsh * R.dim;
            const double* ue = u + e * n;
            const double* uo = u_old ? u_old + e * n : nullptr;
            geo.update(roid, c);
            if (defA) { double* o = defA + e * n; std::fill(o, o + n, 0.0); P->disc.add_def_A_elem(o, geo, ue, uo, dt); }
            if (jacA) { double* o = jacA + e * n * n; std::fill(o, o + n * n, 0.0); P->disc.add_jac_A_elem(o, geo, ue, uo, dt); }
            if (defM) { double* o = defM + e * n; std::fill(o, o + n, 0.0); P->disc.add_def_M_elem(o, geo, ue); }
            if (jacM) { double* o = jacM + e * n * n; std::fill(o, o + n * n, 0.0); P->disc.add_jac_M_elem(o, geo); }
            if (rhs) { double* o = rhs + e * n; std::fill(o, o + n, 0.0); P->disc.add_rhs_elem(o, geo); }
        }
        return 0;
    } catch (std::exception& ex) { P->lastError = ex.what(); return 3; }
}

/* Data exports of the disc (navier_stokes_fv1.cpp:894-1491): per element the
 * velocity, its gradient, the stabilised ip velocity, the pressure or its
 * gradient at a set of local points, and optionally the derivatives w.r.t. the
 * element's unknowns, with the reference's conventions:
 *  - ipKind 0: the SCVF integration points (the FV1 branch of each export);
 *    1: the SCV integration points (the corners: the nodal branch of the
 *    pressure export, the general branch of the others); 2: nip given points;
 *  - values[e][ip][vs], derivs[e][ip][fct][sh][vs] (vs = dim, dim*dim, dim, 1,
 *    dim for which = 0..4), both zeroed first; entries an export leaves alone
 *    stay zero. A number assigned to a vector derivative (the velocity
 *    exports) sets all of its components, as MathVector's assignment does. The
 *    general branch of the velocity gradient uses the local (reference)
 *    gradients, as the reference does (:1062-1082); the pressure gradient's
 *    general branch maps them with J^-T (:1473-1484). */
int ora_export(void* h, int which, int roid, int64_t nelem, const double* corners, const double* u, const double* u_old, double dt,
               int ipKind, int nipGiven, const double* lips, double* values, double* derivs) {
    auto* P = static_cast<Problem*>(h);
    try {
        P->disc.check();
        const RefElem& R = ref_elem(roid);
        const int dim = R.dim;
        if (dim != P->disc.dim) throw std::runtime_error("element dimension does not match the disc");
        if (which < 0 || which > 4) throw std::runtime_error("unknown export");
        const int nsh = R.nco, b = dim + 1, n = b * nsh, Pc = dim;
        const int vs = (which == 1) ? dim * dim : (which == 3) ? 1 : dim;
        FV1Geometry geo;
        for (int64_t e = 0; e < nelem; ++e) {
            const double* c = corners + e * nsh * dim;
            const double* ue = u + e * n;
            const double* uo = u_old ? u_old + e * n : nullptr;
            geo.update(roid, c);
            const int nip = ipKind == 0 ? geo.nscvf : ipKind == 1 ? nsh : nipGiven;
            double* val = values + e * (int64_t)nip * vs;
            std::fill(val, val + (int64_t)nip * vs, 0.0);
            double* der = derivs ? derivs + e * (int64_t)nip * b * nsh * vs : nullptr;
            if (der) std::fill(der, der + (int64_t)nip * b * nsh * vs, 0.0);
            auto D = [&](int ip, int f, int sh) { return der + (((int64_t)ip * b + f) * nsh + sh) * vs; };
            if (ipKind == 0 && which == 2) {
                // ex_velocity_ip, FV1 branch (:1136-1232): the stabilisation's velocity and shapes
                number StdVel[MAXSCVF][3];
                P->disc.std_vel(geo, ue, StdVel);
                P->disc.stab.update(geo, ue, StdVel, P->disc.bStokes, P->disc.kinVisco, P->disc.density,
                                    P->disc.hasSource ? P->disc.source : nullptr, uo, dt);
                const Stab& st = P->disc.stab;
                for (int ip = 0; ip < nip; ++ip) {
                    for (int d = 0; d < dim; ++d) val[ip * vs + d] = st.stabVel[ip][d];
                    if (!der) continue;
                    for (int sh = 0; sh < nsh; ++sh)
                        for (int d1 = 0; d1 < dim; ++d1) {
                            if (st.vel_comp_connected())
                                for (int d2 = 0; d2 < dim; ++d2) D(ip, d2, sh)[d1] = st.stabShapeVel[ip][d1][d2][sh];
                            else
                                D(ip, d1, sh)[d1] = st.stabShapeVel[ip][d1][d1][sh];
                            D(ip, Pc, sh)[d1] = st.stabShapeP[ip][d1][sh];
                        }
                }
                continue;
            }
            if (ipKind == 1 && which == 3) {
                // ex_nodal_pressure, SCV branch (:1336-1358): the corner's value
                for (int ip = 0; ip < nip; ++ip) {
                    const int co = geo.scv[ip].nodeId;
                    val[ip] = ue[Pc * nsh + co];
                    if (der) for (int sh = 0; sh < nsh; ++sh) D(ip, Pc, sh)[0] = (sh == co) ? 1.0 : 0.0;
                }
                continue;
            }
            for (int ip = 0; ip < nip; ++ip) {
                // shapes, gradients (global at the SCVF ips, local elsewhere) and J^-T at the point
                number N[MAXCO], G[MAXCO][3], JtInv[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
                const bool fv1 = ipKind == 0;
                if (fv1) {
                    for (int sh = 0; sh < nsh; ++sh) {
                        N[sh] = geo.scvf[ip].shape[sh];
                        for (int d = 0; d < 3; ++d) G[sh][d] = geo.scvf[ip].globalGrad[sh][d];
                    }
                } else {
                    number x[3] = {0, 0, 0};
                    for (int d = 0; d < dim; ++d) x[d] = ipKind == 1 ? R.co[ip][d] : lips[ip * dim + d];
                    p1_shapes(roid, x, N);
                    p1_grads(roid, x, G);
                    if (which == 4) {
                        number J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
                        for (int k = 0; k < nsh; ++k)
                            for (int r = 0; r < dim; ++r)
                                for (int cc = 0; cc < dim; ++cc) J[r][cc] += c[k * dim + r] * G[k][cc];
                        det_and_jtinv(dim, J, JtInv);
                    }
                }
                if (which == 0 || which == 2) {
                    // ex_nodal_velocity (:919-990), ex_velocity_ip general branch (:1238-1275)
                    for (int d = 0; d < dim; ++d)
                        for (int sh = 0; sh < nsh; ++sh) {
                            val[ip * vs + d] += ue[d * nsh + sh] * N[sh];
                            if (der) for (int q = 0; q < vs; ++q) D(ip, d, sh)[q] = N[sh];
                        }
                } else if (which == 1) {
                    // ex_velocity_grad (:1017-1098)
                    for (int d1 = 0; d1 < dim; ++d1)
                        for (int d2 = 0; d2 < dim; ++d2) {
                            number v = 0.0;
                            for (int sh = 0; sh < nsh; ++sh) {
                                v += ue[d1 * nsh + sh] * G[sh][d2];
                                if (der) D(ip, d1, sh)[d1 * dim + d2] = G[sh][d2];
                            }
                            val[ip * vs + d1 * dim + d2] = v;
                        }
                } else if (which == 3) {
                    // ex_nodal_pressure, FV1 and general branches (:1307-1333, :1360-1390)
                    number v = 0.0;
                    for (int sh = 0; sh < nsh; ++sh) v += ue[Pc * nsh + sh] * N[sh];
                    val[ip] = v;
                    if (der) for (int sh = 0; sh < nsh; ++sh) D(ip, Pc, sh)[0] = N[sh];
                } else {
                    // ex_pressure_grad (:1421-1448 FV1, :1455-1490 general)
                    if (fv1) {
                        for (int sh = 0; sh < nsh; ++sh)
                            for (int d = 0; d < dim; ++d) val[ip * vs + d] += ue[Pc * nsh + sh] * G[sh][d];
                        if (der) for (int sh = 0; sh < nsh; ++sh) for (int d = 0; d < dim; ++d) D(ip, Pc, sh)[d] = G[sh][d];
                    } else {
                        number lg[3] = {0, 0, 0};
                        for (int sh = 0; sh < nsh; ++sh)
                            for (int d = 0; d < dim; ++d) lg[d] += ue[Pc * nsh + sh] * G[sh][d];
                        for (int r = 0; r < dim; ++r) {
                            number v = 0.0;
                            for (int cc = 0; cc < dim; ++cc) v += JtInv[r][cc] * lg[cc];
                            val[ip * vs + r] = v;
                        }
                        if (der)
                            for (int sh = 0; sh < nsh; ++sh)
                                for (int r = 0; r < dim; ++r) {
                                    number v = 0.0;
                                    for (int cc = 0; cc < dim; ++cc) v += JtInv[r][cc] * G[sh][cc];
                                    D(ip, Pc, sh)[r] = v;
                                }
                    }
                }
            }
        }
        return 0;
    } catch (std::exception& ex) { P->lastError = ex.what(); return 3; }
}

/* vorticityFV1 (incompressible/navier_stokes_tools.h:387-525): per element and
 * corner, the curl (d u_y/dx - d u_x/dy) of the P1 velocity at the corner (the
 * SCV's integration point) times the SCV volume is summed at the node with the
 * SCV volume; the node value is the ratio (elements in mesh order). The formula
 * takes the first two velocity components in 3D as well (the z-component). */
int ora_vorticity(void* h, const double* U, double* vort) {
    auto* P = static_cast<Problem*>(h);
    try {
        const Mesh& m = P->mesh;
        if (m.nElems == 0) throw std::runtime_error("no mesh");
        const RefElem& R = ref_elem(m.roid);
        const int dim = m.dim, nsh = m.nsh, b = dim + 1;
        std::vector<number> vol(m.nNodes, 0.0);
        std::fill(vort, vort + m.nNodes, 0.0);
        FV1Geometry geo;
        number c[MAXCO * 3];
        for (int64_t e = 0; e < m.nElems; ++e) {
            const int32_t* nd = &m.conn[e * nsh];
            for (int k = 0; k < nsh; ++k) for (int d = 0; d < dim; ++d) c[k * dim + d] = m.coords[(int64_t)nd[k] * dim + d];
            geo.update(m.roid, c);
            for (int co = 0; co < nsh; ++co) {
                number x[3] = {0, 0, 0}, LG[MAXCO][3], J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, JtInv[3][3];
                for (int d = 0; d < dim; ++d) x[d] = R.co[co][d];
                p1_grads(m.roid, x, LG);
                for (int k = 0; k < nsh; ++k)
                    for (int r = 0; r < dim; ++r)
                        for (int cc = 0; cc < dim; ++cc) J[r][cc] += c[k * dim + r] * LG[k][cc];
                det_and_jtinv(dim, J, JtInv);
                number lv = 0.0;
                for (int sh = 0; sh < nsh; ++sh) {
                    number g[3] = {0, 0, 0};
                    for (int r = 0; r < dim; ++r) for (int cc = 0; cc < dim; ++cc) g[r] += JtInv[r][cc] * LG[sh][cc];
                    lv += U[(int64_t)nd[sh] * b + 1] * g[0] - U[(int64_t)nd[sh] * b + 0] * g[1];
                }
                const number v = geo.scv[co].vol;
                lv *= v;
                vort[nd[co]] += lv;
                vol[nd[co]] += v;
            }
        }
        for (int64_t i = 0; i < m.nNodes; ++i) vort[i] /= vol[i];
        return 0;
    } catch (std::exception& ex) { P->lastError = ex.what(); return 3; }
}

/* Local coordinates of the global point x in element corners c (the inverse of the
 * P1 / multilinear reference mapping: one solve on simplices, Newton steps from the
 * element centre on quadrilaterals and hexahedra); true if x lies in the element
 * (local coordinates within 1e-10 of the reference element). */
static bool point_in_elem(int roid, int dim, int nsh, const number* c, const number* x, number* xi) {
    const RefElem& R = ref_elem(roid);
    for (int d = 0; d < 3; ++d) xi[d] = 0.0;
    for (int d = 0; d < dim; ++d) { number s = 0; for (int k = 0; k < nsh; ++k) s += R.co[k][d]; xi[d] = s / nsh; }
    for (int it = 0; it < 30; ++it) {
        number N[MAXCO], LG[MAXCO][3], J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, JtInv[3][3], F[3] = {0, 0, 0};
        p1_shapes(roid, xi, N);
        p1_grads(roid, xi, LG);
        for (int k = 0; k < nsh; ++k)
            for (int r = 0; r < dim; ++r) {
                F[r] += N[k] * c[k * dim + r];
                for (int cc = 0; cc < dim; ++cc) J[r][cc] += c[k * dim + r] * LG[k][cc];
            }
        det_and_jtinv(dim, J, JtInv);
        // xi -= J^-1 (F - x), J^-1 = (J^-T)^T
        number dx[3] = {0, 0, 0}, step = 0.0;
        for (int cc = 0; cc < dim; ++cc) {
            number s = 0;
            for (int r = 0; r < dim; ++r) s += JtInv[r][cc] * (F[r] - x[r]);
            dx[cc] = s;
        }
        for (int cc = 0; cc < dim; ++cc) { xi[cc] -= dx[cc]; step = std::max(step, std::fabs(dx[cc])); }
        if (!(step > 1e-15)) break;
    }
    const number tol = 1e-10;
    if (roid == ROID_TRIANGLE) return xi[0] >= -tol && xi[1] >= -tol && 1.0 - xi[0] - xi[1] >= -tol;
    if (roid == ROID_TETRAHEDRON) return xi[0] >= -tol && xi[1] >= -tol && xi[2] >= -tol && 1.0 - xi[0] - xi[1] - xi[2] >= -tol;
    if (roid == ROID_PRISM) return xi[0] >= -tol && xi[1] >= -tol && 1.0 - xi[0] - xi[1] >= -tol && xi[2] >= -tol && xi[2] <= 1.0 + tol;
    for (int d = 0; d < dim; ++d) if (!(xi[d] >= -tol && xi[d] <= 1.0 + tol)) return false;
    return true;
}

/* The P1 solution's function fct at n global points (the point evaluation behind
 * DrivenCavityEvalAtPoints, navier_stokes_tools.h:540-570): the first element in
 * mesh order that contains the point, P1 shapes at its local coordinates; NaN
 * where no element contains the point. */
int ora_eval_points(void* h, const double* U, int64_t np, const double* pts, int fct, double* out) {
    auto* P = static_cast<Problem*>(h);
    try {
        const Mesh& m = P->mesh;
        if (m.nElems == 0) throw std::runtime_error("no mesh");
        const int dim = m.dim, nsh = m.nsh, b = dim + 1;
        if (fct < 0 || fct >= b) throw std::runtime_error("bad function index");
        number c[MAXCO * 3];
        for (int64_t p = 0; p < np; ++p) {
            out[p] = std::numeric_limits<number>::quiet_NaN();
            const number* x = pts + p * dim;
            for (int64_t e = 0; e < m.nElems; ++e) {
                const int32_t* nd = &m.conn[e * nsh];
                bool out_of_box = false;
                for (int d = 0; d < dim && !out_of_box; ++d) {
                    number lo = 1e300, hi = -1e300;
                    for (int k = 0; k < nsh; ++k) {
                        c[k * dim + d] = m.coords[(int64_t)nd[k] * dim + d];
                        lo = std::min(lo, c[k * dim + d]); hi = std::max(hi, c[k * dim + d]);
                    }
                    const number pad = 1e-10 * (hi - lo);
                    out_of_box = x[d] < lo - pad || x[d] > hi + pad;
                }
                if (out_of_box) continue;
                number xi[3];
                if (!point_in_elem(m.roid, dim, nsh, c, x, xi)) continue;
                number N[MAXCO];
                p1_shapes(m.roid, xi, N);
                number v = 0;
                for (int k = 0; k < nsh; ++k) v += N[k] * U[(int64_t)nd[k] * b + fct];
                out[p] = v;
                break;
            }
        }
        return 0;
    } catch (std::exception& ex) { P->lastError = ex.what(); return 3; }
}

int ora_set_mesh(void* h, int roid, int64_t nNodes, const double* coords, int64_t nElems, const int32_t* conn) {
    auto* P = static_cast<Problem*>(h);
    try {
        const RefElem& R = ref_elem(roid);
        if (R.dim != P->disc.dim) throw std::runtime_error("element dimension does not match the disc");
        Mesh& m = P->mesh;
        m = Mesh();
        m.roid = roid; m.dim = R.dim; m.nsh = R.nco; m.nNodes = nNodes; m.nElems = nElems;
        m.coords.assign(coords, coords + nNodes * R.dim);
        m.conn.assign(conn, conn + nElems * R.nco);
        for (int64_t k = 0; k < nElems * R.nco; ++k)
            if (m.conn[k] < 0 || m.conn[k] >= nNodes) throw std::runtime_error("connectivity out of range");
        build_pattern(m);
        build_coloring(m);
        P->dirRow.clear(); P->dirVal.clear();
        return 0;
    } catch (std::exception& ex) { P->lastError = ex.what(); return 1; }
}

int64_t ora_nnz_blocks(void* h) { return (int64_t)static_cast<Problem*>(h)->mesh.colIdx.size(); }
int ora_num_colors(void* h) { return static_cast<Problem*>(h)->mesh.nColors; }

int ora_pattern(void* h, int32_t* rowPtr, int32_t* colIdx) {
    const Mesh& m = static_cast<Problem*>(h)->mesh;
    std::copy(m.rowPtr.begin(), m.rowPtr.end(), rowPtr);
    std::copy(m.colIdx.begin(), m.colIdx.end(), colIdx);
    return 0;
}
int ora_coloring(void* h, int32_t* color) {
    const Mesh& m = static_cast<Problem*>(h)->mesh;
    std::copy(m.color.begin(), m.color.end(), color);
    return 0;
}

int ora_set_dirichlet(void* h, int64_t n, const int32_t* rows, const double* vals) {
    auto* P = static_cast<Problem*>(h);
    P->dirRow.assign(rows, rows + n);
    P->dirVal.assign(vals, vals + n);
    return 0;
}

/* Global defect (D) and/or block-CSR Jacobian values (JV); u_old == NULL -> stationary. */
int ora_assemble(void* h, const double* U, const double* Uold, double dt, double* D, double* JV, int nthreads) {
    auto* P = static_cast<Problem*>(h);
    try { assemble(*P, U, Uold, dt, D, JV, nthreads); return 0; }
    catch (std::exception& ex) { P->lastError = ex.what(); return 3; }
}

/* Plain Newton (ugcore's Newton, restated): u <- u - lambda * du with J du = d,
 * BiCGStab + point-block Jacobi, backtracking line search on ||d||_2.
 * stats: [newton_iters, total_linear_iters, final_rel_defect, initial_defect, status]
 * status 0 converged, 1 max iterations, 2 linear breakdown, 3 non-finite defect. */
int ora_newton(void* h, double* U, const double* Uold, double dt, double rtol, int maxit, double lin_rtol, int lin_maxit,
               int ls_steps, int nthreads, double* stats) {
    auto* P = static_cast<Problem*>(h);
    try {
        Mesh& m = P->mesh;
        const int b = m.dim + 1;
        const int64_t n = m.nNodes * b, nnzb = (int64_t)m.colIdx.size();
        // adjust the solution to the Dirichlet values
        for (size_t k = 0; k < P->dirRow.size(); ++k) U[P->dirRow[k]] = P->dirVal[k];
        std::vector<number> D(n), JV(nnzb * b * b), du(n), Ut(n), Dt(n), Dinv(m.nNodes * b * b);
        assemble(*P, U, Uold, dt, D.data(), nullptr, nthreads);
        number nd = std::sqrt(dot(n, D.data(), D.data()));
        const number nd0 = nd;
        int it = 0, linTot = 0, status = 1;
        if (!std::isfinite(nd0)) status = 3;
        else if (nd0 == 0.0) status = 0;
        while (status == 1 && it < maxit) {
            if (nd / nd0 < rtol) { status = 0; break; }
            ++it;
            assemble(*P, U, Uold, dt, nullptr, JV.data(), nthreads);
            for (int64_t r = 0; r < m.nNodes; ++r) {
                int32_t q = m.rowPtr[r];
                while (m.colIdx[q] != r) ++q;
                if (!invert_block(b, JV.data() + (int64_t)q * b * b, Dinv.data() + r * b * b)) throw std::runtime_error("singular diagonal block");
            }
            number rr = 0;
            const int li = bicgstab(m, b, JV.data(), Dinv.data(), D.data(), du.data(), lin_rtol, lin_maxit, &rr);
            if (li < 0) { status = 2; break; }
            linTot += li;
            number lambda = 1.0, ndt = 0;
            for (int k = 0; k <= ls_steps; ++k) {
                for (int64_t q = 0; q < n; ++q) Ut[q] = U[q] - lambda * du[q];
                assemble(*P, Ut.data(), Uold, dt, Dt.data(), nullptr, nthreads);
                ndt = std::sqrt(dot(n, Dt.data(), Dt.data()));
                if (ndt <= (1.0 - 1e-4 * lambda) * nd || k == ls_steps) break;
                lambda *= 0.5;
            }
            std::copy(Ut.begin(), Ut.end(), U);
            D = Dt;
            nd = ndt;
            if (!std::isfinite(nd)) { status = 3; break; }
        }
        if (status == 1 && nd / nd0 < rtol) status = 0;
        stats[0] = it; stats[1] = linTot; stats[2] = (nd0 > 0) ? nd / nd0 : 0.0; stats[3] = nd0; stats[4] = status;
        return 0;
    } catch (std::exception& ex) { P->lastError = ex.what(); return 3; }
}

/* BSR mat-vec with the oracle's own loop (for SpMV parity tests). */
int ora_add_dirichlet(void* h, int64_t n, const int32_t* rows, const double* vals) {
    auto* P = static_cast<Problem*>(h);
    merge_dirichlet(*P, std::vector<int32_t>(rows, rows + n), std::vector<number>(vals, vals + n));
    return 0;
}

int ora_add_wall(void* h, int64_t n, const int32_t* nodes) {
    auto* P = static_cast<Problem*>(h);
    const int dim = P->mesh.dim, b = dim + 1;
    std::vector<int32_t> rows;
    std::vector<number> vals;
    for (int64_t k = 0; k < n; ++k) {
        if (nodes[k] < 0 || nodes[k] >= P->mesh.nNodes) { P->lastError = "wall node out of range"; return 1; }
        for (int d = 0; d < dim; ++d) { rows.push_back(nodes[k] * b + d); vals.push_back(0.0); }
    }
    merge_dirichlet(*P, rows, vals);
    return 0;
}

int ora_add_inflow(void* h, int64_t nSides, int nco, const int32_t* sides, const double* vel) {
    auto* P = static_cast<Problem*>(h);
    Mesh& m = P->mesh;
    const int dim = m.dim, b = dim + 1, nsh = m.nsh;
    if (P->bndFlux.empty()) P->bndFlux.assign(m.nNodes, 0.0);
    std::vector<int32_t> rows;
    std::vector<number> vals;
    for (int64_t s = 0; s < nSides; ++s) {
        const int32_t* sn = sides + s * nco;
        int64_t owner = -1;
        int owners = 0;
        for (int64_t e = 0; e < m.nElems; ++e) {
            int found = 0;
            for (int j = 0; j < nco; ++j)
                for (int i = 0; i < nsh; ++i) found += (m.conn[e * nsh + i] == sn[j]);
            if (found == nco) { owner = e; ++owners; }
        }
        if (owners != 1) { P->lastError = "inflow side is not a boundary side of exactly one element"; return 1; }
        number x[4][3] = {{0}}, cen[3] = {0, 0, 0};
        for (int j = 0; j < nco; ++j) for (int d = 0; d < dim; ++d) x[j][d] = m.coords[(int64_t)sn[j] * dim + d];
        for (int i = 0; i < nsh; ++i) for (int d = 0; d < dim; ++d) cen[d] += m.coords[(int64_t)m.conn[owner * nsh + i] * dim + d] / nsh;
        for (int j = 0; j < nco; ++j) {
            number n[3];
            boundary_face_normal(dim, nco, x, j, cen, n);
            number vn = 0;
            for (int d = 0; d < dim; ++d) vn += vel[d] * n[d];
            P->bndFlux[sn[j]] += vn;
            for (int d = 0; d < dim; ++d) { rows.push_back(sn[j] * b + d); vals.push_back(vel[d]); }
        }
    }
    merge_dirichlet(*P, rows, vals);
    return 0;
}

/* NavierStokesNoNormalStressOutflowFV1::add(subsets) (no_normal_stress_outflow_fv1.cpp,
 * no_normal_stress_outflow_base): sides[nSides][nco] of the outflow boundary; each
 * corner of a side gets the boundary face {corner, side-edge midpoints, side centre}
 * (2D: {corner, side midpoint}) with its integration point at the mean of those
 * points (in local coordinates) and its outward area-weighted normal. */
int ora_add_outflow(void* h, int64_t nSides, int nco, const int32_t* sides) {
    auto* P = static_cast<Problem*>(h);
    Mesh& m = P->mesh;
    const int dim = m.dim, nsh = m.nsh;
    for (int64_t s = 0; s < nSides; ++s) {
        const int32_t* sn = sides + s * nco;
        int64_t owner = -1;
        int owners = 0;
        for (int64_t e = 0; e < m.nElems; ++e) {
            int found = 0;
            for (int j = 0; j < nco; ++j)
                for (int i = 0; i < nsh; ++i) found += (m.conn[e * nsh + i] == sn[j]);
            if (found == nco) { owner = e; ++owners; }
        }
        if (owners != 1) { P->lastError = "outflow side is not a boundary side of exactly one element"; return 1; }
        number corners[MAXCO * 3];
        int loc[4] = {0, 0, 0, 0};
        for (int i = 0; i < nsh; ++i) {
            for (int d = 0; d < dim; ++d) corners[i * dim + d] = m.coords[(int64_t)m.conn[owner * nsh + i] * dim + d];
            for (int j = 0; j < nco; ++j) if (m.conn[owner * nsh + i] == sn[j]) loc[j] = i;
        }
        side_outflow_faces(m.roid, corners, loc, nco, owner, P->outflow);
    }
    return 0;
}

/* The outflow disc on n independent elements (element-local layouts, outputs zeroed):
 * sideMask[e] bit s marks side s of the reference element as outflow boundary. */
int ora_outflow_elem(void* h, int roid, int64_t n, const double* corners, const double* u, const unsigned* sideMask, double* defA,
                     double* jacA) {
    auto* P = static_cast<Problem*>(h);
    try {
        const RefElem& R = ref_elem(roid);
        const int dim = R.dim, nsh = R.nco, nl = (dim + 1) * nsh;
        for (int64_t e = 0; e < n; ++e) {
            const double* c = corners + e * nsh * dim;
            if (defA) std::fill(defA + e * nl, defA + (e + 1) * nl, 0.0);
            if (jacA) std::fill(jacA + e * nl * nl, jacA + (e + 1) * nl * nl, 0.0);
            std::vector<OutflowBF> bfs;
            for (int s = 0; s < R.nside; ++s)
                if (sideMask[e] >> s & 1u) side_outflow_faces(roid, c, R.side[s], R.side_nco[s], e, bfs);
            for (const OutflowBF& bf : bfs)
                outflow_face_terms(P->disc, roid, c, u + e * nl, bf, 1.0, defA ? defA + e * nl : nullptr, jacA ? jacA + e * nl * nl : nullptr);
        }
        return 0;
    } catch (std::exception& ex) { P->lastError = ex.what(); return 3; }
}

int ora_bsr_mv(void* h, const double* V, const double* x, double* y) {
    auto* P = static_cast<Problem*>(h);
    bsr_mv(P->mesh, P->mesh.dim + 1, V, x, y);
    return 0;
}

}  // extern "C"
