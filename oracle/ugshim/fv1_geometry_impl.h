/*
 * fv1_geometry_impl.h -- the ugcore finite-volume geometries and geometric
 * helpers behind ug_shim.h (TEST INFRASTRUCTURE, see ug_shim.h).
 *
 * FV1Geometry<TElem, worldDim> restates the vertex-centred (box) dual mesh of
 * ugcore's FV1Geometry for P1 elements:
 *  - one sub-control-volume face (SCVF) per element edge, from = edge corner 0,
 *    to = edge corner 1;
 *  - 2D SCVF corners {edge midpoint, element barycentre}, normal = the segment
 *    normal rotated to point from 'from' to 'to', length = segment length;
 *  - 3D SCVF corners {edge midpoint, centre of side A, element barycentre,
 *    centre of side B} with A, B the two sides at the edge ordered so that
 *    the normal 0.5 (c2 - c0) x (c3 - c1) points from 'from' to 'to';
 *  - integration point = mean of the SCVF corners, in local and in global
 *    coordinates; shapes and local gradients at the local point, global
 *    gradients through the inverse transposed Jacobian of the element map;
 *  - one sub-control volume (SCV) per corner: 2D the quadrilateral {corner,
 *    midpoint of the outgoing edge, barycentre, midpoint of the incoming
 *    edge}; 3D the hexahedron {corner, the three edge midpoints, the three
 *    side centres, barycentre} with the volume of the six tetrahedra around
 *    the corner-barycentre diagonal.
 * Element types not run by this shim compile and throw on update().
 */
#ifndef NSFV1_UG_SHIM_FV1_GEOMETRY_IMPL_H
#define NSFV1_UG_SHIM_FV1_GEOMETRY_IMPL_H

namespace ug {

namespace shim_detail {

inline number det_jtinv(int dim, const number J[3][3], number G[3][3]) {
    // J[r][c] = d x_r / d xi_c ; G = (J^T)^-1
    for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) G[i][j] = 0.0;
    if (dim == 2) {
        const number det = J[0][0] * J[1][1] - J[0][1] * J[1][0];
        G[0][0] = J[1][1] / det; G[0][1] = -J[1][0] / det;
        G[1][0] = -J[0][1] / det; G[1][1] = J[0][0] / det;
        return det;
    }
    number C[3][3];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) {
            const int r1 = (r + 1) % 3, r2 = (r + 2) % 3, c1 = (c + 1) % 3, c2 = (c + 2) % 3;
            C[r][c] = J[r1][c1] * J[r2][c2] - J[r1][c2] * J[r2][c1];
        }
    const number det = J[0][0] * C[0][0] + J[0][1] * C[0][1] + J[0][2] * C[0][2];
    for (int r = 0; r < 3; ++r) for (int c = 0; c < 3; ++c) G[r][c] = C[r][c] / det;
    return det;
}

inline number tet_vol6(const number* a, const number* b, const number* c, const number* d) {
    const number u[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
    const number v[3] = {c[0] - a[0], c[1] - a[1], c[2] - a[2]};
    const number w[3] = {d[0] - a[0], d[1] - a[1], d[2] - a[2]};
    return u[0] * (v[1] * w[2] - v[2] * w[1]) + u[1] * (v[2] * w[0] - v[0] * w[2]) + u[2] * (v[0] * w[1] - v[1] * w[0]);
}

}  // namespace shim_detail

template <class TElem, int TWorldDim>
class FV1Geometry : public FVGeometryBase {
  public:
    typedef TElem elem_type;
    typedef typename reference_element_traits<TElem>::reference_element_type ref_elem_type;
    static const int dim = ref_elem_type::dim;
    static const int worldDim = TWorldDim;
    static const ReferenceObjectID ROID = ref_elem_type::REFERENCE_OBJECT_ID;
    static const size_t numSCVF = ref_elem_type::numEdges;
    static const size_t numSCV = ref_elem_type::numCorners;
    static const size_t nsh = ref_elem_type::numCorners;
    static const int order = 1;
    static const bool usesHangingNodes = false;

    class SCVF {
      public:
        static const size_t numCo = (dim == 3) ? 4 : (dim == 2 ? 2 : 1);
        size_t from() const { return m_from; }
        size_t to() const { return m_to; }
        const MathVector<worldDim>& normal() const { return m_normal; }
        size_t num_ip() const { return 1; }
        const MathVector<worldDim>& global_ip() const { return m_gip; }
        const MathVector<dim>& local_ip() const { return m_lip; }
        size_t num_sh() const { return nsh; }
        number shape(size_t sh) const { return m_shape[sh]; }
        const number* shape_vector() const { return m_shape; }
        const MathVector<dim>& local_grad(size_t sh) const { return m_lgrad[sh]; }
        const MathVector<worldDim>& global_grad(size_t sh) const { return m_ggrad[sh]; }
        const MathVector<worldDim>* global_grads() const { return m_ggrad; }
        size_t num_corners() const { return numCo; }
        const MathVector<worldDim>& global_corner(size_t i) const { return m_gco[i]; }
        const MathVector<dim>& local_corner(size_t i) const { return m_lco[i]; }
        number detJ() const { return m_detJ; }

      private:
        friend class FV1Geometry;
        size_t m_from = 0, m_to = 0;
        MathVector<worldDim> m_normal, m_gip;
        MathVector<dim> m_lip;
        MathVector<worldDim> m_gco[numCo];
        MathVector<dim> m_lco[numCo];
        number m_shape[nsh];
        MathVector<dim> m_lgrad[nsh];
        MathVector<worldDim> m_ggrad[nsh];
        number m_detJ = 0;
    };

    class SCV {
      public:
        static const size_t numCo = (dim == 3) ? 8 : (dim == 2 ? 4 : 2);
        number volume() const { return m_vol; }
        size_t node_id() const { return m_node; }
        size_t num_ip() const { return 1; }
        const MathVector<worldDim>& global_ip() const { return m_gco[0]; }
        const MathVector<dim>& local_ip() const { return m_lip; }
        size_t num_corners() const { return numCo; }
        const MathVector<worldDim>& global_corner(size_t i) const { return m_gco[i]; }
        const MathVector<worldDim>* global_corners() const { return m_gco; }
        size_t num_sh() const { return nsh; }

      private:
        friend class FV1Geometry;
        size_t m_node = 0;
        number m_vol = 0;
        MathVector<dim> m_lip;
        MathVector<worldDim> m_gco[numCo];
    };

    FV1Geometry() {}

    void update(GridObject* /*elem*/, const MathVector<worldDim>* vCornerCoords, const ISubsetHandler* /*ish*/ = nullptr) {
        if (!(dim == worldDim && (ROID == ROID_TRIANGLE || ROID == ROID_QUADRILATERAL || ROID == ROID_TETRAHEDRON ||
                                  ROID == ROID_PRISM || ROID == ROID_HEXAHEDRON)))
            UG_THROW("FV1Geometry: element type " << (int)ROID << " in dimension " << worldDim << " not available in this shim");
        const RefTables& R = ref_tables<ROID>();
        for (size_t c = 0; c < nsh; ++c) m_corners[c] = vCornerCoords[c];

        // barycentre, edge midpoints, side centres (global and local)
        number gC[3] = {0, 0, 0}, lC[3] = {0, 0, 0};
        for (size_t c = 0; c < nsh; ++c)
            for (int d = 0; d < worldDim; ++d) { gC[d] += m_corners[c][d]; lC[d] += R.co[c][d]; }
        for (int d = 0; d < 3; ++d) { gC[d] /= (number)nsh; lC[d] /= (number)nsh; }
        number gE[12][3], lE[12][3], gS[6][3], lS[6][3];
        for (int e = 0; e < R.numEdges; ++e)
            for (int d = 0; d < 3; ++d) {
                const int a = R.edge[e][0], b = R.edge[e][1];
                gE[e][d] = d < worldDim ? 0.5 * (m_corners[a][d] + m_corners[b][d]) : 0.0;
                lE[e][d] = 0.5 * (R.co[a][d] + R.co[b][d]);
            }
        for (int s = 0; s < R.numSides; ++s)
            for (int d = 0; d < 3; ++d) {
                number g = 0, l = 0;
                for (int j = 0; j < R.sideNco[s]; ++j) {
                    if (d < worldDim) g += m_corners[R.side[s][j]][d];
                    l += R.co[R.side[s][j]][d];
                }
                gS[s][d] = g / R.sideNco[s];
                lS[s][d] = l / R.sideNco[s];
            }

        for (size_t i = 0; i < numSCVF; ++i) {
            SCVF& f = m_scvf[i];
            f.m_from = R.edge[i][0];
            f.m_to = R.edge[i][1];
            const number* gp[4];
            const number* lp[4];
            if (dim == 2) {
                gp[0] = gE[i]; gp[1] = gC;
                lp[0] = lE[i]; lp[1] = lC;
            } else {
                int sA = -1, sB = -1;
                sides_at_edge(R, (int)i, sA, sB);
                gp[0] = gE[i]; gp[1] = gS[sA]; gp[2] = gC; gp[3] = gS[sB];
                lp[0] = lE[i]; lp[1] = lS[sA]; lp[2] = lC; lp[3] = lS[sB];
            }
            for (size_t k = 0; k < SCVF::numCo; ++k) {
                for (int d = 0; d < worldDim; ++d) f.m_gco[k][d] = gp[k][d];
                for (int d = 0; d < dim; ++d) f.m_lco[k][d] = lp[k][d];
            }
            // normal of the SCVF, oriented from 'from' to 'to'
            MathVector<worldDim> n;
            if (dim == 2) {
                n[0] = gp[1][1] - gp[0][1];
                n[1] = -(gp[1][0] - gp[0][0]);
            } else {
                const number a[3] = {gp[2][0] - gp[0][0], gp[2][1] - gp[0][1], gp[2][2] - gp[0][2]};
                const number b[3] = {gp[3][0] - gp[1][0], gp[3][1] - gp[1][1], gp[3][2] - gp[1][2]};
                n[0] = 0.5 * (a[1] * b[2] - a[2] * b[1]);
                n[1] = 0.5 * (a[2] * b[0] - a[0] * b[2]);
                n[2] = 0.5 * (a[0] * b[1] - a[1] * b[0]);
            }
            f.m_normal = n;
            // integration point: mean of the corners
            for (int d = 0; d < worldDim; ++d) {
                number s = 0;
                for (size_t k = 0; k < SCVF::numCo; ++k) s += gp[k][d];
                f.m_gip[d] = s / (number)SCVF::numCo;
            }
            number xi[3] = {0, 0, 0};
            for (int d = 0; d < dim; ++d) {
                number s = 0;
                for (size_t k = 0; k < SCVF::numCo; ++k) s += lp[k][d];
                xi[d] = s / (number)SCVF::numCo;
                f.m_lip[d] = xi[d];
            }
            number J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, G[3][3];
            for (size_t sh = 0; sh < nsh; ++sh) {
                f.m_shape[sh] = p1_shape(ROID, sh, xi);
                for (int c = 0; c < dim; ++c) {
                    f.m_lgrad[sh][c] = p1_deriv(ROID, sh, c, xi);
                    for (int r = 0; r < worldDim; ++r) J[r][c] += m_corners[sh][r] * f.m_lgrad[sh][c];
                }
            }
            f.m_detJ = shim_detail::det_jtinv(dim, J, G);
            for (size_t sh = 0; sh < nsh; ++sh)
                for (int r = 0; r < worldDim; ++r) {
                    number s = 0;
                    for (int c = 0; c < dim; ++c) s += G[r][c] * f.m_lgrad[sh][c];
                    f.m_ggrad[sh][r] = s;
                }
            m_gips[i] = f.m_gip;
            m_lips[i] = f.m_lip;
        }

        for (size_t a = 0; a < numSCV; ++a) {
            SCV& v = m_scv[a];
            v.m_node = a;
            for (int d = 0; d < dim; ++d) v.m_lip[d] = R.co[a][d];
            if (dim == 2) {
                int out = -1, in = -1;
                for (int e = 0; e < R.numEdges; ++e) {
                    if (R.edge[e][0] == (int)a) out = e;
                    if (R.edge[e][1] == (int)a) in = e;
                }
                const number* q[4] = {nullptr, gE[out], gC, gE[in]};
                number c0[3] = {0, 0, 0};
                for (int d = 0; d < worldDim; ++d) c0[d] = m_corners[a][d];
                q[0] = c0;
                for (int k = 0; k < 4; ++k) for (int d = 0; d < worldDim; ++d) v.m_gco[k][d] = q[k][d];
                // area of the quadrilateral: half the cross product of its diagonals
                const number cr = (q[2][0] - q[0][0]) * (q[3][1] - q[1][1]) - (q[2][1] - q[0][1]) * (q[3][0] - q[1][0]);
                v.m_vol = 0.5 * std::fabs(cr);
            } else {
                int nb[3], eid[3], k = 0;
                for (int e = 0; e < R.numEdges && k < 3; ++e) {
                    if (R.edge[e][0] == (int)a) { nb[k] = R.edge[e][1]; eid[k++] = e; }
                    else if (R.edge[e][1] == (int)a) { nb[k] = R.edge[e][0]; eid[k++] = e; }
                }
                number c0[3];
                for (int d = 0; d < 3; ++d) c0[d] = m_corners[a][d];
                const number* q[8] = {c0, gE[eid[0]], gS[side_with(R, (int)a, nb[0], nb[1])], gE[eid[1]],
                                      gE[eid[2]], gS[side_with(R, (int)a, nb[0], nb[2])], gC, gS[side_with(R, (int)a, nb[1], nb[2])]};
                for (int j = 0; j < 8; ++j) for (int d = 0; d < 3; ++d) v.m_gco[j][d] = q[j][d];
                const number s6 = shim_detail::tet_vol6(q[0], q[1], q[2], q[6]) + shim_detail::tet_vol6(q[0], q[2], q[3], q[6]) +
                                  shim_detail::tet_vol6(q[0], q[3], q[7], q[6]) + shim_detail::tet_vol6(q[0], q[7], q[4], q[6]) +
                                  shim_detail::tet_vol6(q[0], q[4], q[5], q[6]) + shim_detail::tet_vol6(q[0], q[5], q[1], q[6]);
                v.m_vol = std::fabs(s6) / 6.0;
            }
            m_scvGips[a] = m_corners[a];
            m_scvLips[a] = v.m_lip;
        }
        update_boundary_faces(R, lC, gC);
    }

    // Boundary faces (ugcore FV1Geometry::BF, restated): for every element side on a
    // registered boundary subset and every corner of that side, the corner's part of
    // the side -- 2D {corner, side midpoint}, 3D {corner, midpoint of the side edge to
    // the next corner, side centre, midpoint of the side edge from the previous
    // corner} -- with its integration point at the mean of those points, its normal
    // (the half side turned outward; in 3D half the cross product of the diagonals)
    // pointing out of the element, and the shapes / gradients at that point.
    class BF {
      public:
        size_t node_id() const { return m_node; }
        const MathVector<worldDim>& normal() const { return m_normal; }
        size_t num_ip() const { return 1; }
        const MathVector<dim>& local_ip() const { return m_lip; }
        const MathVector<worldDim>& global_ip() const { return m_gip; }
        size_t num_sh() const { return nsh; }
        number shape(size_t sh) const { return m_shape[sh]; }
        const MathVector<dim>& local_grad(size_t sh) const { return m_lgrad[sh]; }
        const MathVector<worldDim>& global_grad(size_t sh) const { return m_ggrad[sh]; }
        number volume() const { return m_vol; }

      private:
        friend class FV1Geometry;
        size_t m_node = 0;
        number m_vol = 0;
        MathVector<worldDim> m_normal, m_gip;
        MathVector<dim> m_lip;
        number m_shape[nsh];
        MathVector<dim> m_lgrad[nsh];
        MathVector<worldDim> m_ggrad[nsh];
    };
    void add_boundary_subset(int si) { if (si == 1) m_bnd1 = true; }
    void remove_boundary_subset(int si) { if (si == 1) m_bnd1 = false; }
    size_t num_bf(int si) const { return si == 1 ? m_bf1.size() : 0; }
    const std::vector<BF>& bf(int si) const {
        if (si != 1) UG_THROW("FV1Geometry: no boundary faces of subset " << si);
        return m_bf1;
    }

  private:
    void update_boundary_faces(const RefTables& R, const number* lC, const number* gC) {
        m_bf1.clear();
        if (!m_bnd1 || dim != worldDim) return;
        const unsigned mask = shim_boundary_sides();
        for (int s = 0; s < R.numSides; ++s) {
            if (!(mask >> s & 1u)) continue;
            const int nco = dim == 2 ? 2 : R.sideNco[s];
            const int* sc = dim == 2 ? R.edge[s] : R.side[s];
            number lS[3] = {0, 0, 0}, gS[3] = {0, 0, 0};
            for (int j = 0; j < nco; ++j)
                for (int d = 0; d < 3; ++d) {
                    lS[d] += (d < dim ? R.co[sc[j]][d] : 0.0) / nco;
                    gS[d] += (d < worldDim ? m_corners[sc[j]][d] : 0.0) / nco;
                }
            for (int j = 0; j < nco; ++j) {
                BF f;
                const int co = sc[j];
                f.m_node = co;
                number lq[4][3] = {{0}}, gq[4][3] = {{0}};
                int nq;
                for (int d = 0; d < 3; ++d) {
                    lq[0][d] = d < dim ? R.co[co][d] : 0.0;
                    gq[0][d] = d < worldDim ? m_corners[co][d] : 0.0;
                }
                if (dim == 2) {
                    nq = 2;
                    for (int d = 0; d < 3; ++d) { lq[1][d] = lS[d]; gq[1][d] = gS[d]; }
                } else {
                    nq = 4;
                    const int nx = sc[(j + 1) % nco], pv = sc[(j + nco - 1) % nco];
                    for (int d = 0; d < 3; ++d) {
                        lq[1][d] = 0.5 * (R.co[co][d] + R.co[nx][d]);
                        gq[1][d] = 0.5 * (m_corners[co][d] + m_corners[nx][d]);
                        lq[2][d] = lS[d];
                        gq[2][d] = gS[d];
                        lq[3][d] = 0.5 * (R.co[pv][d] + R.co[co][d]);
                        gq[3][d] = 0.5 * (m_corners[pv][d] + m_corners[co][d]);
                    }
                }
                for (int d = 0; d < dim; ++d) { number l = 0; for (int q = 0; q < nq; ++q) l += lq[q][d]; f.m_lip[d] = l / nq; }
                for (int d = 0; d < worldDim; ++d) { number g = 0; for (int q = 0; q < nq; ++q) g += gq[q][d]; f.m_gip[d] = g / nq; }
                number n[3] = {0, 0, 0};
                if (dim == 2) {
                    n[0] = gq[1][1] - gq[0][1];
                    n[1] = -(gq[1][0] - gq[0][0]);
                } else {
                    number d1[3], d2[3];
                    for (int d = 0; d < 3; ++d) { d1[d] = gq[2][d] - gq[0][d]; d2[d] = gq[3][d] - gq[1][d]; }
                    n[0] = 0.5 * (d1[1] * d2[2] - d1[2] * d2[1]);
                    n[1] = 0.5 * (d1[2] * d2[0] - d1[0] * d2[2]);
                    n[2] = 0.5 * (d1[0] * d2[1] - d1[1] * d2[0]);
                }
                number dot = 0, nn = 0;
                for (int d = 0; d < worldDim; ++d) { dot += n[d] * (gS[d] - gC[d]); nn += n[d] * n[d]; }
                if (dot < 0) for (int d = 0; d < 3; ++d) n[d] = -n[d];
                for (int d = 0; d < worldDim; ++d) f.m_normal[d] = n[d];
                f.m_vol = std::sqrt(nn);
                // shapes and gradients at the local integration point
                number xi[3] = {0, 0, 0};
                for (int d = 0; d < dim; ++d) xi[d] = f.m_lip[d];
                number J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, G[3][3];
                for (size_t k = 0; k < nsh; ++k) {
                    f.m_shape[k] = p1_shape(ROID, k, xi);
                    for (int c = 0; c < dim; ++c) {
                        f.m_lgrad[k][c] = p1_deriv(ROID, k, c, xi);
                        for (int r = 0; r < worldDim; ++r) J[r][c] += m_corners[k][r] * f.m_lgrad[k][c];
                    }
                }
                shim_detail::det_jtinv(dim, J, G);
                for (size_t k = 0; k < nsh; ++k)
                    for (int r = 0; r < worldDim; ++r) {
                        number v = 0;
                        for (int c = 0; c < dim; ++c) v += G[r][c] * f.m_lgrad[k][c];
                        f.m_ggrad[k][r] = v;
                    }
                m_bf1.push_back(f);
            }
        }
    }

  public:

    size_t num_scvf() const { return numSCVF; }
    const SCVF& scvf(size_t i) const { return m_scvf[i]; }
    size_t num_scv() const { return numSCV; }
    const SCV& scv(size_t i) const { return m_scv[i]; }
    size_t num_sh() const { return nsh; }
    const MathVector<worldDim>* corners() const { return m_corners; }
    size_t num_scvf_ips() const { return numSCVF; }
    const MathVector<dim>* scvf_local_ips() const { return m_lips; }
    const MathVector<worldDim>* scvf_global_ips() const { return m_gips; }
    size_t num_scv_ips() const { return numSCV; }
    const MathVector<dim>* scv_local_ips() const { return m_scvLips; }
    const MathVector<worldDim>* scv_global_ips() const { return m_scvGips; }
    ReferenceObjectID roid() const { return ROID; }

  private:
    // the two sides at edge e, ordered so that the SCVF normal points from corner 0 to 1
    static void sides_at_edge(const RefTables& R, int e, int& sA, int& sB) {
        const int a = R.edge[e][0], b = R.edge[e][1];
        int f[2], n = 0;
        for (int s = 0; s < R.numSides && n < 2; ++s) {
            bool ha = false, hb = false;
            for (int j = 0; j < R.sideNco[s]; ++j) { ha |= R.side[s][j] == a; hb |= R.side[s][j] == b; }
            if (ha && hb) f[n++] = s;
        }
        if (n != 2) UG_THROW("FV1Geometry: edge without two sides");
        // orientation test on the reference element
        number cen[3] = {0, 0, 0}, sc[2][3] = {{0, 0, 0}, {0, 0, 0}};
        for (int c = 0; c < R.numCorners; ++c) for (int d = 0; d < 3; ++d) cen[d] += R.co[c][d] / R.numCorners;
        for (int k = 0; k < 2; ++k)
            for (int j = 0; j < R.sideNco[f[k]]; ++j)
                for (int d = 0; d < 3; ++d) sc[k][d] += R.co[R.side[f[k]][j]][d] / R.sideNco[f[k]];
        number x[3], y[3];
        for (int d = 0; d < 3; ++d) { x[d] = cen[d] - 0.5 * (R.co[a][d] + R.co[b][d]); y[d] = sc[1][d] - sc[0][d]; }
        const number n0 = x[1] * y[2] - x[2] * y[1], n1 = x[2] * y[0] - x[0] * y[2], n2 = x[0] * y[1] - x[1] * y[0];
        const number dir = n0 * (R.co[b][0] - R.co[a][0]) + n1 * (R.co[b][1] - R.co[a][1]) + n2 * (R.co[b][2] - R.co[a][2]);
        if (dir > 0) { sA = f[0]; sB = f[1]; }
        else { sA = f[1]; sB = f[0]; }
    }
    static int side_with(const RefTables& R, int a, int x, int y) {
        for (int s = 0; s < R.numSides; ++s) {
            bool ha = false, hx = false, hy = false;
            for (int j = 0; j < R.sideNco[s]; ++j) { ha |= R.side[s][j] == a; hx |= R.side[s][j] == x; hy |= R.side[s][j] == y; }
            if (ha && hx && hy) return s;
        }
        UG_THROW("FV1Geometry: no side through three corners");
    }

    bool m_bnd1 = false;
    std::vector<BF> m_bf1;
    MathVector<worldDim> m_corners[nsh];
    SCVF m_scvf[numSCVF];
    SCV m_scv[numSCV];
    MathVector<dim> m_lips[numSCVF];
    MathVector<worldDim> m_gips[numSCVF];
    MathVector<dim> m_scvLips[numSCV];
    MathVector<worldDim> m_scvGips[numSCV];
};

// Crouzeix-Raviart geometries: the upwind classes register compute functions
// for them, so they must compile; they are never updated here.
template <class TElem, int TWorldDim>
class CRFVGeometry : public FVGeometryBase {
  public:
    typedef typename reference_element_traits<TElem>::reference_element_type ref_elem_type;
    static const int dim = ref_elem_type::dim;
    static const int worldDim = TWorldDim;
    static const size_t numSCVF = ref_elem_type::numEdges;
    static const size_t numSCV = ref_elem_type::numSides;
    static const int order = 1;
    static const bool usesHangingNodes = false;
    class SCVF {
      public:
        size_t from() const { return 0; }
        size_t to() const { return 0; }
        const MathVector<worldDim>& normal() const { return m_v; }
        const MathVector<worldDim>& global_ip() const { return m_v; }
        size_t num_sh() const { return 0; }
        number shape(size_t) const { return 0; }
        const MathVector<worldDim>& global_grad(size_t) const { return m_v; }

      private:
        MathVector<worldDim> m_v;
    };
    class SCV {
      public:
        number volume() const { return 0; }
        const MathVector<worldDim>& global_ip() const { return m_v; }

      private:
        MathVector<worldDim> m_v;
    };
    class CONSTRAINED_DOF {
      public:
        size_t index() const { return 0; }
        size_t num_constraining_dofs() const { return 0; }
        size_t constraining_dofs_index(size_t) const { return 0; }
        number constraining_dofs_weight(size_t) const { return 0; }
    };
    void update(GridObject*, const MathVector<worldDim>*, const ISubsetHandler* = nullptr) {
        UG_THROW("CRFVGeometry: not available in this shim");
    }
    size_t num_scvf() const { return 0; }
    const SCVF& scvf(size_t) const { return m_f; }
    size_t num_scv() const { return 0; }
    const SCV& scv(size_t) const { return m_s; }
    size_t num_sh() const { return 0; }
    const MathVector<worldDim>* corners() const { return &m_c; }
    const MathVector<worldDim>* scv_global_ips() const { return &m_c; }
    size_t num_constrained_dofs() const { return 0; }
    const CONSTRAINED_DOF& constrained_dof(size_t) const { return m_cd; }

  private:
    SCVF m_f;
    SCV m_s;
    MathVector<worldDim> m_c;
    CONSTRAINED_DOF m_cd;
};

template <class TElem, int TWorldDim>
class HCRFVGeometry : public CRFVGeometry<TElem, TWorldDim> {};

/* ---- ray intersections (ugcore: lib_disc/common/geometry_util.h) ---------- */
// ElementSideRayIntersection: the first side of the element (in reference
// order; a quadrilateral side as the triangles (0,1,2) and (0,2,3)) hit by the
// ray From + t Direction, with t >= 0 (bPositiv) or t <= 0 (the upwind search).
// The local intersection is the same barycentric combination of the side's
// reference corners. Points on a side within 1e-12 (barycentric) count as hits.
template <class TRefElem, int TWorldDim>
bool ElementSideRayIntersection(size_t& sideOut, MathVector<TWorldDim>& GlobalIntersectionPointOut,
                                MathVector<TRefElem::dim>& LocalIntersectionPoint, const MathVector<TWorldDim>& From,
                                const MathVector<TWorldDim>& Direction, bool bPositiv, const MathVector<TWorldDim>* vCornerCoords) {
    static const int dim = TRefElem::dim;
    const RefTables& R = ref_tables<TRefElem::REFERENCE_OBJECT_ID>();
    const number tol = 1e-12;
    if (dim != TWorldDim || (dim != 2 && dim != 3)) UG_THROW("ElementSideRayIntersection: not available in this shim");
    for (int s = 0; s < R.numSides; ++s) {
        const int ntri = (dim == 3 && R.sideNco[s] == 4) ? 2 : 1;
        for (int tr = 0; tr < ntri; ++tr) {
            const int i0 = R.side[s][0], i1 = R.side[s][tr == 0 ? 1 : 2], i2 = (dim == 3) ? R.side[s][tr == 0 ? 2 : 3] : -1;
            number w1 = 0, w2 = 0, t = 0;
            if (dim == 2) {
                // x0 + w1 (x1 - x0) = From + t Direction
                const number e0 = vCornerCoords[i1][0] - vCornerCoords[i0][0], e1 = vCornerCoords[i1][1] - vCornerCoords[i0][1];
                const number r0 = From[0] - vCornerCoords[i0][0], r1 = From[1] - vCornerCoords[i0][1];
                const number det = e0 * (-Direction[1]) - (-Direction[0]) * e1;
                if (det == 0.0) continue;
                w1 = (r0 * (-Direction[1]) - (-Direction[0]) * r1) / det;
                t = (e0 * r1 - r0 * e1) / det;
                if (w1 < -tol || w1 > 1.0 + tol) continue;
            } else {
                number e[3], f[3], m[3], r[3];
                for (int d = 0; d < 3; ++d) {
                    e[d] = vCornerCoords[i1][d] - vCornerCoords[i0][d];
                    f[d] = vCornerCoords[i2][d] - vCornerCoords[i0][d];
                    m[d] = -Direction[d];
                    r[d] = From[d] - vCornerCoords[i0][d];
                }
                // Cramer's rule for [e f m] (w1, w2, t)^T = r
                auto det3 = [](const number* a, const number* b, const number* c) {
                    return a[0] * (b[1] * c[2] - b[2] * c[1]) - b[0] * (a[1] * c[2] - a[2] * c[1]) + c[0] * (a[1] * b[2] - a[2] * b[1]);
                };
                const number det = det3(e, f, m);
                if (det == 0.0) continue;
                w1 = det3(r, f, m) / det;
                w2 = det3(e, r, m) / det;
                t = det3(e, f, r) / det;
                if (w1 < -tol || w2 < -tol || w1 + w2 > 1.0 + tol) continue;
            }
            if (bPositiv ? !(t >= 0.0) : !(t <= 0.0)) continue;
            sideOut = (size_t)s;
            for (int d = 0; d < TWorldDim; ++d) {
                number g = vCornerCoords[i0][d] + w1 * (vCornerCoords[i1][d] - vCornerCoords[i0][d]);
                if (dim == 3) g += w2 * (vCornerCoords[i2][d] - vCornerCoords[i0][d]);
                GlobalIntersectionPointOut[d] = g;
            }
            for (int d = 0; d < dim; ++d) {
                number l = R.co[i0][d] + w1 * (R.co[i1][d] - R.co[i0][d]);
                if (dim == 3) l += w2 * (R.co[i2][d] - R.co[i0][d]);
                LocalIntersectionPoint[d] = l;
            }
            return true;
        }
    }
    return false;
}

// SCVFofSCVRayIntersection (2D): the ray From + t Direction against the sides of
// the sub-control volume given by its four corners {corner, edge midpoint,
// barycentre, edge midpoint}; returns true if it leaves through one of the two
// SCVF sides (1: corner 1 -> 2, 2: corner 2 -> 3), false if through an element
// side (0 or 3). 'lambda' is the parameter of the hit on that side.
template <int TDim, int TWorldDim>
bool SCVFofSCVRayIntersection(size_t& sideOut, number& bc, MathVector<TWorldDim>& GlobalIntersectionPointOut,
                              MathVector<TDim>& LocalIntersectionPoint, const MathVector<TWorldDim>& From,
                              const MathVector<TWorldDim>& Direction, bool bPositiv, const MathVector<TWorldDim>* vCornerCoords) {
    if (TDim != 2 || TWorldDim != 2) UG_THROW("SCVFofSCVRayIntersection: 2D only");
    const number tol = 1e-12;
    for (int s = 0; s < 4; ++s) {
        const int i0 = s, i1 = (s + 1) % 4;
        const number e0 = vCornerCoords[i1][0] - vCornerCoords[i0][0], e1 = vCornerCoords[i1][1] - vCornerCoords[i0][1];
        const number r0 = From[0] - vCornerCoords[i0][0], r1 = From[1] - vCornerCoords[i0][1];
        const number det = e0 * (-Direction[1]) - (-Direction[0]) * e1;
        if (det == 0.0) continue;
        const number w = (r0 * (-Direction[1]) - (-Direction[0]) * r1) / det;
        const number t = (e0 * r1 - r0 * e1) / det;
        if (w < -tol || w > 1.0 + tol) continue;
        if (bPositiv ? !(t > tol) : !(t < -tol)) continue;
        sideOut = (size_t)s;
        bc = w;
        for (int d = 0; d < 2; ++d) GlobalIntersectionPointOut[d] = vCornerCoords[i0][d] + w * (vCornerCoords[i1][d] - vCornerCoords[i0][d]);
        LocalIntersectionPoint[0] = w;
        LocalIntersectionPoint[1] = 0;
        return s == 1 || s == 2;
    }
    UG_THROW("SCVFofSCVRayIntersection: no side found");
}

}  // namespace ug

#endif  // NSFV1_UG_SHIM_FV1_GEOMETRY_IMPL_H
