// Post-processing of an FV1 solution on the device (incompressible/navier_stokes_tools.h):
//  - vorticityFV1 (:387-525): per element and corner, the curl d u_y/dx - d u_x/dy
//    of the P1 velocity at the corner (the SCV's integration point) times the SCV
//    volume, summed per node with the SCV volumes, then the ratio. One launch per
//    element colour with plain adds (a node belongs to one element of a colour),
//    so every node's sum keeps a fixed order: the result is reproducible.
//  - point evaluation (the GlobalGridFunctionNumberData::evaluate_global behind
//    DrivenCavityEvalAtPoints, :540-570): one thread per point, the first element
//    in mesh order whose bounding box and reference mapping contain it, the P1
//    interpolation of one function there; NaN where no element does.
#include "nsfv1_asm_common.cuh"

namespace nsfv1 {

namespace {

template <int ROID>
__global__ void __launch_bounds__(128) k_vorticity(const AsmArgs A, double* __restrict__ vort, double* __restrict__ vol) {
    using R = Ref<ROID>;
    constexpr int dim = R::dim, nsh = R::nsh, b = R::b;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= A.count) return;
    const int32_t e = __ldg(A.elems + t);
    int32_t nodes[nsh];
#pragma unroll
    for (int k = 0; k < nsh; ++k) {
        nodes[k] = __ldg(A.conn + (int64_t)e * nsh + k);
        if (!NSFV1_IN_RANGE(nodes[k], A.nNodes, A.err)) return;
    }
    Elem<ROID, double> E;
    load_corners<ROID, double>(A.coords, nodes, E);
    elem_setup<ROID, double>(E);
    double u[b][nsh];
    load_u<ROID, double>(A.U, nodes, u);
    const auto& tb = tab<ROID, double>();
#pragma unroll 1
    for (int co = 0; co < nsh; ++co) {
        double x[3] = {0.0, 0.0, 0.0}, N[nsh], LG[nsh][3];
#pragma unroll
        for (int d = 0; d < dim; ++d) x[d] = tb.refCo[co][d];
        p1_eval<ROID>(x, N, LG);
        double J[3][3] = {{0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}}, JtInv[3][3] = {{0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}};
#pragma unroll
        for (int k = 0; k < nsh; ++k)
#pragma unroll
            for (int r = 0; r < dim; ++r)
#pragma unroll
                for (int c = 0; c < dim; ++c) J[r][c] += E.x[k][r] * LG[k][c];
        jt_inverse<dim, double>(J, JtInv);
        double lv = 0.0;
#pragma unroll
        for (int sh = 0; sh < nsh; ++sh) {
            double g[3] = {0.0, 0.0, 0.0};
#pragma unroll
            for (int r = 0; r < dim; ++r)
#pragma unroll
                for (int c = 0; c < dim; ++c) g[r] += JtInv[r][c] * LG[sh][c];
            lv += u[1][sh] * g[0] - u[0][sh] * g[1];
        }
        double v = E.vol[0];
        int32_t node = nodes[0];
#pragma unroll
        for (int k = 1; k < nsh; ++k) {
            v = (k == co) ? E.vol[k] : v;
            node = (k == co) ? nodes[k] : node;
        }
        lv *= v;
        vort[node] += lv;
        vol[node] += v;
    }
}

__global__ void k_divide(int64_t n, double* __restrict__ a, const double* __restrict__ d) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) a[i] /= d[i];
}

// local coordinates of x in the element (one solve for simplices, Newton steps from the
// centre for quadrilaterals / hexahedra); true if inside within 1e-10
template <int ROID>
__device__ bool point_in_elem(const Elem<ROID, double>& E, const double* x, double (&xi)[3]) {
    using R = Ref<ROID>;
    constexpr int dim = R::dim, nsh = R::nsh;
    const auto& tb = tab<ROID, double>();
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        double s = 0.0;
#pragma unroll
        for (int k = 0; k < nsh; ++k) s += (d < dim) ? tb.refCo[k][d] : 0.0;
        xi[d] = d < dim ? s / nsh : 0.0;
    }
#pragma unroll 1
    for (int it = 0; it < 30; ++it) {
        double N[nsh], LG[nsh][3], F[3] = {0.0, 0.0, 0.0};
        double J[3][3] = {{0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}}, JtInv[3][3] = {{0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}};
        p1_eval<ROID>(xi, N, LG);
#pragma unroll
        for (int k = 0; k < nsh; ++k)
#pragma unroll
            for (int r = 0; r < dim; ++r) {
                F[r] += N[k] * E.x[k][r];
#pragma unroll
                for (int c = 0; c < dim; ++c) J[r][c] += E.x[k][r] * LG[k][c];
            }
        jt_inverse<dim, double>(J, JtInv);
        double step = 0.0;
        double dx[3] = {0.0, 0.0, 0.0};
#pragma unroll
        for (int c = 0; c < dim; ++c) {
            double s = 0.0;
#pragma unroll
            for (int r = 0; r < dim; ++r) s += JtInv[r][c] * (F[r] - x[r]);
            dx[c] = s;
        }
#pragma unroll
        for (int c = 0; c < dim; ++c) {
            xi[c] -= dx[c];
            step = fmax(step, fabs(dx[c]));
        }
        if (!(step > 1e-15)) break;
    }
    const double tol = 1e-10;
    if constexpr (ROID == ROID_TRIANGLE) return xi[0] >= -tol && xi[1] >= -tol && 1.0 - xi[0] - xi[1] >= -tol;
    if constexpr (ROID == ROID_TETRAHEDRON) return xi[0] >= -tol && xi[1] >= -tol && xi[2] >= -tol && 1.0 - xi[0] - xi[1] - xi[2] >= -tol;
    if constexpr (ROID == ROID_PRISM) return xi[0] >= -tol && xi[1] >= -tol && 1.0 - xi[0] - xi[1] >= -tol && xi[2] >= -tol && xi[2] <= 1.0 + tol;
    bool in = true;
#pragma unroll
    for (int d = 0; d < dim; ++d) in &= (xi[d] >= -tol && xi[d] <= 1.0 + tol);
    return in;
}

template <int ROID>
__global__ void __launch_bounds__(128) k_eval_points(int64_t nElems, int64_t nNodes, const double* __restrict__ coords,
                                                     const int32_t* __restrict__ conn, const double* __restrict__ U, int64_t np,
                                                     const double* __restrict__ pts, int fct, double* __restrict__ out) {
    using R = Ref<ROID>;
    constexpr int dim = R::dim, nsh = R::nsh, b = R::b;
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= np) return;
    double x[3] = {0.0, 0.0, 0.0};
#pragma unroll
    for (int d = 0; d < dim; ++d) x[d] = pts[p * dim + d];
    double res = __longlong_as_double(0x7FF8000000000000LL);   // quiet NaN: no element contains the point
    for (int64_t e = 0; e < nElems; ++e) {
        int32_t nodes[nsh];
        bool ok = true;
#pragma unroll
        for (int k = 0; k < nsh; ++k) {
            nodes[k] = __ldg(conn + e * nsh + k);
            ok &= nodes[k] >= 0 && nodes[k] < nNodes;
        }
        if (!ok) continue;
        Elem<ROID, double> E;
        bool outside = false;
#pragma unroll
        for (int d = 0; d < dim; ++d) {
            double lo = 1e300, hi = -1e300;
#pragma unroll
            for (int k = 0; k < nsh; ++k) {
                E.x[k][d] = __ldg(coords + (int64_t)nodes[k] * dim + d);
                lo = fmin(lo, E.x[k][d]);
                hi = fmax(hi, E.x[k][d]);
            }
            const double pad = 1e-10 * (hi - lo);
            outside |= x[d] < lo - pad || x[d] > hi + pad;
        }
        if (outside) continue;
        double xi[3];
        if (!point_in_elem<ROID>(E, x, xi)) continue;
        double N[nsh], LG[nsh][3];
        p1_eval<ROID>(xi, N, LG);
        double v = 0.0;
#pragma unroll
        for (int k = 0; k < nsh; ++k) v += N[k] * __ldg(U + (int64_t)nodes[k] * b + fct);
        res = v;
        break;
    }
    out[p] = res;
}

// NavierStokesNoNormalStressOutflowFV1 (no_normal_stress_outflow_fv1.cpp:343-504): per
// boundary face (corner c of an outflow side, normal n, P1 shapes N and global
// gradients G at its integration point) the momentum rows of c get the viscous
// flux -nu rho ((grad u + grad u^T) n) with its component along n removed
// (v - (v.n) n, n area-weighted as in the reference) and the outgoing convective
// flux max(rho u.n, 0) u; the continuity row gets rho u.n. The Jacobian takes the
// viscous and continuity terms exactly and the convective one with the flux frozen
// (max(rho u.n, 0) N), as the reference does. One thread per node, its faces in order.
template <int ROID, typename VT>
__global__ void __launch_bounds__(128) k_outflow(const DiscParams P, const AsmArgs A, const OutflowArgs O, const double scale) {
    using R = Ref<ROID>;
    constexpr int dim = R::dim, nsh = R::nsh, b = R::b, Pc = dim;
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= O.nSeg) return;
    const int32_t f0 = O.segPtr[s], f1 = O.segPtr[s + 1];
    const int32_t node = __ldg(A.conn + (int64_t)O.elem[f0] * nsh + O.local[f0]);
    if (!NSFV1_IN_RANGE(node, A.nNodes, A.err)) return;
    double dacc[b];
#pragma unroll
    for (int f = 0; f < b; ++f) dacc[f] = 0.0;
    for (int32_t q = f0; q < f1; ++q) {
        const int32_t e = O.elem[q], li = O.local[q];
        int32_t nodes[nsh];
        bool ok = true;
#pragma unroll
        for (int k = 0; k < nsh; ++k) {
            nodes[k] = __ldg(A.conn + (int64_t)e * nsh + k);
            ok &= NSFV1_IN_RANGE(nodes[k], A.nNodes, A.err);
        }
        if (!ok) continue;
        Elem<ROID, double> E;
        load_corners<ROID, double>(A.coords, nodes, E);
        double u[b][nsh];
        load_u<ROID, double>(A.U, nodes, u);
        double xi[3], n[3], N[nsh], LG[nsh][3], G[nsh][3];
#pragma unroll
        for (int d = 0; d < 3; ++d) { xi[d] = O.xi[3 * (int64_t)q + d]; n[d] = O.nrm[3 * (int64_t)q + d]; }
        p1_eval<ROID>(xi, N, LG);
        double J[3][3] = {{0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}}, JtInv[3][3] = {{0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}};
#pragma unroll
        for (int k = 0; k < nsh; ++k)
#pragma unroll
            for (int r = 0; r < dim; ++r)
#pragma unroll
                for (int c = 0; c < dim; ++c) J[r][c] += E.x[k][r] * LG[k][c];
        jt_inverse<dim, double>(J, JtInv);
#pragma unroll
        for (int k = 0; k < nsh; ++k)
#pragma unroll
            for (int r = 0; r < dim; ++r) {
                double g = 0.0;
#pragma unroll
                for (int c = 0; c < dim; ++c) g += JtInv[r][c] * LG[k][c];
                G[k][r] = g;
            }
        const double nu = A.nuElem ? __ldg(A.nuElem + e) : P.nu, rho = P.rho, mnr = -nu * rho;
        double sv[3] = {0.0, 0.0, 0.0}, vn = 0.0;
#pragma unroll
        for (int d = 0; d < dim; ++d) {
#pragma unroll
            for (int sh = 0; sh < nsh; ++sh) sv[d] += u[d][sh] * N[sh];
            vn += sv[d] * n[d];
        }
        if (A.D) {
            double gv[3][3], df[3] = {0.0, 0.0, 0.0};
#pragma unroll
            for (int d1 = 0; d1 < dim; ++d1)
#pragma unroll
                for (int d2 = 0; d2 < dim; ++d2) {
                    double g = 0.0;
#pragma unroll
                    for (int sh = 0; sh < nsh; ++sh) g += G[sh][d2] * u[d1][sh];
                    gv[d1][d2] = g;
                }
#pragma unroll
            for (int d1 = 0; d1 < dim; ++d1)
#pragma unroll
                for (int d2 = 0; d2 < dim; ++d2) df[d1] += gv[d1][d2] * n[d2];
            if (!P.laplace) {
#pragma unroll
                for (int d1 = 0; d1 < dim; ++d1)
#pragma unroll
                    for (int d2 = 0; d2 < dim; ++d2) df[d1] += gv[d2][d1] * n[d2];
            }
            double dot = 0.0;
#pragma unroll
            for (int d = 0; d < dim; ++d) dot += df[d] * n[d];
#pragma unroll
            for (int d = 0; d < dim; ++d) {
                df[d] += -dot * n[d];
                dacc[d] += scale * (df[d] * mnr);
            }
            if (!P.stokes) {
                const double flux = fmax(vn * rho, 0.0);
#pragma unroll
                for (int d = 0; d < dim; ++d) dacc[d] += scale * (flux * sv[d]);
            }
            dacc[Pc] += scale * (vn * rho);
        }
        if (A.vals) {
            VT* vals = reinterpret_cast<VT*>(A.vals);
            const double old = P.stokes ? 0.0 : fmax(vn * rho, 0.0);
#pragma unroll 1
            for (int sh = 0; sh < nsh; ++sh) {
                const int32_t bq = __ldg(A.elemBlk + ((int64_t)e * nsh + li) * nsh + sh);
                if (!NSFV1_IN_RANGE(bq, A.nnzb, A.err)) continue;
                VT* B = vals + (int64_t)bq * b * b;
                double M[3][3] = {{0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}}, ns[3] = {0.0, 0.0, 0.0}, gn = 0.0;
#pragma unroll
                for (int d = 0; d < dim; ++d) gn += G[sh][d] * n[d];
#pragma unroll
                for (int d = 0; d < dim; ++d) M[d][d] = gn;
                if (!P.laplace) {
#pragma unroll
                    for (int d1 = 0; d1 < dim; ++d1)
#pragma unroll
                        for (int d2 = 0; d2 < dim; ++d2) M[d1][d2] += G[sh][d1] * n[d2];
                }
#pragma unroll
                for (int d2 = 0; d2 < dim; ++d2)
#pragma unroll
                    for (int d1 = 0; d1 < dim; ++d1) ns[d2] += M[d1][d2] * n[d1];
#pragma unroll
                for (int d1 = 0; d1 < dim; ++d1)
#pragma unroll
                    for (int d2 = 0; d2 < dim; ++d2) {
                        double v = scale * ((M[d1][d2] - n[d1] * ns[d2]) * mnr);
                        if (d1 == d2 && !P.stokes) v += scale * (old * N[sh]);
                        B[d1 * b + d2] += (VT)v;
                    }
#pragma unroll
                for (int d2 = 0; d2 < dim; ++d2) B[Pc * b + d2] += (VT)(scale * (N[sh] * n[d2] * rho));
            }
        }
    }
    if (A.D) {
#pragma unroll
        for (int f = 0; f < b; ++f) A.D[(int64_t)node * b + f] += dacc[f];
    }
}

template <class F>
cudaError_t dispatch_roid_tools(int roid, F&& f) {
    switch (roid) {
        case ROID_TRIANGLE: f(std::integral_constant<int, ROID_TRIANGLE>{}); break;
        case ROID_QUADRILATERAL: f(std::integral_constant<int, ROID_QUADRILATERAL>{}); break;
        case ROID_TETRAHEDRON: f(std::integral_constant<int, ROID_TETRAHEDRON>{}); break;
        case ROID_PRISM: f(std::integral_constant<int, ROID_PRISM>{}); break;
        case ROID_HEXAHEDRON: f(std::integral_constant<int, ROID_HEXAHEDRON>{}); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_vorticity(int roid, const AsmArgs& a, double* vort, double* vol, cudaStream_t s) {
    if (a.count <= 0) return cudaSuccess;
    const int grid = (a.count + 127) / 128;
    return dispatch_roid_tools(roid, [&](auto r) { k_vorticity<decltype(r)::value><<<grid, 128, 0, s>>>(a, vort, vol); });
}

cudaError_t launch_outflow(int roid, const DiscParams& P, const AsmArgs& a, const OutflowArgs& o, int prec, cudaStream_t s) {
    if (o.nSeg <= 0) return cudaSuccess;
    const int grid = (o.nSeg + 127) / 128;
    const double scale = P.transient ? P.dt : 1.0;
    return dispatch_roid_tools(roid, [&](auto r) {
        if (prec == 0) k_outflow<decltype(r)::value, double><<<grid, 128, 0, s>>>(P, a, o, scale);
        else k_outflow<decltype(r)::value, float><<<grid, 128, 0, s>>>(P, a, o, scale);
    });
}

cudaError_t launch_divide(int64_t n, double* a, const double* d, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    k_divide<<<(int)((n + 255) / 256), 256, 0, s>>>(n, a, d);
    return cudaGetLastError();
}

cudaError_t launch_eval_points(int roid, int64_t nElems, int64_t nNodes, const double* coords, const int32_t* conn, const double* U,
                               int64_t np, const double* pts, int fct, double* out, cudaStream_t s) {
    if (np <= 0) return cudaSuccess;
    const int grid = (int)((np + 127) / 128);
    return dispatch_roid_tools(roid, [&](auto r) {
        k_eval_points<decltype(r)::value><<<grid, 128, 0, s>>>(nElems, nNodes, coords, conn, U, np, pts, fct, out);
    });
}

}  // namespace nsfv1
