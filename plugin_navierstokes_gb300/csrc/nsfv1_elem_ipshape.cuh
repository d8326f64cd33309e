// nsfv1_elem_ipshape.cuh -- FV1 element terms for upwinds whose shapes reach the
// other integration points of the element: the positive upwind
// (upwind.cpp:643-786, upwind.h:268 sets non_zero_shape_ip). With such an upwind
//  - the upwind velocity of an SCVF adds ip shapes times the ip velocities of
//    the other SCVFs (upwind_interface.h:333-358);
//  - the convective Jacobian interpolates those ip velocities from the corners
//    (navier_stokes_fv1.cpp:431-447);
//  - FIELDS and FLOW take their non-diagonal branch (stabilization.cpp:244-403,
//    589-771): the stabilised velocities of all SCVFs solve one ip-ip system,
//    inverted once per element and applied to the corner contributions.
// These couple all SCVFs of an element, so the path evaluates an element in
// phases (state of every SCVF, then fluxes / per-column Jacobian blocks) and
// keeps the per-SCVF state in a per-thread slice of a global workspace (entry i
// of a thread at ws[i * stride], coalesced over the threads of a launch); it is
// one thread per element with a grid-stride loop over a fixed number of
// threads. The arithmetic is FP64; FP32 Jacobians are converted at the sink.
#pragma once

#include "nsfv1_elem.cuh"

namespace nsfv1 {

// One thread's slice of the workspace.
struct IpWs {
    double* p;
    int64_t s;
    __device__ __forceinline__ double& operator[](const int i) const { return p[(int64_t)i * s]; }
};

// Offsets (in doubles) of the per-element state of one thread.
template <int ROID>
struct IpWsLayout {
    static constexpr int nip = Ref<ROID>::nip, nsh = Ref<ROID>::nsh;
    static constexpr int stdv = 0;                      // ip velocities [nip][3]
    static constexpr int nrm = stdv + 3 * nip;          // SCVF normals [nip][3]
    static constexpr int gip = nrm + 3 * nip;           // global ips [nip][3]
    static constexpr int jt = gip + 3 * nip;            // J^-T at each ip [nip][3][3]
    static constexpr int upC = jt + 9 * nip;            // convection upwind: corner shapes [nip][nsh]
    static constexpr int upCi = upC + nip * nsh;        //   ip shapes [nip][nip]
    static constexpr int upS = upCi + nip * nip;        // stabilisation upwind
    static constexpr int upSi = upS + nip * nsh;
    static constexpr int dnS = upSi + nip * nip;        // stabilisation downwind (FLOW)
    static constexpr int dnSi = dnS + nip * nsh;
    static constexpr int lup = dnSi + nip * nip;        // convection lengths of the stabilisation's up- / downwind
    static constexpr int ldn = lup + nip;
    static constexpr int lconv = ldn + nip;             // of the convection's own upwind (unused by the terms)
    static constexpr int nuL = lconv + nip;             // nu / L_diff^2
    static constexpr int ncl = nuL + nip;               // |v| / L_up
    static constexpr int ndl = ncl + nip;               // |v| / (L_down + L_up)
    static constexpr int aug = ndl + nip;               // [nip][2 nip]: the ip-ip matrix, then its inverse in the right half
    static constexpr int stab = aug + 2 * nip * nip;    // stabilised velocities [nip][3]
    static constexpr int upv = stab + 3 * nip;          // convective upwind velocity (after the Peclet blend) [nip][3]
    static constexpr int pw = upv + 3 * nip;            // Peclet blend weight [nip]
    static constexpr int cont = pw + nip;               // column-corner contributions [nip][12]: 3x3 velocity, 3 pressure
    static constexpr int flux = cont + 12 * nip;        // positive upwind: mass flux per SCVF [nip]
    static constexpr int size = flux + nip;
};

// doubles per thread of the largest element type of a dimension
constexpr int ipws_doubles(const int dim) {
    return dim == 2 ? (IpWsLayout<ROID_QUADRILATERAL>::size > IpWsLayout<ROID_TRIANGLE>::size ? IpWsLayout<ROID_QUADRILATERAL>::size
                                                                                               : IpWsLayout<ROID_TRIANGLE>::size)
                    : (IpWsLayout<ROID_HEXAHEDRON>::size > IpWsLayout<ROID_TETRAHEDRON>::size ? IpWsLayout<ROID_HEXAHEDRON>::size
                                                                                              : IpWsLayout<ROID_TETRAHEDRON>::size);
}

// Positive upwind of all SCVFs for the ip velocities sign * StdVel (sign -1: the
// downwind): for every SCV, each of its outflow faces takes the SCV's inflow
// faces as ip shapes, weighted by their flux over the larger of the SCV's total
// in- and outflow, and the SCV's corner the remainder; faces without flux take
// the mean of their two corners. The convection length is the distance of the
// ip from the point these shapes interpolate.
template <int ROID>
__device__ void positive_upwind(const Elem<ROID, double>& E, const IpWs& w, const double sign, const int oSh, const int oIp, const int oL) {
    using L = IpWsLayout<ROID>;
    using R = Ref<ROID>;
    constexpr int nip = R::nip, nsh = R::nsh, dim = R::dim;
    const auto& tb = tab<ROID, double>();
    const double eps = 2.220446049250313e-15;   // 10 x the FP64 machine epsilon
    unsigned hasFlux = 0u;
    int numNoFlux = 0;
#pragma unroll 1
    for (int ip = 0; ip < nip; ++ip) {
        const int from = tb.edge[ip][0], to = tb.edge[ip][1];
#pragma unroll 1
        for (int sh = 0; sh < nsh; ++sh) w[oSh + ip * nsh + sh] = 0.0;
#pragma unroll 1
        for (int j = 0; j < nip; ++j) w[oIp + ip * nip + j] = 0.0;
        double v[3], normSq = 0.0;
#pragma unroll
        for (int d = 0; d < dim; ++d) { v[d] = sign * w[L::stdv + 3 * ip + d]; normSq += v[d] * v[d]; }
        bool flux = fabs(normSq) > eps;
        if (flux) {
            double mf = 0.0, nn = 0.0;
#pragma unroll
            for (int d = 0; d < dim; ++d) {
                const double n = w[L::nrm + 3 * ip + d];
                mf += v[d] * n;
                nn += n * n;
            }
            w[L::flux + ip] = mf;
            flux = fabs(mf / sqrt(sqrt(normSq) * sqrt(nn))) > eps;
        }
        if (!flux) {
            w[oSh + ip * nsh + from] = 0.5;
            w[oSh + ip * nsh + to] = 0.5;
            ++numNoFlux;
        } else {
            hasFlux |= 1u << ip;
        }
    }
    if (numNoFlux != nip) {
#pragma unroll 1
        for (int sh = 0; sh < nsh; ++sh) {
            // the SCV's faces with flux, in SCVF order, with the flux leaving the SCV
            double mIn = 0.0, mOut = 0.0;
#pragma unroll 1
            for (int ip = 0; ip < nip; ++ip) {
                if (!(hasFlux >> ip & 1u)) continue;
                const double mf = w[L::flux + ip];
                double f;
                if (tb.edge[ip][0] == sh) f = mf;
                else if (tb.edge[ip][1] == sh) f = -1.0 * mf;
                else continue;
                mIn += -1.0 * fmin(f, 0.0);
                mOut += fmax(f, 0.0);
            }
            const double F = fmax(mIn, mOut);
#pragma unroll 1
            for (int i = 0; i < nip; ++i) {
                if (!(hasFlux >> i & 1u)) continue;
                double fi;
                if (tb.edge[i][0] == sh) fi = w[L::flux + i];
                else if (tb.edge[i][1] == sh) fi = -1.0 * w[L::flux + i];
                else continue;
                if (!(fi > 0.0)) continue;
                double sum = 0.0;
#pragma unroll 1
                for (int j = 0; j < nip; ++j) {
                    if (!(hasFlux >> j & 1u)) continue;
                    double fj;
                    if (tb.edge[j][0] == sh) fj = w[L::flux + j];
                    else if (tb.edge[j][1] == sh) fj = -1.0 * w[L::flux + j];
                    else continue;
                    if (fj < 0.0) {
                        const double s = -1.0 * fj / F;
                        w[oIp + i * nip + j] = s;
                        sum += s;
                    }
                }
                w[oSh + i * nsh + sh] = 1.0 - sum;
            }
        }
    }
#pragma unroll 1
    for (int ip = 0; ip < nip; ++ip) {
        double up[3] = {0.0, 0.0, 0.0};
#pragma unroll 1
        for (int sh = 0; sh < nsh; ++sh) {
            const double s = w[oSh + ip * nsh + sh];
#pragma unroll
            for (int d = 0; d < dim; ++d) up[d] += s * E.x[sh][d];
        }
#pragma unroll 1
        for (int j = 0; j < nip; ++j) {
            const double s = w[oIp + ip * nip + j];
#pragma unroll
            for (int d = 0; d < dim; ++d) up[d] += s * w[L::gip + 3 * j + d];
        }
        double dd = 0.0;
#pragma unroll
        for (int d = 0; d < dim; ++d) {
            const double x = w[L::gip + 3 * ip + d] - up[d];
            dd += x * x;
        }
        w[oL + ip] = sqrt(dd);
    }
}

// Shapes of one upwind object for all SCVFs (sign -1: the downwind). Returns
// false if a skewed / LPS ray found no side.
template <int ROID>
__device__ bool upwind_all(const int type, const Elem<ROID, double>& E, const IpWs& w, const double sign, const int oSh, const int oIp,
                           const int oL) {
    using L = IpWsLayout<ROID>;
    using R = Ref<ROID>;
    constexpr int nip = R::nip, nsh = R::nsh, dim = R::dim;
    if (type == UPW_POS) {
        positive_upwind<ROID>(E, w, sign, oSh, oIp, oL);
        return true;
    }
    bool ok = true;
#pragma unroll 1
    for (int ip = 0; ip < nip; ++ip) {
        IpGeo<double> G;
        ip_geom<ROID, double>(E, ip, G);
        double sv[3] = {0.0, 0.0, 0.0}, vel[3] = {0.0, 0.0, 0.0}, vv = 0.0;
#pragma unroll
        for (int d = 0; d < dim; ++d) {
            sv[d] = w[L::stdv + 3 * ip + d];
            vel[d] = sign < 0.0 ? sv[d] * -1.0 : sv[d];
            vv += sv[d] * sv[d];
        }
        const double norm = sqrt(vv);
        double wref[3] = {0.0, 0.0, 0.0};
        if (type == UPW_LPS && E.affine) {
#pragma unroll
            for (int a = 0; a < dim; ++a) {
                double s = 0.0;
#pragma unroll
                for (int r = 0; r < dim; ++r) s += E.JtInv[r][a] * sv[r];
                wref[a] = s;
            }
        }
        double sh[nsh], len;
        ok &= upwind_shapes<ROID, double>(type, E, G, ip, vel, norm, sign < 0.0, wref, sh, len);
#pragma unroll
        for (int k = 0; k < nsh; ++k) w[oSh + ip * nsh + k] = sh[k];
#pragma unroll 1
        for (int j = 0; j < nip; ++j) w[oIp + ip * nip + j] = 0.0;
        w[oL + ip] = len;
    }
    return ok;
}

// global gradient of shape k at SCVF ip from the stored J^-T
template <int ROID>
__device__ __forceinline__ void ws_grad(const IpWs& w, const int ip, const int k, double g[3]) {
    using L = IpWsLayout<ROID>;
    constexpr int dim = Ref<ROID>::dim;
    const auto& tb = tab<ROID, double>();
#pragma unroll
    for (int r = 0; r < dim; ++r) {
        double s = 0.0;
#pragma unroll
        for (int c = 0; c < dim; ++c) s += w[L::jt + 9 * ip + 3 * r + c] * tb.ipLGrad[ip][k][c];
        g[r] = s;
    }
}

// The stabilisation's contribution of corner k's velocity component d2 to the
// equation of component d at SCVF ip (before the division by the diagonal /
// the inverse of the ip-ip system), in the reference's order of terms.
template <int ROID>
__device__ __forceinline__ double cont_vel(const DiscParams& P, const IpWs& w, const int ip, const int k, const int d, const int d2) {
    using L = IpWsLayout<ROID>;
    constexpr int dim = Ref<ROID>::dim, nsh = Ref<ROID>::nsh;
    const bool flow = P.stab == STAB_FLOW;
    double g[3];
    ws_grad<ROID>(w, ip, k, g);
    if (d2 != d) return flow ? w[L::stdv + 3 * ip + d] * g[d2] : 0.0;
    double v = w[L::nuL + ip] * ipN<ROID, double>(ip, k);
    if (!P.stokes) {
        v += w[L::ncl + ip] * w[L::upS + ip * nsh + k];
        if (flow) v += w[L::ndl + ip] * (w[L::dnS + ip * nsh + k] - w[L::upS + ip * nsh + k]);
    }
    if (flow) {
#pragma unroll
        for (int d3 = 0; d3 < dim; ++d3)
            if (d3 != d) v -= w[L::stdv + 3 * ip + d3] * g[d3];
    }
    return v;
}

// the diagonal branch's divisor of SCVF ip
template <int ROID>
__device__ __forceinline__ double stab_diag(const DiscParams& P, const IpWs& w, const int ip) {
    using L = IpWsLayout<ROID>;
    double diag = w[L::nuL + ip];
    if (P.transient) diag += 1. / P.dt;
    if (!P.stokes) diag += w[L::ncl + ip];
    return diag;
}

// the stabilisation takes the non-diagonal branch
__device__ __forceinline__ bool stab_nondiag(const DiscParams& P) { return P.stab != STAB_WITHOUT && !P.stokes && P.stabUpwind == UPW_POS; }

// Per-element state of all SCVFs: geometry, ip velocities, upwind shapes, the
// stabilisation's coefficients, the ip-ip inverse (non-diagonal branch), the
// stabilised velocities and the convective upwind velocities. Returns false if
// an upwind ray found no side; *singular is set if the ip-ip matrix is singular.
template <int ROID>
__device__ bool ipshape_state(const DiscParams& P, const Elem<ROID, double>& E, const double (&u)[Ref<ROID>::b][Ref<ROID>::nsh],
                              const double (&uo)[Ref<ROID>::dim][Ref<ROID>::nsh], const double nu, const IpWs& w, bool& singular) {
    using L = IpWsLayout<ROID>;
    using R = Ref<ROID>;
    constexpr int nip = R::nip, nsh = R::nsh, dim = R::dim, Pc = dim;
    const bool stokes = P.stokes != 0, flow = P.stab == STAB_FLOW, without = P.stab == STAB_WITHOUT;
    const double rho = P.rho;
    singular = false;
#pragma unroll 1
    for (int ip = 0; ip < nip; ++ip) {
        IpGeo<double> G;
        ip_geom<ROID, double>(E, ip, G);
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            double s = 0.0;
#pragma unroll
            for (int sh = 0; sh < nsh; ++sh)
                if (d < dim) s += u[d][sh] * ipN<ROID, double>(ip, sh);
            w[L::stdv + 3 * ip + d] = s;
            w[L::nrm + 3 * ip + d] = G.n[d];
            w[L::gip + 3 * ip + d] = G.gip[d];
#pragma unroll
            for (int c = 0; c < 3; ++c) w[L::jt + 9 * ip + 3 * d + c] = G.JtInv[d][c];
        }
    }
    bool ok = true;
    const bool convHasOwn = !P.sameUpwind;
    if (!stokes) {
        ok &= upwind_all<ROID>(P.stabUpwind, E, w, 1.0, L::upS, L::upSi, L::lup);
        if (flow) ok &= upwind_all<ROID>(P.stabUpwind, E, w, -1.0, L::dnS, L::dnSi, L::ldn);
        if (convHasOwn) ok &= upwind_all<ROID>(P.convUpwind, E, w, 1.0, L::upC, L::upCi, L::lconv);
    }
    // diffusion lengths and convective coefficients
    double corMinN = 0.0, corMinD = 0.0, corAvgN = 1.0;
    if (!without && P.diffLen == DL_COR) cor_data<ROID, double>(E, corMinN, corMinD, corAvgN);
#pragma unroll 1
    for (int ip = 0; ip < nip; ++ip) {
        double nuL = 0.0, ncl = 0.0, ndl = 0.0;
        if (!without) {
            IpGeo<double> G;
            ip_geom<ROID, double>(E, ip, G);
            nuL = nu * diff_len_sq_inv<ROID, double>(P.diffLen, E, G, corMinN, corMinD, corAvgN);
            if (!stokes) {
                double vv = 0.0;
#pragma unroll
                for (int d = 0; d < dim; ++d) vv += w[L::stdv + 3 * ip + d] * w[L::stdv + 3 * ip + d];
                const double norm = sqrt(vv);
                ncl = norm / w[L::lup + ip];
                if (flow) ndl = norm / (w[L::ldn + ip] + w[L::lup + ip]);
            }
        }
        w[L::nuL + ip] = nuL;
        w[L::ncl + ip] = ncl;
        w[L::ndl + ip] = ndl;
    }
    // stabilised velocities
    if (without) {
#pragma unroll 1
        for (int i = 0; i < 3 * nip; ++i) w[L::stab + i] = w[L::stdv + i];
    } else if (!stab_nondiag(P)) {
        // diagonal branch
#pragma unroll 1
        for (int ip = 0; ip < nip; ++ip) {
            const double diag = stab_diag<ROID>(P, w, ip);
#pragma unroll 1
            for (int d = 0; d < dim; ++d) {
                double rhs = 0.0;
                if (P.hasSource) rhs = P.src[d];
                if (P.transient) {
                    double oldIPVel = 0.0;
#pragma unroll
                    for (int sh = 0; sh < nsh; ++sh) oldIPVel += ipN<ROID, double>(ip, sh) * uo[d][sh];
                    rhs += oldIPVel / P.dt;
                }
#pragma unroll 1
                for (int k = 0; k < nsh; ++k) {
                    rhs += cont_vel<ROID>(P, w, ip, k, d, d) * u[d][k];
                    if (flow) {
#pragma unroll
                        for (int d2 = 0; d2 < dim; ++d2)
                            if (d2 != d) rhs += cont_vel<ROID>(P, w, ip, k, d, d2) * u[d2][k];
                    }
                    double g[3];
                    ws_grad<ROID>(w, ip, k, g);
                    rhs += (-1.0 * g[d] / rho) * u[Pc][k];
                }
                w[L::stab + 3 * ip + d] = rhs / diag;
            }
#pragma unroll
            for (int d = dim; d < 3; ++d) w[L::stab + 3 * ip + d] = 0.0;
        }
    } else {
        // non-diagonal branch: the ip-ip matrix (time, diffusion, convection with the
        // upwind's ip shapes, FLOW's divergence correction), inverted by Gauss-Jordan
        // elimination with partial pivoting in place of its augmented form
        constexpr int n2 = 2 * nip;
#pragma unroll 1
        for (int ip = 0; ip < nip; ++ip) {
#pragma unroll 1
            for (int j = 0; j < n2; ++j) w[L::aug + ip * n2 + j] = (j == nip + ip) ? 1.0 : 0.0;
            double m = 0.0;
            if (P.transient) m += 1. / P.dt;
            m += w[L::nuL + ip];
            m += w[L::ncl + ip];
            w[L::aug + ip * n2 + ip] = m;
#pragma unroll 1
            for (int ip2 = 0; ip2 < nip; ++ip2) {
                double a = w[L::aug + ip * n2 + ip2];
                a -= w[L::upSi + ip * nip + ip2] * w[L::ncl + ip];
                if (flow) a += w[L::ndl + ip] * (w[L::upSi + ip * nip + ip2] - w[L::dnSi + ip * nip + ip2]);
                w[L::aug + ip * n2 + ip2] = a;
            }
        }
#pragma unroll 1
        for (int c = 0; c < nip; ++c) {
            int p = c;
#pragma unroll 1
            for (int q = c + 1; q < nip; ++q)
                if (fabs(w[L::aug + q * n2 + c]) > fabs(w[L::aug + p * n2 + c])) p = q;
            if (w[L::aug + p * n2 + c] == 0.0) { singular = true; return ok; }
            if (p != c) {
#pragma unroll 1
                for (int j = 0; j < n2; ++j) {
                    const double t = w[L::aug + p * n2 + j];
                    w[L::aug + p * n2 + j] = w[L::aug + c * n2 + j];
                    w[L::aug + c * n2 + j] = t;
                }
            }
            const double piv = 1.0 / w[L::aug + c * n2 + c];
#pragma unroll 1
            for (int j = 0; j < n2; ++j) w[L::aug + c * n2 + j] *= piv;
#pragma unroll 1
            for (int q = 0; q < nip; ++q) {
                if (q == c) continue;
                const double f = w[L::aug + q * n2 + c];
                if (f == 0.0) continue;
#pragma unroll 1
                for (int j = 0; j < n2; ++j) w[L::aug + q * n2 + j] -= f * w[L::aug + c * n2 + j];
            }
        }
        // stabilised velocity, one component at a time: x = inv f (f in the cont slots)
#pragma unroll 1
        for (int d = 0; d < dim; ++d) {
#pragma unroll 1
            for (int ip = 0; ip < nip; ++ip) {
                double oldTerm = 0.0;
                if (P.transient) {
                    double oldIPVel = 0.0;
#pragma unroll
                    for (int sh = 0; sh < nsh; ++sh) oldIPVel += ipN<ROID, double>(ip, sh) * uo[d][sh];
                    oldTerm = oldIPVel / P.dt;
                }
                double f;
                if (!flow) {
                    f = P.hasSource ? P.src[d] : 0.0;
                    if (P.transient) f += oldTerm;
                } else {
                    f = 0.0;
                }
#pragma unroll 1
                for (int k = 0; k < nsh; ++k) {
                    double g[3];
                    ws_grad<ROID>(w, ip, k, g);
                    if (flow) {
#pragma unroll
                        for (int d2 = 0; d2 < dim; ++d2) f = 1.0 * f + u[d2][k] * cont_vel<ROID>(P, w, ip, k, d, d2);
                    } else {
                        f = 1.0 * f + u[d][k] * cont_vel<ROID>(P, w, ip, k, d, d);
                    }
                    f = 1.0 * f + u[Pc][k] * (-1.0 * g[d] / rho);
                }
                if (flow) {
                    if (P.hasSource) f += P.src[d];
                    if (P.transient) f += oldTerm;
                }
                w[L::cont + 12 * ip] = f;
            }
#pragma unroll 1
            for (int ip = 0; ip < nip; ++ip) {
                double s = 0.0;
#pragma unroll 1
                for (int j = 0; j < nip; ++j) s += w[L::aug + ip * n2 + nip + j] * w[L::cont + 12 * j];
                w[L::stab + 3 * ip + d] = 1.0 * s;
            }
        }
#pragma unroll 1
        for (int ip = 0; ip < nip; ++ip)
#pragma unroll
            for (int d = dim; d < 3; ++d) w[L::stab + 3 * ip + d] = 0.0;
    }
    // convective upwind velocities (PAC: the stabilised velocity) and the Peclet blend
    if (!stokes) {
        const int oC = convHasOwn ? L::upC : L::upS, oCi = convHasOwn ? L::upCi : L::upSi;
        const int convType = convHasOwn ? P.convUpwind : P.stabUpwind;
#pragma unroll 1
        for (int ip = 0; ip < nip; ++ip) {
            double uv[3] = {0.0, 0.0, 0.0}, sv[3] = {0.0, 0.0, 0.0};
#pragma unroll
            for (int d = 0; d < dim; ++d) sv[d] = w[L::stdv + 3 * ip + d];
            if (P.pac) {
#pragma unroll
                for (int d = 0; d < dim; ++d) uv[d] = w[L::stab + 3 * ip + d];
            } else {
#pragma unroll 1
                for (int sh = 0; sh < nsh; ++sh) {
                    const double s = w[oC + ip * nsh + sh];
#pragma unroll
                    for (int d = 0; d < dim; ++d) uv[d] += s * u[d][sh];
                }
                if (convType == UPW_POS) {
#pragma unroll 1
                    for (int j = 0; j < nip; ++j) {
                        const double s = w[oCi + ip * nip + j];
#pragma unroll
                        for (int d = 0; d < dim; ++d) uv[d] += s * w[L::stdv + 3 * j + d];
                    }
                }
            }
            double wt = 1.0;
            if (P.peclet) {
                IpGeo<double> G;
                ip_geom<ROID, double>(E, ip, G);
                wt = peclet_blend<ROID, double>(G, sv, nu, uv);
            }
#pragma unroll
            for (int d = 0; d < 3; ++d) w[L::upv + 3 * ip + d] = uv[d];
            w[L::pw + ip] = wt;
        }
    }
    return ok;
}

// Stiffness defect of the element (the fluxes of every SCVF to the sink:
// + at 'from', - at 'to'), from the state ipshape_state left in w.
template <int ROID, class Sink>
__device__ void ipshape_def_A(const DiscParams& P, const Elem<ROID, double>& E, const double (&u)[Ref<ROID>::b][Ref<ROID>::nsh],
                              const IpWs& w, Sink& sink, const double nu) {
    using L = IpWsLayout<ROID>;
    using R = Ref<ROID>;
    constexpr int nip = R::nip, nsh = R::nsh, dim = R::dim, Pc = dim;
    const double rho = P.rho;
#pragma unroll 1
    for (int ip = 0; ip < nip; ++ip) {
        IpGeo<double> G;
        ip_geom<ROID, double>(E, ip, G);
        double gradVel[3][3], gradP[3];
        ip_gradients<ROID, double>(G, ip, u, gradVel, gradP);
        double flux[3];
#pragma unroll
        for (int d1 = 0; d1 < dim; ++d1) {
            double f = 0.0;
#pragma unroll
            for (int d2 = 0; d2 < dim; ++d2) f += gradVel[d1][d2] * G.n[d2];
            if (!P.laplace) {
#pragma unroll
                for (int d2 = 0; d2 < dim; ++d2) f += gradVel[d2][d1] * G.n[d2];
            }
            flux[d1] = f * ((-1.0) * nu * rho);
        }
        if (!P.stokes) {
            double prod = 0.0;
#pragma unroll
            for (int d = 0; d < dim; ++d) prod += w[L::stdv + 3 * ip + d] * G.n[d];
            prod *= rho;
#pragma unroll
            for (int d1 = 0; d1 < dim; ++d1) flux[d1] += w[L::upv + 3 * ip + d1] * prod;
        }
        double pressure = 0.0;
#pragma unroll
        for (int sh = 0; sh < nsh; ++sh) pressure += ipN<ROID, double>(ip, sh) * u[Pc][sh];
#pragma unroll
        for (int d1 = 0; d1 < dim; ++d1) flux[d1] += pressure * G.n[d1];
        double contFlux = 0.0;
#pragma unroll
        for (int d = 0; d < dim; ++d) contFlux += w[L::stab + 3 * ip + d] * G.n[d];
        contFlux *= rho;
#pragma unroll
        for (int d1 = 0; d1 < dim; ++d1) { sink.add(G.from, d1, flux[d1]); sink.add(G.to, d1, flip_sign(flux[d1])); }
        sink.add(G.from, Pc, contFlux);
        sink.add(G.to, Pc, flip_sign(contFlux));
    }
}

// The contributions of column corner k at every SCVF (the cont slots), before
// the stabilisation's division / inverse.
template <int ROID>
__device__ void ipshape_cont_k(const DiscParams& P, const IpWs& w, const int k) {
    using L = IpWsLayout<ROID>;
    constexpr int nip = Ref<ROID>::nip, dim = Ref<ROID>::dim;
    if (P.stab == STAB_WITHOUT) return;
#pragma unroll 1
    for (int ip = 0; ip < nip; ++ip) {
        double g[3];
        ws_grad<ROID>(w, ip, k, g);
#pragma unroll
        for (int a = 0; a < dim; ++a) {
#pragma unroll
            for (int c = 0; c < dim; ++c) w[L::cont + 12 * ip + 3 * a + c] = cont_vel<ROID>(P, w, ip, k, a, c);
            w[L::cont + 12 * ip + 9 + a] = -1.0 * g[a] / P.rho;
        }
    }
}

// The stabilisation's shapes of column corner k at SCVF ip (after ipshape_cont_k):
// V[a][c] = d stabVel_a / d u_c(k), Q[a] = d stabVel_a / d p(k) -- diagonal branch:
// contribution / diagonal; non-diagonal: the ip-ip inverse applied to the
// contributions of all SCVFs; without stabilisation: the interpolation shape.
template <int ROID>
__device__ __forceinline__ void ipshape_VQ(const DiscParams& P, const IpWs& w, const int ip, const int k, double (&V)[3][3], double (&Q)[3]) {
    using L = IpWsLayout<ROID>;
    constexpr int nip = Ref<ROID>::nip, dim = Ref<ROID>::dim, n2 = 2 * nip;
    if (P.stab == STAB_WITHOUT) {
        const double N = ipN<ROID, double>(ip, k);
#pragma unroll
        for (int a = 0; a < dim; ++a) {
#pragma unroll
            for (int c = 0; c < dim; ++c) V[a][c] = (a == c) ? N : 0.0;
            Q[a] = 0.0;
        }
    } else if (stab_nondiag(P)) {
#pragma unroll
        for (int a = 0; a < dim; ++a) {
#pragma unroll
            for (int c = 0; c < dim; ++c) {
                double s = 0.0;
#pragma unroll 1
                for (int j = 0; j < nip; ++j) s += w[L::aug + ip * n2 + nip + j] * w[L::cont + 12 * j + 3 * a + c];
                V[a][c] = 1.0 * s;
            }
            double s = 0.0;
#pragma unroll 1
            for (int j = 0; j < nip; ++j) s += w[L::aug + ip * n2 + nip + j] * w[L::cont + 12 * j + 9 + a];
            Q[a] = 1.0 * s;
        }
    } else {
        const double diag = stab_diag<ROID>(P, w, ip);
#pragma unroll
        for (int a = 0; a < dim; ++a) {
#pragma unroll
            for (int c = 0; c < dim; ++c) V[a][c] = w[L::cont + 12 * ip + 3 * a + c] / diag;
            Q[a] = w[L::cont + 12 * ip + 9 + a] / diag;
        }
    }
}

// Stiffness Jacobian of the element, column corner by column corner: the
// stabilisation's shapes of corner k at every SCVF, then the b x b block of each
// SCVF (scaled, + at 'from', - at 'to').
template <int ROID, class Sink>
__device__ void ipshape_jac_A(const DiscParams& P, const IpWs& w, const double scale, Sink& sink, const double nu) {
    using L = IpWsLayout<ROID>;
    using R = Ref<ROID>;
    constexpr int nip = R::nip, nsh = R::nsh, dim = R::dim, b = R::b, Pc = dim;
    const double rho = P.rho;
    const bool flow = P.stab == STAB_FLOW;
    const bool pac = P.pac && !P.stokes, fullNewton = !P.stokes && P.fullNewton != 0.0;
    const bool convHasOwn = !P.sameUpwind;
    const int oC = convHasOwn ? L::upC : L::upS, oCi = convHasOwn ? L::upCi : L::upSi;
    const bool convIp = (convHasOwn ? P.convUpwind : P.stabUpwind) == UPW_POS;
#pragma unroll 1
    for (int k = 0; k < nsh; ++k) {
        ipshape_cont_k<ROID>(P, w, k);
#pragma unroll 1
        for (int ip = 0; ip < nip; ++ip) {
            const auto& tb = tab<ROID, double>();
            const int from = tb.edge[ip][0], to = tb.edge[ip][1];
            const double N = ipN<ROID, double>(ip, k);
            double g[3], n[3];
            ws_grad<ROID>(w, ip, k, g);
#pragma unroll
            for (int d = 0; d < dim; ++d) n[d] = w[L::nrm + 3 * ip + d];
            double V[3][3], Q[3];
            ipshape_VQ<ROID>(P, w, ip, k, V, Q);
            double B[b][b];
#pragma unroll
            for (int r = 0; r < b; ++r)
#pragma unroll
                for (int c = 0; c < b; ++c) B[r][c] = 0.0;
            // diffusion
            double gn = 0.0;
#pragma unroll
            for (int d = 0; d < dim; ++d) gn += g[d] * n[d];
            const double fsh = -1.0 * nu * rho * gn;
#pragma unroll
            for (int d1 = 0; d1 < dim; ++d1) B[d1][d1] += fsh;
            if (!P.laplace) {
#pragma unroll
                for (int d1 = 0; d1 < dim; ++d1)
#pragma unroll
                    for (int d2 = 0; d2 < dim; ++d2) B[d1][d2] += -1.0 * nu * rho * g[d1] * n[d2];
            }
            // pressure
#pragma unroll
            for (int d1 = 0; d1 < dim; ++d1) B[d1][Pc] += N * n[d1];
            // convection
            if (!P.stokes) {
                double uv[3];
#pragma unroll
                for (int d = 0; d < 3; ++d) uv[d] = w[L::upv + 3 * ip + d];
                const double wt = w[L::pw + ip];
                double prod = 0.0;
#pragma unroll
                for (int d = 0; d < dim; ++d) prod += w[L::stdv + 3 * ip + d] * n[d];
                prod *= rho;
                if (pac) {
#pragma unroll
                    for (int d1 = 0; d1 < dim; ++d1) {
#pragma unroll
                        for (int d2 = 0; d2 < dim; ++d2)
                            if (flow || d1 == d2) B[d1][d2] += prod * wt * V[d1][d2];
                    }
#pragma unroll
                    for (int d1 = 0; d1 < dim; ++d1) B[d1][Pc] += prod * wt * Q[d1];
                } else {
                    double cf = w[oC + ip * nsh + k];
                    if (convIp) {
#pragma unroll 1
                        for (int j = 0; j < nip; ++j) cf += ipN<ROID, double>(j, k) * w[oCi + ip * nip + j];
                    }
                    cf *= prod * wt;
#pragma unroll
                    for (int d1 = 0; d1 < dim; ++d1) B[d1][d1] += cf;
                }
                if (P.peclet) {
                    const double cpe = prod * (1.0 - wt) * N;
#pragma unroll
                    for (int d1 = 0; d1 < dim; ++d1) B[d1][d1] += cpe;
                }
                if (fullNewton && pac) {
#pragma unroll
                    for (int d1 = 0; d1 < dim; ++d1) {
#pragma unroll
                        for (int d2 = 0; d2 < dim; ++d2) {
                            double pv = 0.0;
                            if (flow) {
#pragma unroll
                                for (int q = 0; q < dim; ++q) pv += wt * V[q][d2] * n[q];
                            } else {
                                pv = V[d1][d1] * n[d1];
                            }
                            pv *= P.fullNewton * rho;
                            B[d1][d2] += pv * uv[d1];
                        }
                        double pp = 0.0;
#pragma unroll
                        for (int q = 0; q < dim; ++q) pp += Q[q] * n[q];
                        pp *= P.fullNewton * rho;
                        B[d1][Pc] += pp * uv[d1];
                    }
                }
                if (fullNewton) {
                    if (!pac) {
#pragma unroll
                        for (int d1 = 0; d1 < dim; ++d1)
#pragma unroll
                            for (int d2 = 0; d2 < dim; ++d2) B[d1][d2] += (wt * w[oC + ip * nsh + k] * n[d2] * rho) * uv[d1];
                    }
                    if (P.peclet) {
#pragma unroll
                        for (int d1 = 0; d1 < dim; ++d1)
#pragma unroll
                            for (int d2 = 0; d2 < dim; ++d2) B[d1][d2] += uv[d1] * (1.0 - wt) * N * n[d2] * rho;
                    }
                }
            }
            // continuity
#pragma unroll
            for (int d1 = 0; d1 < dim; ++d1) {
                double cv = 0.0;
                if (flow) {
#pragma unroll
                    for (int d2 = 0; d2 < dim; ++d2) cv += V[d2][d1] * n[d2] * rho;
                } else {
                    cv = V[d1][d1] * n[d1] * rho;
                }
                B[Pc][d1] += cv;
            }
            double cp = 0.0;
#pragma unroll
            for (int d1 = 0; d1 < dim; ++d1) cp += Q[d1] * n[d1] * rho;
            B[Pc][Pc] += cp;
            if (scale != 1.0) {
#pragma unroll
                for (int r = 0; r < b; ++r)
#pragma unroll
                    for (int c = 0; c < b; ++c) B[r][c] *= scale;
            }
            sink.add(from, k, B, true);
            sink.add(to, k, B, false);
        }
    }
}

}  // namespace nsfv1
