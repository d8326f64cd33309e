// Assembly kernels of the positive-upwind element path (nsfv1_elem_ipshape.cuh):
// one thread per element of a colour with a grid-stride loop over a fixed launch
// width (one CTA of kIpwsCtaThreads threads per SM), each thread owning one slice
// of the workspace. The scatter is the one of the other assembly kernels
// (L2 reductions, one owner per address within a colour: deterministic).
#include "nsfv1_asm_common.cuh"
#include "nsfv1_elem_ipshape.cuh"

namespace nsfv1 {

int ipws_doubles_host(const int dim) { return ipws_doubles(dim); }

namespace {

template <int ROID, bool TRANSIENT>
__global__ void __launch_bounds__(kIpwsCtaThreads) k_defect_ipshape(const DiscParams P, const AsmArgs A) {
    using R = Ref<ROID>;
    constexpr int dim = R::dim, nsh = R::nsh, b = R::b;
    const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t nth = (int64_t)gridDim.x * blockDim.x;
    const IpWs w{P.ipws + tid, (int64_t)P.ipwsStride};
    DiscParams Q = P;
    Q.transient = TRANSIENT ? 1 : 0;
    for (int64_t t = tid; t < A.count; t += nth) {
        const int32_t e = __ldg(A.elems + t);
        if (A.elemInst && !__ldg(A.instActive + __ldg(A.elemInst + e))) continue;
        const double nuEl = A.nuElem ? __ldg(A.nuElem + e) : P.nu;
        GlobalDefSink<nsh, b> sink;
        sink.D = A.D;
        bool inRange = true;
#pragma unroll
        for (int k = 0; k < nsh; ++k) {
            sink.nodes[k] = __ldg(A.conn + (int64_t)e * nsh + k);
            inRange &= NSFV1_IN_RANGE(sink.nodes[k], A.nNodes, A.err);
        }
        if (!inRange) continue;
        Elem<ROID, double> E;
        load_corners<ROID, double>(A.coords, sink.nodes, E);
        elem_setup<ROID, double>(E);
        double u[b][nsh], uo[dim][nsh];
        load_u<ROID, double>(A.U, sink.nodes, u);
        if constexpr (TRANSIENT) {
            double t4[b][nsh];
            load_u<ROID, double>(A.Uold, sink.nodes, t4);
#pragma unroll
            for (int d = 0; d < dim; ++d)
#pragma unroll
                for (int k = 0; k < nsh; ++k) uo[d][k] = t4[d][k];
        } else {
#pragma unroll
            for (int d = 0; d < dim; ++d)
#pragma unroll
                for (int k = 0; k < nsh; ++k) uo[d][k] = 0.0;
        }
        bool singular = false;
        if (!ipshape_state<ROID>(Q, E, u, uo, nuEl, w, singular)) atomicOr(A.err, 1);
        if (singular) { atomicOr(A.err, 8); continue; }
        if constexpr (TRANSIENT) {
            struct Scaled {
                GlobalDefSink<nsh, b>& s; double dt;
                __device__ __forceinline__ void add(int i, int f, double v) { s.add(i, f, v * dt); }
            } ss{sink, P.dt};
            ipshape_def_A<ROID>(Q, E, u, w, ss, nuEl);
        } else {
            ipshape_def_A<ROID>(Q, E, u, w, sink, nuEl);
        }
        // mass (implicit Euler) and source parts, per SCV (as the other defect kernels)
        const double rho = P.rho;
#pragma unroll
        for (int k = 0; k < nsh; ++k) {
#pragma unroll
            for (int f = 0; f < dim; ++f) {
                double v = 0.0;
                bool any = false;
                if (P.hasSource) { v -= P.src[f] * E.vol[k] * rho; any = true; }
                if constexpr (TRANSIENT) { v = (u[f][k] * E.vol[k] * rho - uo[f][k] * E.vol[k] * rho) + v * P.dt; any = true; }
                if (any) atomicAdd(A.D + (int64_t)sink.nodes[k] * b + f, v);
            }
        }
    }
}

template <int ROID, typename VT>
__global__ void __launch_bounds__(kIpwsCtaThreads) k_jacobian_ipshape(const DiscParams P, const AsmArgs A) {
    using R = Ref<ROID>;
    constexpr int dim = R::dim, nsh = R::nsh, b = R::b;
    const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t nth = (int64_t)gridDim.x * blockDim.x;
    const IpWs w{P.ipws + tid, (int64_t)P.ipwsStride};
    for (int64_t t = tid; t < A.count; t += nth) {
        const int32_t e = __ldg(A.elems + t);
        if (A.elemInst && !__ldg(A.instActive + __ldg(A.elemInst + e))) continue;
        const double nuEl = A.nuElem ? __ldg(A.nuElem + e) : P.nu;
        int32_t nodes[nsh];
        bool inRange = true;
#pragma unroll
        for (int k = 0; k < nsh; ++k) {
            nodes[k] = __ldg(A.conn + (int64_t)e * nsh + k);
            inRange &= NSFV1_IN_RANGE(nodes[k], A.nNodes, A.err);
        }
        if (!inRange) continue;
        Elem<ROID, double> E;
        load_corners<ROID, double>(A.coords, nodes, E);
        elem_setup<ROID, double>(E);
        double u[b][nsh], uo[dim][nsh];
        load_u<ROID, double>(A.U, nodes, u);
        // the old-time state enters through the stabilised velocity (PAC exact-Jacobian terms)
        if (P.transient) {
            double t4[b][nsh];
            load_u<ROID, double>(A.Uold, nodes, t4);
#pragma unroll
            for (int d = 0; d < dim; ++d)
#pragma unroll
                for (int k = 0; k < nsh; ++k) uo[d][k] = t4[d][k];
        } else {
#pragma unroll
            for (int d = 0; d < dim; ++d)
#pragma unroll
                for (int k = 0; k < nsh; ++k) uo[d][k] = 0.0;
        }
        bool singular = false;
        if (!ipshape_state<ROID>(P, E, u, uo, nuEl, w, singular)) atomicOr(A.err, 1);
        if (singular) { atomicOr(A.err, 8); continue; }
        GlobalJacSink<VT, nsh> sink{reinterpret_cast<VT*>(A.vals), A.elemBlk + (int64_t)e * nsh * nsh, A.nnzb, A.err};
        ipshape_jac_A<ROID>(P, w, P.transient ? P.dt : 1.0, sink, nuEl);
        if (P.transient) {
            // mass part: J(d, sh, d, sh) += |SCV| rho
#pragma unroll
            for (int k = 0; k < nsh; ++k) {
                const int32_t q = __ldg(sink.blk + k * nsh + k);
                if (!NSFV1_IN_RANGE(q, A.nnzb, A.err)) continue;
                VT* p = sink.vals + (int64_t)q * (b * b);
#pragma unroll
                for (int d = 0; d < dim; ++d) atomicAdd(p + d * b + d, (VT)(E.vol[k] * P.rho));
            }
        }
    }
}

// the stiffness parts (add_def_A_elem, add_jac_A_elem) of the batched element callbacks
template <int ROID>
__global__ void __launch_bounds__(kIpwsCtaThreads) k_elem_batch_ipshape(const DiscParams P, const ElemBatchArgs A) {
    using R = Ref<ROID>;
    constexpr int dim = R::dim, nsh = R::nsh, b = R::b, n = b * nsh;
    const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t nth = (int64_t)gridDim.x * blockDim.x;
    const IpWs w{P.ipws + tid, (int64_t)P.ipwsStride};
    DiscParams Q = P;
    Q.transient = A.uold != nullptr;
    for (int64_t e = tid; e < A.n; e += nth) {
        Elem<ROID, double> E;
#pragma unroll
        for (int k = 0; k < nsh; ++k)
#pragma unroll
            for (int d = 0; d < dim; ++d) E.x[k][d] = A.corners[(e * nsh + k) * dim + d];
        elem_setup<ROID, double>(E);
        double u[b][nsh], uo[dim][nsh];
#pragma unroll
        for (int f = 0; f < b; ++f)
#pragma unroll
            for (int k = 0; k < nsh; ++k) {
                u[f][k] = A.u[e * n + f * nsh + k];
                if (f < dim) uo[f][k] = A.uold ? A.uold[e * n + f * nsh + k] : 0.0;
            }
        bool singular = false;
        if (!ipshape_state<ROID>(Q, E, u, uo, P.nu, w, singular)) atomicOr(A.err, 1);
        if (singular) { atomicOr(A.err, 8); continue; }
        if (A.defA) {
            double dA[b][nsh];
#pragma unroll
            for (int f = 0; f < b; ++f)
#pragma unroll
                for (int k = 0; k < nsh; ++k) dA[f][k] = 0.0;
            LocalDefSink<nsh, b> ls{dA};
            ipshape_def_A<ROID>(Q, E, u, w, ls, P.nu);
#pragma unroll
            for (int f = 0; f < b; ++f)
#pragma unroll
                for (int k = 0; k < nsh; ++k) A.defA[e * n + f * nsh + k] = dA[f][k];
        }
        if (A.jacA) {
            double* J = A.jacA + e * n * n;
            for (int q = 0; q < n * n; ++q) J[q] = 0.0;
            LocalJacSink<nsh> sink{J};
            ipshape_jac_A<ROID>(Q, w, 1.0, sink, P.nu);
        }
    }
}

// The data exports of one element per thread (navier_stokes_fv1.cpp:894-1491):
//  0 ex_nodal_velocity, 1 ex_velocity_grad, 2 ex_velocity_ip, 3 ex_nodal_pressure,
//  4 ex_pressure_grad; at the SCVF ips with the global shape gradients, at the
//  SCV ips / given points with the local ones (the velocity gradient keeps them,
//  as the reference does; the pressure gradient maps them with J^-T at the point).
//  Derivative entries an export does not set stay zero; a scalar derivative of a
//  vector value is written to all of its components (the reference assigns a
//  number to a MathVector). The stabilised ip velocity uses the positive-upwind
//  element path's per-SCVF state (any upwind, either stabilisation branch).
template <int ROID>
__global__ void __launch_bounds__(kIpwsCtaThreads) k_export(const DiscParams P, const ExportArgs A) {
    using R = Ref<ROID>;
    constexpr int dim = R::dim, nsh = R::nsh, b = R::b, Pc = dim;
    const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t nth = (int64_t)gridDim.x * blockDim.x;
    const IpWs w{P.ipws + tid, (int64_t)P.ipwsStride};
    const int which = A.which;
    const int nip = A.ipKind == 0 ? R::nip : A.ipKind == 1 ? nsh : A.nip;
    const int vs = (which == 1) ? dim * dim : (which == 3) ? 1 : dim;
    DiscParams Q = P;
    Q.transient = A.uold != nullptr;
    for (int64_t e = tid; e < A.n; e += nth) {
        Elem<ROID, double> E;
#pragma unroll
        for (int k = 0; k < nsh; ++k)
#pragma unroll
            for (int d = 0; d < dim; ++d) E.x[k][d] = A.corners[(e * nsh + k) * dim + d];
        elem_setup<ROID, double>(E);
        double u[b][nsh], uo[dim][nsh];
#pragma unroll
        for (int f = 0; f < b; ++f)
#pragma unroll
            for (int k = 0; k < nsh; ++k) {
                u[f][k] = A.u[e * b * nsh + f * nsh + k];
                if (f < dim) uo[f][k] = A.uold ? A.uold[e * b * nsh + f * nsh + k] : 0.0;
            }
        double* val = A.values + e * (int64_t)nip * vs;
        double* der = A.derivs ? A.derivs + e * (int64_t)nip * b * nsh * vs : nullptr;
        for (int i = 0; i < nip * vs; ++i) val[i] = 0.0;
        if (der)
            for (int i = 0; i < nip * b * nsh * vs; ++i) der[i] = 0.0;
        auto D = [&](int ip, int f, int sh) { return der + (((int64_t)ip * b + f) * nsh + sh) * vs; };
        if (A.ipKind == 0 && which == 2) {
            // the stabilised velocity and its shapes (:1136-1232)
            bool singular = false;
            if (!ipshape_state<ROID>(Q, E, u, uo, P.nu, w, singular)) atomicOr(A.err, 1);
            if (singular) { atomicOr(A.err, 8); continue; }
            using L = IpWsLayout<ROID>;
            for (int ip = 0; ip < nip; ++ip)
#pragma unroll
                for (int d = 0; d < dim; ++d) val[ip * vs + d] = w[L::stab + 3 * ip + d];
            if (der) {
                const bool connected = P.stab == STAB_FLOW;
#pragma unroll 1
                for (int k = 0; k < nsh; ++k) {
                    ipshape_cont_k<ROID>(Q, w, k);
#pragma unroll 1
                    for (int ip = 0; ip < nip; ++ip) {
                        double V[3][3], Qs[3];
                        ipshape_VQ<ROID>(Q, w, ip, k, V, Qs);
#pragma unroll
                        for (int d1 = 0; d1 < dim; ++d1) {
                            if (connected) {
#pragma unroll
                                for (int d2 = 0; d2 < dim; ++d2) D(ip, d2, k)[d1] = V[d1][d2];
                            } else {
                                D(ip, d1, k)[d1] = V[d1][d1];
                            }
                            D(ip, Pc, k)[d1] = Qs[d1];
                        }
                    }
                }
            }
            continue;
        }
        if (A.ipKind == 1 && which == 3) {
            // the nodal pressure at the SCV ips (:1336-1358)
            for (int ip = 0; ip < nip; ++ip) {
                double p = u[Pc][0];
#pragma unroll
                for (int k = 1; k < nsh; ++k) p = (k == ip) ? u[Pc][k] : p;
                val[ip] = p;
                if (der)
                    for (int sh = 0; sh < nsh; ++sh) D(ip, Pc, sh)[0] = (sh == ip) ? 1.0 : 0.0;
            }
            continue;
        }
#pragma unroll 1
        for (int ip = 0; ip < nip; ++ip) {
            double N[nsh], G[nsh][3], JtInv[3][3] = {{0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}};
            const bool fv1 = A.ipKind == 0;
            if (fv1) {
                IpGeo<double> Gi;
                ip_geom<ROID, double>(E, ip, Gi);
#pragma unroll
                for (int sh = 0; sh < nsh; ++sh) {
                    N[sh] = ipN<ROID, double>(ip, sh);
                    double g[3];
                    ip_grad<ROID, double>(Gi, ip, sh, g);
#pragma unroll
                    for (int d = 0; d < 3; ++d) G[sh][d] = d < dim ? g[d] : 0.0;
                }
            } else {
                double x[3] = {0.0, 0.0, 0.0};
                if (A.ipKind == 1) {
                    const auto& tb = tab<ROID, double>();
#pragma unroll
                    for (int d = 0; d < dim; ++d) x[d] = tb.refCo[ip][d];
                } else {
#pragma unroll
                    for (int d = 0; d < dim; ++d) x[d] = A.lips[ip][d];
                }
                p1_eval<ROID>(x, N, G);
                if (which == 4) {
                    double J[3][3] = {{0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}};
#pragma unroll
                    for (int k = 0; k < nsh; ++k)
#pragma unroll
                        for (int r = 0; r < dim; ++r)
#pragma unroll
                            for (int c = 0; c < dim; ++c) J[r][c] += E.x[k][r] * G[k][c];
                    jt_inverse<dim, double>(J, JtInv);
                }
            }
            if (which == 0 || which == 2) {
#pragma unroll
                for (int d = 0; d < dim; ++d)
#pragma unroll
                    for (int sh = 0; sh < nsh; ++sh) {
                        val[ip * vs + d] += u[d][sh] * N[sh];
                        if (der)
                            for (int q = 0; q < vs; ++q) D(ip, d, sh)[q] = N[sh];
                    }
            } else if (which == 1) {
#pragma unroll
                for (int d1 = 0; d1 < dim; ++d1)
#pragma unroll
                    for (int d2 = 0; d2 < dim; ++d2) {
                        double v = 0.0;
#pragma unroll
                        for (int sh = 0; sh < nsh; ++sh) {
                            v += u[d1][sh] * G[sh][d2];
                            if (der) D(ip, d1, sh)[d1 * dim + d2] = G[sh][d2];
                        }
                        val[ip * vs + d1 * dim + d2] = v;
                    }
            } else if (which == 3) {
                double v = 0.0;
#pragma unroll
                for (int sh = 0; sh < nsh; ++sh) v += u[Pc][sh] * N[sh];
                val[ip] = v;
                if (der)
#pragma unroll
                    for (int sh = 0; sh < nsh; ++sh) D(ip, Pc, sh)[0] = N[sh];
            } else if (fv1) {
#pragma unroll
                for (int sh = 0; sh < nsh; ++sh)
#pragma unroll
                    for (int d = 0; d < dim; ++d) val[ip * vs + d] += u[Pc][sh] * G[sh][d];
                if (der)
#pragma unroll
                    for (int sh = 0; sh < nsh; ++sh)
#pragma unroll
                        for (int d = 0; d < dim; ++d) D(ip, Pc, sh)[d] = G[sh][d];
            } else {
                double lg[3] = {0.0, 0.0, 0.0};
#pragma unroll
                for (int sh = 0; sh < nsh; ++sh)
#pragma unroll
                    for (int d = 0; d < dim; ++d) lg[d] += u[Pc][sh] * G[sh][d];
#pragma unroll
                for (int r = 0; r < dim; ++r) {
                    double v = 0.0;
#pragma unroll
                    for (int c = 0; c < dim; ++c) v += JtInv[r][c] * lg[c];
                    val[ip * vs + r] = v;
                }
                if (der)
#pragma unroll
                    for (int sh = 0; sh < nsh; ++sh)
#pragma unroll
                        for (int r = 0; r < dim; ++r) {
                            double v = 0.0;
#pragma unroll
                            for (int c = 0; c < dim; ++c) v += JtInv[r][c] * G[sh][c];
                            D(ip, Pc, sh)[r] = v;
                        }
            }
        }
    }
}

template <class F>
cudaError_t dispatch_roid_ip(int roid, F&& f) {
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

// CTAs of one launch: enough for the work, at most the workspace's width
int ip_grid(const DiscParams& P, int64_t work) {
    const int64_t maxCta = P.ipwsStride / kIpwsCtaThreads;
    const int64_t need = (work + kIpwsCtaThreads - 1) / kIpwsCtaThreads;
    return (int)(need < maxCta ? need : maxCta);
}

}  // namespace

cudaError_t launch_export(int roid, const DiscParams& P, const ExportArgs& a, cudaStream_t s) {
    if (a.n <= 0) return cudaSuccess;
    if (!P.ipws || P.ipwsStride < kIpwsCtaThreads) return cudaErrorInvalidValue;
    const int grid = ip_grid(P, a.n);
    return dispatch_roid_ip(roid, [&](auto r) { k_export<decltype(r)::value><<<grid, kIpwsCtaThreads, 0, s>>>(P, a); });
}

cudaError_t launch_defect_ipshape(int roid, const DiscParams& P, const AsmArgs& a, cudaStream_t s) {
    if (a.count <= 0) return cudaSuccess;
    if (!P.ipws || P.ipwsStride < kIpwsCtaThreads) return cudaErrorInvalidValue;
    const int grid = ip_grid(P, a.count);
    return dispatch_roid_ip(roid, [&](auto r) {
        if (P.transient) k_defect_ipshape<decltype(r)::value, true><<<grid, kIpwsCtaThreads, 0, s>>>(P, a);
        else k_defect_ipshape<decltype(r)::value, false><<<grid, kIpwsCtaThreads, 0, s>>>(P, a);
    });
}

cudaError_t launch_jacobian_ipshape(int roid, const DiscParams& P, const AsmArgs& a, int prec, cudaStream_t s) {
    if (a.count <= 0) return cudaSuccess;
    if (!P.ipws || P.ipwsStride < kIpwsCtaThreads) return cudaErrorInvalidValue;
    const int grid = ip_grid(P, a.count);
    return dispatch_roid_ip(roid, [&](auto r) {
        if (prec == 0) k_jacobian_ipshape<decltype(r)::value, double><<<grid, kIpwsCtaThreads, 0, s>>>(P, a);
        else k_jacobian_ipshape<decltype(r)::value, float><<<grid, kIpwsCtaThreads, 0, s>>>(P, a);
    });
}

cudaError_t launch_elem_batch_ipshape(int roid, const DiscParams& P, const ElemBatchArgs& a, cudaStream_t s) {
    if (a.n <= 0 || (!a.defA && !a.jacA)) return cudaSuccess;
    if (!P.ipws || P.ipwsStride < kIpwsCtaThreads) return cudaErrorInvalidValue;
    const int grid = ip_grid(P, a.n);
    return dispatch_roid_ip(roid, [&](auto r) { k_elem_batch_ipshape<decltype(r)::value><<<grid, kIpwsCtaThreads, 0, s>>>(P, a); });
}

}  // namespace nsfv1
