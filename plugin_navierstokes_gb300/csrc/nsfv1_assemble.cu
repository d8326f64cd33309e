// FV1 assembly kernels for sm_103a: one thread per element, elements of one
// colour per launch (no two share a node). The scatter into the global defect /
// block-CSR Jacobian uses fire-and-forget L2 reductions (red.global.add); within
// a colour every address is updated by one thread only, so the summation order
// per entry is fixed (colour order, then SCVF order): runs are bitwise
// reproducible.
#include "nsfv1_asm_common.cuh"

namespace nsfv1 {

template <int ROID, bool TRANSIENT>
__global__ void __launch_bounds__(kThreads) k_defect(const DiscParams P, const AsmArgs A) {
    using R = Ref<ROID>;
    constexpr int dim = R::dim, nsh = R::nsh, b = R::b;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= A.count) return;
    const int32_t e = __ldg(A.elems + t);
    if (A.elemInst && !__ldg(A.instActive + __ldg(A.elemInst + e))) return;
    const double nuEl = A.nuElem ? __ldg(A.nuElem + e) : P.nu;
    GlobalDefSink<nsh, b> sink;
    sink.D = A.D;
#pragma unroll
    for (int k = 0; k < nsh; ++k) {
        sink.nodes[k] = __ldg(A.conn + (int64_t)e * nsh + k);
        if (!NSFV1_IN_RANGE(sink.nodes[k], A.nNodes, A.err)) return;
    }
    Elem<ROID, double> E;
    load_corners<ROID, double>(A.coords, sink.nodes, E);
    elem_setup<ROID, double>(E);
    double u[b][nsh];
    load_u<ROID, double>(A.U, sink.nodes, u);
    double uo[TRANSIENT ? dim : 1][nsh];
    if constexpr (TRANSIENT) {
        double t4[b][nsh];
        load_u<ROID, double>(A.Uold, sink.nodes, t4);
#pragma unroll
        for (int d = 0; d < dim; ++d)
#pragma unroll
            for (int k = 0; k < nsh; ++k) uo[d][k] = t4[d][k];
    }
    DiscParams Q = P;
    Q.transient = TRANSIENT ? 1 : 0;
    // the stiffness defect is scaled by dt in the implicit-Euler form: scale the
    // fluxes through a scaled sink there
    bool ok;
    if constexpr (TRANSIENT) {
        struct Scaled {
            GlobalDefSink<nsh, b>& s; double dt;
            __device__ __forceinline__ void add(int i, int f, double v) { s.add(i, f, v * dt); }
        } ss{sink, P.dt};
        ok = elem_def_A<ROID, double>(Q, E, u, reinterpret_cast<const double(&)[dim][nsh]>(uo), ss, nuEl);
    } else {
        ok = elem_def_A<ROID, double>(Q, E, u, reinterpret_cast<const double(&)[dim][nsh]>(u), sink, nuEl);
    }
    if (!ok) atomicOr(A.err, 1);
    // mass (implicit Euler) and source parts, per SCV
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

template <int ROID, typename T, typename VT, bool PAC>
__global__ void __launch_bounds__(kThreads) k_jacobian(const DiscParams P, const AsmArgs A) {
    using R = Ref<ROID>;
    constexpr int dim = R::dim, nsh = R::nsh, b = R::b;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= A.count) return;
    const int32_t e = __ldg(A.elems + t);
    if (A.elemInst && !__ldg(A.instActive + __ldg(A.elemInst + e))) return;
    const T nuEl = (T)(A.nuElem ? __ldg(A.nuElem + e) : P.nu);
    int32_t nodes[nsh];
#pragma unroll
    for (int k = 0; k < nsh; ++k) {
        nodes[k] = __ldg(A.conn + (int64_t)e * nsh + k);
        if (!NSFV1_IN_RANGE(nodes[k], A.nNodes, A.err)) return;
    }
    Elem<ROID, T> E;
    load_corners<ROID, T>(A.coords, nodes, E);
    elem_setup<ROID, T>(E);
    T u[b][nsh];
    load_u<ROID, T>(A.U, nodes, u);
    // the old-time state enters the Jacobian only through the stabilised velocity of
    // the exact-Jacobian PAC terms
    T uo[dim][nsh];
    if (PAC && P.transient && P.pac && P.fullNewton != 0.0) {
        T t4[b][nsh];
        load_u<ROID, T>(A.Uold, nodes, t4);
#pragma unroll
        for (int d = 0; d < dim; ++d)
#pragma unroll
            for (int k = 0; k < nsh; ++k) uo[d][k] = t4[d][k];
    } else {
#pragma unroll
        for (int d = 0; d < dim; ++d)
#pragma unroll
            for (int k = 0; k < nsh; ++k) uo[d][k] = T(0);
    }
    GlobalJacSink<VT, nsh> sink{reinterpret_cast<VT*>(A.vals), A.elemBlk + (int64_t)e * nsh * nsh, A.nnzb, A.err};
    const T scale = P.transient ? (T)P.dt : T(1);
    if (!elem_jac_A<ROID, T, PAC>(P, E, u, uo, scale, sink, nuEl)) atomicOr(A.err, 1);
    if (P.transient) {
        // mass part: J(d, sh, d, sh) += |SCV| rho
#pragma unroll
        for (int k = 0; k < nsh; ++k) {
            const int32_t q = __ldg(sink.blk + k * nsh + k);
            if (!NSFV1_IN_RANGE(q, A.nnzb, A.err)) continue;
            VT* p = sink.vals + (int64_t)q * (b * b);
#pragma unroll
            for (int d = 0; d < dim; ++d) atomicAdd(p + d * b + d, (VT)(E.vol[k] * T(P.rho)));
        }
    }
}

// Defect and FP64 Jacobian at the same state in one pass over the elements of a
// colour (one launch per colour instead of two): the per-SCVF geometry, upwinds
// and stabilisation are evaluated once for both outputs.
template <int ROID, bool TRANSIENT, bool PAC>
__global__ void __launch_bounds__(kThreads) k_defect_jacobian(const DiscParams P, const AsmArgs A) {
    using VT = double;
    using R = Ref<ROID>;
    constexpr int dim = R::dim, nsh = R::nsh, b = R::b;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= A.count) return;
    const int32_t e = __ldg(A.elems + t);
    if (A.elemInst && !__ldg(A.instActive + __ldg(A.elemInst + e))) return;
    const double nuEl = A.nuElem ? __ldg(A.nuElem + e) : P.nu;
    GlobalDefSink<nsh, b> sink;
    sink.D = A.D;
#pragma unroll
    for (int k = 0; k < nsh; ++k) {
        sink.nodes[k] = __ldg(A.conn + (int64_t)e * nsh + k);
        if (!NSFV1_IN_RANGE(sink.nodes[k], A.nNodes, A.err)) return;
    }
    Elem<ROID, double> E;
    load_corners<ROID, double>(A.coords, sink.nodes, E);
    elem_setup<ROID, double>(E);
    double u[b][nsh];
    load_u<ROID, double>(A.U, sink.nodes, u);
    double uo[TRANSIENT ? dim : 1][nsh];
    if constexpr (TRANSIENT) {
        double t4[b][nsh];
        load_u<ROID, double>(A.Uold, sink.nodes, t4);
#pragma unroll
        for (int d = 0; d < dim; ++d)
#pragma unroll
            for (int k = 0; k < nsh; ++k) uo[d][k] = t4[d][k];
    }
    GlobalJacSink<VT, nsh> jsink{reinterpret_cast<VT*>(A.vals), A.elemBlk + (int64_t)e * nsh * nsh, A.nnzb, A.err};
    DiscParams Q = P;
    Q.transient = TRANSIENT ? 1 : 0;
    bool ok;
    struct Scaled {
        GlobalDefSink<nsh, b>& s; double dt;
        __device__ __forceinline__ void add(int i, int f, double v) { s.add(i, f, v * dt); }
    } ss{sink, P.dt};
    const double* uoPtr = TRANSIENT ? &uo[0][0] : &u[0][0];
    const double(&uoRef)[dim][nsh] = *reinterpret_cast<const double(*)[dim][nsh]>(uoPtr);
    if constexpr (TRANSIENT) ok = elem_def_jac_A<ROID, double, PAC>(Q, E, u, uoRef, ss, P.dt, jsink, nuEl);
    else ok = elem_def_jac_A<ROID, double, PAC>(Q, E, u, uoRef, sink, 1.0, jsink, nuEl);
    if (!ok) atomicOr(A.err, 1);
    // mass (implicit Euler) and source parts, per SCV: defect as in k_defect, Jacobian as in k_jacobian
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
        if constexpr (TRANSIENT) {
            const int32_t q = __ldg(jsink.blk + k * nsh + k);
            if (!NSFV1_IN_RANGE(q, A.nnzb, A.err)) continue;
            VT* p = jsink.vals + (int64_t)q * (b * b);
#pragma unroll
            for (int d = 0; d < dim; ++d) atomicAdd(p + d * b + d, (VT)(E.vol[k] * rho));
        }
    }
}

// ---- batched element-local callbacks ----------------------------------------

template <int ROID>
__global__ void __launch_bounds__(kThreads) k_elem_batch(const DiscParams P, const ElemBatchArgs A) {
    using R = Ref<ROID>;
    constexpr int dim = R::dim, nsh = R::nsh, b = R::b, n = b * nsh;
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= A.n) return;
    Elem<ROID, double> E;
#pragma unroll
    for (int k = 0; k < nsh; ++k)
#pragma unroll
        for (int d = 0; d < dim; ++d) E.x[k][d] = A.corners[(e * nsh + k) * dim + d];
    elem_setup<ROID, double>(E);
    double u[b][nsh], uo[b][nsh];
#pragma unroll
    for (int f = 0; f < b; ++f)
#pragma unroll
        for (int k = 0; k < nsh; ++k) {
            u[f][k] = A.u[e * n + f * nsh + k];
            uo[f][k] = A.uold ? A.uold[e * n + f * nsh + k] : 0.0;
        }
    DiscParams Q = P;
    Q.transient = A.uold != nullptr;
    if (A.defA) {
        double dA[b][nsh];
#pragma unroll
        for (int f = 0; f < b; ++f)
#pragma unroll
            for (int k = 0; k < nsh; ++k) dA[f][k] = 0.0;
        LocalDefSink<nsh, b> ls{dA};
        if (!elem_def_A<ROID, double>(Q, E, u, reinterpret_cast<const double(&)[dim][nsh]>(uo), ls, P.nu)) atomicOr(A.err, 1);
#pragma unroll
        for (int f = 0; f < b; ++f)
#pragma unroll
            for (int k = 0; k < nsh; ++k) A.defA[e * n + f * nsh + k] = dA[f][k];
    }
    if (A.jacA) {
        double* J = A.jacA + e * n * n;
        for (int q = 0; q < n * n; ++q) J[q] = 0.0;
        LocalJacSink<nsh> sink{J};
        const double(&uoRef)[dim][nsh] = reinterpret_cast<const double(&)[dim][nsh]>(uo);
        const bool ok = P.pac ? elem_jac_A<ROID, double, true>(Q, E, u, uoRef, 1.0, sink, P.nu)
                              : elem_jac_A<ROID, double, false>(Q, E, u, uoRef, 1.0, sink, P.nu);
        if (!ok) atomicOr(A.err, 1);
    }
    if (A.defM) {
        for (int q = 0; q < n; ++q) A.defM[e * n + q] = 0.0;
#pragma unroll
        for (int k = 0; k < nsh; ++k)
#pragma unroll
            for (int d = 0; d < dim; ++d) A.defM[e * n + d * nsh + k] = u[d][k] * E.vol[k] * P.rho;
    }
    if (A.jacM) {
        double* J = A.jacM + e * n * n;
        for (int q = 0; q < n * n; ++q) J[q] = 0.0;
#pragma unroll
        for (int k = 0; k < nsh; ++k)
#pragma unroll
            for (int d = 0; d < dim; ++d) J[((d * nsh + k) * b + d) * nsh + k] = E.vol[k] * P.rho;
    }
    if (A.rhs) {
        for (int q = 0; q < n; ++q) A.rhs[e * n + q] = 0.0;
        if (P.hasSource) {
#pragma unroll
            for (int k = 0; k < nsh; ++k)
#pragma unroll
                for (int d = 0; d < dim; ++d) A.rhs[e * n + d * nsh + k] = P.src[d] * E.vol[k] * P.rho;
        }
    }
}

// ---- Dirichlet rows ------------------------------------------------------------
// defect = u - g ; Jacobian row = identity row (off-diagonal blocks stay in the pattern)
template <typename VT>
__global__ void k_dirichlet(int b, int64_t n, const int32_t* __restrict__ rows, const double* __restrict__ vals,
                            const int32_t* __restrict__ rowPtr, const int32_t* __restrict__ colIdx,
                            const double* __restrict__ U, double* D, VT* J) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int32_t dof = rows[i];
    const int32_t node = dof / b, f = dof % b;
    if (D) D[dof] = U[dof] - vals[i];
    if (J) {
        for (int32_t q = rowPtr[node]; q < rowPtr[node + 1]; ++q) {
            VT* blk = J + (int64_t)q * b * b;
            const bool diag = colIdx[q] == node;
            for (int c = 0; c < b; ++c) blk[f * b + c] = (diag && c == f) ? VT(1) : VT(0);
        }
    }
}

// ---- inflow boundary flux of the continuity rows ---------------------------------
__global__ void k_bnd_flux(int b, int64_t n, double scale, const double* __restrict__ flux, double* D) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double f = flux[i];
    if (f != 0.0) D[i * b + b - 1] += scale * f;
}

// ---- launchers ------------------------------------------------------------------

template <class F>
static cudaError_t dispatch_roid(int roid, F&& f) {
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

// The element kernels hold up to 255 registers per thread, so an SM runs only
// a few CTAs of a colour at once; small CTAs spread a colour evenly over the
// 152 SMs (the block size is a per-handle parameter picked by the autotuner).
static int clamp_threads(int t) { return (t >= 32 && t <= kThreads && t % 32 == 0) ? t : kThreads; }

cudaError_t launch_defect(int roid, const DiscParams& P, const AsmArgs& a, cudaStream_t s, int threads) {
    if (a.count <= 0) return cudaSuccess;
    if (uses_ipshape(P)) return launch_defect_ipshape(roid, P, a, s);
    const int t = clamp_threads(threads);
    const int grid = (a.count + t - 1) / t;
    return dispatch_roid(roid, [&](auto r) {
        if (P.transient) k_defect<decltype(r)::value, true><<<grid, t, 0, s>>>(P, a);
        else k_defect<decltype(r)::value, false><<<grid, t, 0, s>>>(P, a);
    });
}

cudaError_t launch_jacobian(int roid, const DiscParams& P, const AsmArgs& a, int prec, cudaStream_t s, int threads) {
    if (a.count <= 0) return cudaSuccess;
    if (uses_ipshape(P)) return launch_jacobian_ipshape(roid, P, a, prec, s);
    if (prec != 0) return launch_jacobian_lanes(roid, P, a, s);
    const int t = clamp_threads(threads);
    const int grid = (a.count + t - 1) / t;
    return dispatch_roid(roid, [&](auto r) {
        constexpr int RO = decltype(r)::value;
        if (P.pac && !P.stokes) k_jacobian<RO, double, double, true><<<grid, t, 0, s>>>(P, a);
        else k_jacobian<RO, double, double, false><<<grid, t, 0, s>>>(P, a);
    });
}

cudaError_t launch_defect_jacobian(int roid, const DiscParams& P, const AsmArgs& a, int prec, cudaStream_t s, int threads) {
    if (a.count <= 0) return cudaSuccess;
    if (uses_ipshape(P)) {
        // the positive-upwind path evaluates the element state per pass: defect, then Jacobian
        const cudaError_t e = launch_defect_ipshape(roid, P, a, s);
        return e != cudaSuccess ? e : launch_jacobian_ipshape(roid, P, a, prec, s);
    }
    if (prec != 0) {
        // FP32 blocks: the FP64 defect, then the lane-per-corner FP32 Jacobian of the
        // same colour (faster than forming FP32 blocks inside the FP64 pass)
        const cudaError_t e = launch_defect(roid, P, a, s, threads);
        return e != cudaSuccess ? e : launch_jacobian_lanes(roid, P, a, s);
    }
    const int t = clamp_threads(threads);
    const int grid = (a.count + t - 1) / t;
    return dispatch_roid(roid, [&](auto r) {
        constexpr int RO = decltype(r)::value;
        const bool pac = P.pac && !P.stokes;
        if (P.transient) {
            if (pac) k_defect_jacobian<RO, true, true><<<grid, t, 0, s>>>(P, a);
            else k_defect_jacobian<RO, true, false><<<grid, t, 0, s>>>(P, a);
        } else {
            if (pac) k_defect_jacobian<RO, false, true><<<grid, t, 0, s>>>(P, a);
            else k_defect_jacobian<RO, false, false><<<grid, t, 0, s>>>(P, a);
        }
    });
}

cudaError_t launch_elem_batch(int roid, const DiscParams& P, const ElemBatchArgs& a, cudaStream_t s) {
    if (a.n <= 0) return cudaSuccess;
    const int grid = (int)((a.n + kThreads - 1) / kThreads);
    if (uses_ipshape(P)) {
        // mass and source parts here, the stiffness parts on the positive-upwind path
        ElemBatchArgs m = a;
        m.defA = nullptr;
        m.jacA = nullptr;
        const cudaError_t e = dispatch_roid(roid, [&](auto r) { k_elem_batch<decltype(r)::value><<<grid, kThreads, 0, s>>>(P, m); });
        return e != cudaSuccess ? e : launch_elem_batch_ipshape(roid, P, a, s);
    }
    return dispatch_roid(roid, [&](auto r) { k_elem_batch<decltype(r)::value><<<grid, kThreads, 0, s>>>(P, a); });
}

cudaError_t launch_bnd_flux(int b, int64_t nNodes, double scale, const double* flux, double* D, cudaStream_t s) {
    if (!flux || nNodes <= 0) return cudaSuccess;
    k_bnd_flux<<<(int)((nNodes + 255) / 256), 256, 0, s>>>(b, nNodes, scale, flux, D);
    return cudaGetLastError();
}

cudaError_t launch_dirichlet(int b, int64_t n, const int32_t* rows, const double* vals, const int32_t* rowPtr,
                             const int32_t* colIdx, const double* U, double* D, void* J, int prec, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    const int grid = (int)((n + 255) / 256);
    if (prec == 0) k_dirichlet<double><<<grid, 256, 0, s>>>(b, n, rows, vals, rowPtr, colIdx, U, D, (double*)J);
    else k_dirichlet<float><<<grid, 256, 0, s>>>(b, n, rows, vals, rowPtr, colIdx, U, D, (float*)J);
    return cudaGetLastError();
}

}  // namespace nsfv1
