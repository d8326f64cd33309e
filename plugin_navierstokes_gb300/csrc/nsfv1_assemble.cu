// FV1 assembly kernels for sm_103a: one thread per element, elements of one
// colour per launch (no two share a node). The scatter into the global defect /
// block-CSR Jacobian uses fire-and-forget L2 reductions (red.global.add); within
// a colour every address is updated by one thread only, so the summation order
// per entry is fixed (colour order, then SCVF order): runs are bitwise
// reproducible.
#include <type_traits>
#include "nsfv1_internal.h"
#include "nsfv1_elem.cuh"

// NSFV1_BOUNDS_CHECK (compile-time; the bounds-checked library variant): every
// node id read from the connectivity and every block index of the scatter is
// checked against the mesh; an index out of range sets bit 2 of the handle's
// error word (NSFV1_ERR_ARGUMENT on the host) and the access is skipped. This
// replaces the reference's UG_NSUPWIND_ASSERT / UG_NSSTAB_ASSERT bounds asserts
// (upwind_interface.h:36-38, stabilization.h:36-38) without trapping the GPU.
#ifdef NSFV1_BOUNDS_CHECK
#define NSFV1_IN_RANGE(i, n, err) (((int64_t)(i) >= 0 && (int64_t)(i) < (int64_t)(n)) ? true : (atomicOr((err), 4), false))
#else
#define NSFV1_IN_RANGE(i, n, err) true
#endif

namespace nsfv1 {

static constexpr int kThreads = 128;

// ---- element gather --------------------------------------------------------

// Corner coordinates; in float mode relative to corner 0 (all geometry used is
// translation invariant) so that single precision keeps the local detail.
template <int ROID, typename T>
__device__ __forceinline__ void load_corners(const double* __restrict__ coords, const int32_t (&nodes)[Ref<ROID>::nsh], Elem<ROID, T>& E) {
    using R = Ref<ROID>;
    constexpr int dim = R::dim, nsh = R::nsh;
    if constexpr (std::is_same<T, double>::value) {
#pragma unroll
        for (int k = 0; k < nsh; ++k)
#pragma unroll
            for (int d = 0; d < dim; ++d) E.x[k][d] = __ldg(coords + (int64_t)nodes[k] * dim + d);
    } else {
        double x0[dim];
#pragma unroll
        for (int d = 0; d < dim; ++d) x0[d] = __ldg(coords + (int64_t)nodes[0] * dim + d);
#pragma unroll
        for (int k = 0; k < nsh; ++k)
#pragma unroll
            for (int d = 0; d < dim; ++d) E.x[k][d] = (T)(__ldg(coords + (int64_t)nodes[k] * dim + d) - x0[d]);
    }
}

template <int ROID, typename T>
__device__ __forceinline__ void load_u(const double* __restrict__ U, const int32_t (&nodes)[Ref<ROID>::nsh], T (&u)[Ref<ROID>::b][Ref<ROID>::nsh]) {
    using R = Ref<ROID>;
    constexpr int b = R::b, nsh = R::nsh;
#pragma unroll
    for (int k = 0; k < nsh; ++k) {
        if constexpr (b == 4) {
            const double2* p = reinterpret_cast<const double2*>(U + (int64_t)nodes[k] * 4);
            const double2 a = __ldg(p), c = __ldg(p + 1);
            u[0][k] = (T)a.x; u[1][k] = (T)a.y; u[2][k] = (T)c.x; u[3][k] = (T)c.y;
        } else {
#pragma unroll
            for (int f = 0; f < b; ++f) u[f][k] = (T)__ldg(U + (int64_t)nodes[k] * b + f);
        }
    }
}

// ---- sinks for the local Jacobian blocks ------------------------------------

template <typename VT, int nsh>
struct GlobalJacSink {
    VT* __restrict__ vals;
    const int32_t* __restrict__ blk;   // this element's [nsh][nsh] block indices
    int64_t nnzb = 0;                  // checked with NSFV1_BOUNDS_CHECK
    int* err = nullptr;
    template <int b, typename T>
    __device__ __forceinline__ void add(const int i, const int k, const T (&B)[b][b], const bool plus) {
        // fire-and-forget reductions (executed in L2, no load latency); within a
        // colour no other thread touches this block and one thread's updates to an
        // address apply in program order, so the sums stay deterministic
        const int32_t q = __ldg(blk + i * nsh + k);
        if (!NSFV1_IN_RANGE(q, nnzb, err)) return;
        VT* p = vals + (int64_t)q * (b * b);
        if constexpr (std::is_same<VT, float>::value && b == 4) {
            // one 16-byte vector reduction per block row (the value array is 16-byte aligned)
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                const float s = plus ? 1.f : -1.f;
                asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(p + r * 4), "f"(s * (float)B[r][0]),
                             "f"(s * (float)B[r][1]), "f"(s * (float)B[r][2]), "f"(s * (float)B[r][3])
                             : "memory");
            }
        } else {
#pragma unroll
            for (int r = 0; r < b; ++r)
#pragma unroll
                for (int c = 0; c < b; ++c) {
                    const VT v = (VT)B[r][c];
                    atomicAdd(p + r * b + c, plus ? v : -v);
                }
        }
    }
};

template <int nsh>
struct LocalJacSink {
    double* __restrict__ J;   // element-local [(f1 * nsh + s1) * b + f2] * nsh + s2
    template <int b, typename T>
    __device__ __forceinline__ void add(int i, int k, const T (&B)[b][b], bool plus) {
#pragma unroll
        for (int r = 0; r < b; ++r)
#pragma unroll
            for (int c = 0; c < b; ++c) {
                double* q = J + ((r * nsh + i) * b + c) * nsh + k;
                *q = plus ? *q + (double)B[r][c] : *q - (double)B[r][c];
            }
    }
};

// ---- global assembly kernels -------------------------------------------------

// defect sink of the global assembly: reductions into D[node * b + fct]
template <int nsh, int b>
struct GlobalDefSink {
    double* __restrict__ D;
    int32_t nodes[nsh];
    __device__ __forceinline__ void add(const int i, const int f, const double v) {
        int32_t n = nodes[0];
#pragma unroll
        for (int k = 1; k < nsh; ++k) n = (k == i) ? nodes[k] : n;
        atomicAdd(D + (int64_t)n * b + f, v);
    }
};

// defect sink of the element-local callbacks: dA[f][corner]
template <int nsh, int b>
struct LocalDefSink {
    double (&dA)[b][nsh];
    __device__ __forceinline__ void add(const int i, const int f, const double v) {
#pragma unroll
        for (int k = 0; k < nsh; ++k)
            if (k == i) dA[f][k] += v;
    }
};

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
template <int ROID, bool TRANSIENT, typename VT, bool PAC>
__global__ void __launch_bounds__(kThreads) k_defect_jacobian(const DiscParams P, const AsmArgs A) {
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
    if constexpr (std::is_same<VT, double>::value) {
        if constexpr (TRANSIENT) ok = elem_def_jac_A<ROID, double, PAC>(Q, E, u, uoRef, ss, P.dt, jsink, nuEl);
        else ok = elem_def_jac_A<ROID, double, PAC>(Q, E, u, uoRef, sink, 1.0, jsink, nuEl);
    } else {
        if constexpr (TRANSIENT) ok = elem_def_jac_A_mixed<ROID, PAC>(Q, E, u, uoRef, ss, (float)P.dt, jsink, nuEl);
        else ok = elem_def_jac_A_mixed<ROID, PAC>(Q, E, u, uoRef, sink, 1.0f, jsink, nuEl);
    }
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
    const int t = clamp_threads(threads);
    const int grid = (a.count + t - 1) / t;
    return dispatch_roid(roid, [&](auto r) {
        if (P.transient) k_defect<decltype(r)::value, true><<<grid, t, 0, s>>>(P, a);
        else k_defect<decltype(r)::value, false><<<grid, t, 0, s>>>(P, a);
    });
}

cudaError_t launch_jacobian(int roid, const DiscParams& P, const AsmArgs& a, int prec, cudaStream_t s, int threads) {
    if (a.count <= 0) return cudaSuccess;
    const int t = clamp_threads(threads);
    const int grid = (a.count + t - 1) / t;
    return dispatch_roid(roid, [&](auto r) {
        constexpr int RO = decltype(r)::value;
        if (P.pac && !P.stokes) {
            if (prec == 0) k_jacobian<RO, double, double, true><<<grid, t, 0, s>>>(P, a);
            else k_jacobian<RO, float, float, true><<<grid, t, 0, s>>>(P, a);
        } else {
            if (prec == 0) k_jacobian<RO, double, double, false><<<grid, t, 0, s>>>(P, a);
            else k_jacobian<RO, float, float, false><<<grid, t, 0, s>>>(P, a);
        }
    });
}

cudaError_t launch_defect_jacobian(int roid, const DiscParams& P, const AsmArgs& a, int prec, cudaStream_t s, int threads) {
    if (a.count <= 0) return cudaSuccess;
    const int t = clamp_threads(threads);
    const int grid = (a.count + t - 1) / t;
    return dispatch_roid(roid, [&](auto r) {
        constexpr int RO = decltype(r)::value;
        const bool pac = P.pac && !P.stokes;
        if (prec == 0) {
            if (P.transient) {
                if (pac) k_defect_jacobian<RO, true, double, true><<<grid, t, 0, s>>>(P, a);
                else k_defect_jacobian<RO, true, double, false><<<grid, t, 0, s>>>(P, a);
            } else {
                if (pac) k_defect_jacobian<RO, false, double, true><<<grid, t, 0, s>>>(P, a);
                else k_defect_jacobian<RO, false, double, false><<<grid, t, 0, s>>>(P, a);
            }
        } else {
            if (P.transient) {
                if (pac) k_defect_jacobian<RO, true, float, true><<<grid, t, 0, s>>>(P, a);
                else k_defect_jacobian<RO, true, float, false><<<grid, t, 0, s>>>(P, a);
            } else {
                if (pac) k_defect_jacobian<RO, false, float, true><<<grid, t, 0, s>>>(P, a);
                else k_defect_jacobian<RO, false, float, false><<<grid, t, 0, s>>>(P, a);
            }
        }
    });
}

cudaError_t launch_elem_batch(int roid, const DiscParams& P, const ElemBatchArgs& a, cudaStream_t s) {
    if (a.n <= 0) return cudaSuccess;
    const int grid = (int)((a.n + kThreads - 1) / kThreads);
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
