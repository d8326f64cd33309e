// nsfv1_asm_common.cuh -- what the assembly kernels share: the element gather
// (corner coordinates, nodal states), the compile-time bounds checks and the
// sinks that take the element's fluxes and Jacobian blocks into the global
// defect / block-CSR matrix or into element-local arrays.
#pragma once

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
                float v[4];
#pragma unroll
                for (int c = 0; c < 4; ++c) v[c] = plus ? (float)B[r][c] : flip_sign((float)B[r][c]);
                asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(p + r * 4), "f"(v[0]), "f"(v[1]), "f"(v[2]),
                             "f"(v[3])
                             : "memory");
            }
        } else {
#pragma unroll
            for (int r = 0; r < b; ++r)
#pragma unroll
                for (int c = 0; c < b; ++c) {
                    const VT v = (VT)B[r][c];
                    atomicAdd(p + r * b + c, plus ? v : flip_sign(v));
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

}  // namespace nsfv1
