// Device linear algebra on the handle's block-CSR pattern and the Newton
// driver: block SpMV, point-block Jacobi (inverted b x b diagonal blocks),
// right-preconditioned BiCGStab and restarted GMRES, FP64 defect norms.
// The Jacobian and its block inverses are stored in MT (double for the plain
// method, float for the FP32-Jacobian mode); Krylov vectors are FP64 in both;
// reductions accumulate in FP64 with a fixed grid and a fixed summation tree,
// so results are bitwise reproducible run to run.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <type_traits>
#include <vector>
#include "nsfv1_internal.h"
#include "nsfv1_host.h"
#include "nsfv1_linalg.cuh"
#include "../../include/nsfv1_gb300.h"

namespace nsfv1 {

static constexpr int kRedBlocks = 608;   // 4 x 152 SMs
static constexpr int kRedThreads = 256;

// ---------------------------------------------------------------------------
// block SpMV y = A x: one group of G lanes per block row; lane l takes the
// blocks l, l+G, ... of the row (consecutive lanes read consecutive blocks)
// and applies each whole b x b block to the b entries of x it multiplies, so
// every matrix entry costs one fused multiply-add; the group then reduces its
// b row sums with butterfly shuffles in a fixed order, and lane r stores component r
// (a warp-wide FP64 instruction costs its full issue time however few lanes are
// active, so the conversions are spread over the lanes).
//
// GB300 issues only two FP64 instructions per clock per SM, so the FP32-matrix
// variant keeps its arithmetic off the FP64 pipe: x (FP64) is split into two
// floats by integer operations (xh = the leading 24 bits, xl = the next ones),
// and the products are accumulated in double-float (TwoSum of the FP32
// products plus their exact FMA errors), converted to FP64 once per row. The
// result is accurate to about 1e-13 of sum |a x|, far below the FP32 rounding
// of the matrix itself, at a handful of FP32/INT operations per entry.
// ---------------------------------------------------------------------------
struct DFloat {
    float hi, lo;
};

// x = xh + xl (+ |x| 2^-47): both floats from the bits of x by integer operations
// only (GB300 has little FP64 throughput, and a conversion would use it).
// |x| < 2^-126 flushes to 0; |x| >= 2^128 becomes +-inf; nan stays nan.
__device__ __forceinline__ void split_double(double x, float& xh, float& xl) {
    const unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
    const unsigned e = (hi >> 20) & 0x7FFu;
    const unsigned sgn = hi & 0x80000000u;
    const unsigned mh = hi & 0xFFFFFu;                    // top 20 mantissa bits
    // leading 23 mantissa bits: mh (20) and the top 3 bits of lo
    const unsigned m23 = (mh << 3) | (lo >> 29);
    const unsigned r = lo & 0x1FFFFFFFu;                  // the 29 mantissa bits below them
    unsigned hbits;
    if (e >= 897u && e <= 1150u) hbits = sgn | ((e - 896u) << 23) | m23;
    else if (e > 1150u) hbits = sgn | 0x7F800000u | ((e == 0x7FFu && (mh | lo)) ? 0x400000u : 0u);
    else hbits = sgn;
    xh = __uint_as_float(hbits);
    // xl = +-r 2^(e - 1075) when that is a normal float (e >= 949), else 0
    const bool has_lo = (e >= 949u) && (e <= 1150u) && (r != 0u);
    const float scale = __uint_as_float(((has_lo ? e : 1075u) - 1075u + 127u) << 23);
    xl = has_lo ? __uint_as_float(__float_as_uint(__uint2float_rn(r) * scale) | sgn) : 0.f;
}

// a + b exactly as s + err (Knuth's TwoSum; _rn intrinsics keep the compiler
// from contracting or reassociating the error-free steps)
__device__ __forceinline__ float two_sum(float a, float b, float& err) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    err = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return s;
}

template <typename MT, typename XT, int b>
struct RowAcc;

template <typename XT, int b>
struct RowAcc<double, XT, b> {
    double v[b];
    __device__ __forceinline__ void zero() {
#pragma unroll
        for (int i = 0; i < b; ++i) v[i] = 0.0;
    }
    __device__ __forceinline__ void block(const double* __restrict__ blk, const XT* __restrict__ xc) {
        double x[b];
#pragma unroll
        for (int j = 0; j < b; ++j) x[j] = (double)__ldg(xc + j);
#pragma unroll
        for (int i = 0; i < b; ++i)
#pragma unroll
            for (int j = 0; j < b; ++j) v[i] = fma(__ldg(blk + i * b + j), x[j], v[i]);
    }
    // butterfly: every lane of the group ends with the sums
    template <int G>
    __device__ __forceinline__ void reduce() {
#pragma unroll
        for (int off = G / 2; off > 0; off >>= 1)
#pragma unroll
            for (int i = 0; i < b; ++i) v[i] += __shfl_xor_sync(0xffffffffu, v[i], off, G);
    }
    __device__ __forceinline__ double value(int i) const {
        double r = v[0];
#pragma unroll
        for (int k = 1; k < b; ++k) r = (i == k) ? v[k] : r;
        return r;
    }
};

template <int b>
struct RowAcc<float, double, b> {
    DFloat v[b];
    __device__ __forceinline__ void zero() {
#pragma unroll
        for (int i = 0; i < b; ++i) v[i] = DFloat{0.f, 0.f};
    }
    __device__ __forceinline__ void block(const float* __restrict__ blk, const double* __restrict__ xc) {
        float xh[b], xl[b];
#pragma unroll
        for (int j = 0; j < b; ++j) split_double(__ldg(xc + j), xh[j], xl[j]);
        accumulate(blk, xh, xl);
    }
    // x already split (split_double by the kernel that produced it): the same products
    __device__ __forceinline__ void block(const float* __restrict__ blk, const float2* __restrict__ xc) {
        float xh[b], xl[b];
#pragma unroll
        for (int j = 0; j < b; ++j) {
            const float2 t = __ldg(xc + j);
            xh[j] = t.x; xl[j] = t.y;
        }
        accumulate(blk, xh, xl);
    }
    __device__ __forceinline__ void accumulate(const float* __restrict__ blk, const float (&xh)[b], const float (&xl)[b]) {
#pragma unroll
        for (int i = 0; i < b; ++i)
#pragma unroll
            for (int j = 0; j < b; ++j) {
                const float a = __ldg(blk + i * b + j);
                const float p = __fmul_rn(a, xh[j]);
                const float pe = fmaf(a, xh[j], -p);   // a xh = p + pe exactly
                float e;
                v[i].hi = two_sum(v[i].hi, p, e);
                v[i].lo += e + fmaf(a, xl[j], pe);
            }
    }
    template <int G>
    __device__ __forceinline__ void reduce() {
#pragma unroll
        for (int off = G / 2; off > 0; off >>= 1)
#pragma unroll
            for (int i = 0; i < b; ++i) {
                const float oh = __shfl_xor_sync(0xffffffffu, v[i].hi, off, G);
                const float ol = __shfl_xor_sync(0xffffffffu, v[i].lo, off, G);
                float e;
                v[i].hi = two_sum(v[i].hi, oh, e);
                v[i].lo += e + ol;
            }
    }
    // component i in FP64: the float pair is selected first, so a lane converts one value
    __device__ __forceinline__ double value(int i) const {
        float h = v[0].hi, l = v[0].lo;
#pragma unroll
        for (int k = 1; k < b; ++k) {
            h = (i == k) ? v[k].hi : h;
            l = (i == k) ? v[k].lo : l;
        }
        return (double)h + (double)l;
    }
};

template <int b>
struct RowAcc<float, float, b> {
    float v[b];
    __device__ __forceinline__ void zero() {
#pragma unroll
        for (int i = 0; i < b; ++i) v[i] = 0.f;
    }
    __device__ __forceinline__ void block(const float* __restrict__ blk, const float* __restrict__ xc) {
        float x[b];
#pragma unroll
        for (int j = 0; j < b; ++j) x[j] = __ldg(xc + j);
#pragma unroll
        for (int i = 0; i < b; ++i)
#pragma unroll
            for (int j = 0; j < b; ++j) v[i] = fmaf(__ldg(blk + i * b + j), x[j], v[i]);
    }
    template <int G>
    __device__ __forceinline__ void reduce() {
#pragma unroll
        for (int off = G / 2; off > 0; off >>= 1)
#pragma unroll
            for (int i = 0; i < b; ++i) v[i] += __shfl_xor_sync(0xffffffffu, v[i], off, G);
    }
    __device__ __forceinline__ float value(int i) const {
        float r = v[0];
#pragma unroll
        for (int k = 1; k < b; ++k) r = (i == k) ? v[k] : r;
        return r;
    }
};

// gate: null, or a flag in device memory; a nonzero flag makes the launch a no-op
// (the BiCGStab iterations queued after the solver stopped)
template <typename VT, typename XT, int b, int G>
__global__ void __launch_bounds__(256) k_bsr_mv(int64_t nRows, const int32_t* __restrict__ rowPtr, const int32_t* __restrict__ colIdx,
                                                const VT* __restrict__ vals, const XT* __restrict__ x, XT* __restrict__ y,
                                                const double* __restrict__ gate) {
    static_assert(G >= b, "a lane per row component");
    if (gate && *gate != 0.0) return;
    const int64_t gid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t row = gid / G;
    const int lane = threadIdx.x % G;
    // rows past the end run the (empty) loop so every lane reaches the shuffles
    const bool valid = row < nRows;
    // block indices fit in 32 bits (the pattern is built with int32 row pointers)
    const int q0 = valid ? rowPtr[row] : 0, q1 = valid ? rowPtr[row + 1] : 0;
    RowAcc<VT, XT, b> acc;
    acc.zero();
    for (int q = q0 + lane; q < q1; q += G) acc.block(vals + (size_t)q * (b * b), x + (size_t)__ldg(colIdx + q) * b);
    acc.template reduce<G>();
    // lanes 0..b-1 of the group each store one component (G >= b)
    if (valid && lane < b) y[row * b + lane] = (XT)acc.value(lane);
}

// xs[i] = split_double(x[i]) (the SpMV operand of k_bsr_mv_split)
__global__ void k_split_vector(int64_t n, const double* __restrict__ x, float2* __restrict__ xs) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float h, l;
    split_double(x[i], h, l);
    xs[i] = make_float2(h, l);
}

// k_bsr_mv for an FP32 matrix and an FP64 x stored as split float pairs (xs[i] =
// split_double(x[i])): the FP64 result of k_bsr_mv<float, double>, bit for bit,
// without the split per block
template <int b, int G>
__global__ void __launch_bounds__(256) k_bsr_mv_split(int64_t nRows, const int32_t* __restrict__ rowPtr, const int32_t* __restrict__ colIdx,
                                                      const float* __restrict__ vals, const float2* __restrict__ xs, double* __restrict__ y,
                                                      const double* __restrict__ gate) {
    static_assert(G >= b, "a lane per row component");
    if (gate && *gate != 0.0) return;
    const int64_t gid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t row = gid / G;
    const int lane = threadIdx.x % G;
    const bool valid = row < nRows;
    const int q0 = valid ? rowPtr[row] : 0, q1 = valid ? rowPtr[row + 1] : 0;
    RowAcc<float, double, b> acc;
    acc.zero();
    for (int q = q0 + lane; q < q1; q += G) acc.block(vals + (size_t)q * (b * b), xs + (size_t)__ldg(colIdx + q) * b);
    acc.template reduce<G>();
    if (valid && lane < b) y[row * b + lane] = acc.value(lane);
}

template <typename VT, typename OT, int b>
__global__ void k_block_inv(int64_t nRows, const int32_t* __restrict__ diagPos, const VT* __restrict__ vals, OT* __restrict__ Dinv, int* err) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nRows) return;
    if (!block_inverse<b>(vals + (int64_t)diagPos[r] * b * b, Dinv + r * b * b)) atomicOr(err, 2);
}

// out = Dinv in per node block (Dinv of type MT, vectors of type VT, products in VT)
template <typename MT, typename VT, int b>
__global__ void k_prec(int64_t nRows, const MT* __restrict__ Dinv, const VT* __restrict__ in, VT* __restrict__ out) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nRows) return;
    VT x[b];
#pragma unroll
    for (int j = 0; j < b; ++j) x[j] = in[r * b + j];
    const MT* M = Dinv + r * b * b;
#pragma unroll
    for (int i = 0; i < b; ++i) {
        VT a = VT(0);
#pragma unroll
        for (int j = 0; j < b; ++j) a += (VT)M[i * b + j] * x[j];
        out[r * b + i] = a;
    }
}

// ---------------------------------------------------------------------------
// deterministic reductions: K dot products at once, partials per block, then
// one block sums the partials in a fixed order.
// pairs: dot_k = sum a_k[i] * c_k[i]
// ---------------------------------------------------------------------------
template <typename VT, int K>
struct DotArgs { const VT* a[K]; const VT* c[K]; };

template <typename VT, int K>
__global__ void __launch_bounds__(kRedThreads) k_dot_partial(int64_t n, DotArgs<VT, K> A, double* __restrict__ partials,
                                                             const double* __restrict__ gate) {
    if (gate && *gate != 0.0) return;
    __shared__ double sh[K][kRedThreads];
    double acc[K];
#pragma unroll
    for (int k = 0; k < K; ++k) acc[k] = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * kRedThreads + threadIdx.x; i < n; i += (int64_t)gridDim.x * kRedThreads) {
#pragma unroll
        for (int k = 0; k < K; ++k) acc[k] += (double)A.a[k][i] * (double)A.c[k][i];
    }
#pragma unroll
    for (int k = 0; k < K; ++k) sh[k][threadIdx.x] = acc[k];
    __syncthreads();
    for (int s = kRedThreads / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) {
#pragma unroll
            for (int k = 0; k < K; ++k) sh[k][threadIdx.x] += sh[k][threadIdx.x + s];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < K; ++k) partials[k * gridDim.x + blockIdx.x] = sh[k][0];
    }
}

// sums K x nb partials into out[k] (one block, fixed order)
template <int K>
__device__ __forceinline__ void block_sum_partials(const double* __restrict__ partials, int nb, double* out) {
    __shared__ double sh[K][kRedThreads];
    double acc[K];
#pragma unroll
    for (int k = 0; k < K; ++k) acc[k] = 0.0;
    for (int i = threadIdx.x; i < nb; i += kRedThreads)
#pragma unroll
        for (int k = 0; k < K; ++k) acc[k] += partials[k * nb + i];
#pragma unroll
    for (int k = 0; k < K; ++k) sh[k][threadIdx.x] = acc[k];
    __syncthreads();
    for (int s = kRedThreads / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) {
#pragma unroll
            for (int k = 0; k < K; ++k) sh[k][threadIdx.x] += sh[k][threadIdx.x + s];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < K; ++k) out[k] = sh[k][0];
    }
}

// scalar slots of the BiCGStab state in ws.scal
// S_DONE: 0 while iterating; set by the end-of-iteration kernel to 1 (converged), 2 (non-finite
// residual) or 3 (breakdown: restart), after which every kernel of the iteration returns at once.
// S_ITER counts the iterations run.
enum { S_RHO = 0, S_ALPHA, S_OMEGA, S_RHO1, S_BETA, S_R0V, S_TS, S_TT, S_NR2, S_NR02, S_FLAG, S_DONE, S_ITER, S_NSCAL = 16 };
enum { DONE_CONVERGED = 1, DONE_NONFINITE = 2, DONE_BREAKDOWN = 3 };

template <int K>
__global__ void k_dot_final(const double* partials, int nb, double* out) { block_sum_partials<K>(partials, nb, out); }

// rho1 = (r0, r); beta = (rho1 / rho) * (alpha / omega)
__global__ void k_bicg_beta(const double* partials, int nb, double* S) {
    double v[1];
    block_sum_partials<1>(partials, nb, v);
    if (threadIdx.x == 0) {
        S[S_RHO1] = v[0];
        double beta = (v[0] / S[S_RHO]) * (S[S_ALPHA] / S[S_OMEGA]);
        // breakdown: rho1 = 0 or a non-finite beta (relative thresholds restart far too often
        // on the convection-dominated systems, where a large beta is ordinary)
        if (v[0] == 0.0 || !isfinite(beta)) { S[S_FLAG] = 1.0; beta = 0.0; }
        S[S_BETA] = beta;
    }
}

// ---- fused BiCGStab steps (FP64 Krylov vectors, Jacobian / inverse blocks of type MT) ----

// sums the per-thread values v[k] of one block in a fixed tree into partials[k * gridDim.x + block]
template <int K>
__device__ __forceinline__ void block_partials(double (&v)[K], double* __restrict__ partials) {
    __shared__ double sh[K][kRedThreads];
#pragma unroll
    for (int k = 0; k < K; ++k) sh[k][threadIdx.x] = v[k];
    __syncthreads();
    for (int st = kRedThreads / 2; st > 0; st >>= 1) {
        if (threadIdx.x < st) {
#pragma unroll
            for (int k = 0; k < K; ++k) sh[k][threadIdx.x] += sh[k][threadIdx.x + st];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < K; ++k) partials[k * gridDim.x + blockIdx.x] = sh[k][0];
    }
}

// After block_partials<K>: the block that finishes last (counted in *counter)
// sums the partials of all blocks, in block order (the sums of block_sum_partials),
// into out (valid in thread 0) and returns true; the counter is left at 0.
// Partials are read past L1 (other SMs wrote them).
template <int K>
__device__ __forceinline__ bool last_block_sum(const double* __restrict__ partials, unsigned* counter, double (&out)[K]) {
    __shared__ bool amLast;
    __shared__ double sh[K][kRedThreads];
    if (threadIdx.x == 0) {
        __threadfence();
        amLast = atomicAdd(counter, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!amLast) return false;
    __threadfence();
    const int nb = gridDim.x;
    double acc[K];
#pragma unroll
    for (int k = 0; k < K; ++k) acc[k] = 0.0;
    for (int i = threadIdx.x; i < nb; i += kRedThreads)
#pragma unroll
        for (int k = 0; k < K; ++k) acc[k] += __ldcg(partials + k * nb + i);
#pragma unroll
    for (int k = 0; k < K; ++k) sh[k][threadIdx.x] = acc[k];
    __syncthreads();
    for (int st = kRedThreads / 2; st > 0; st >>= 1) {
        if (threadIdx.x < st) {
#pragma unroll
            for (int k = 0; k < K; ++k) sh[k][threadIdx.x] += sh[k][threadIdx.x + st];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < K; ++k) out[k] = sh[k][0];
        *counter = 0u;
    }
    return true;
}

// out = Dinv_row x (the point-block Jacobi apply of k_prec, same summation)
template <typename MT, int b>
__device__ __forceinline__ void prec_row(const MT* __restrict__ M, const double (&x)[b], double* __restrict__ out) {
#pragma unroll
    for (int i = 0; i < b; ++i) {
        double a = 0.0;
#pragma unroll
        for (int j = 0; j < b; ++j) a += (double)M[i * b + j] * x[j];
        out[i] = a;
    }
}

// the preconditioned vector of a row, and for FP32 matrices its split float pairs
// (the SpMV's x operand, k_bsr_mv_split). With FP32 blocks the products run in
// double-float on the FP32 pipe (x split by integer operations, exact products,
// TwoSum sums: about 1e-14 of sum |M x|) and only the result goes to FP64 (two
// conversions and an add per entry): GB300's FP64 pipe would otherwise spend b
// conversions and b FMAs per entry on it.
template <typename MT, int b>
__device__ __forceinline__ void prec_row_out(const MT* __restrict__ M, const double (&x)[b], double* __restrict__ out,
                                             float2* __restrict__ outSplit) {
    if constexpr (std::is_same<MT, float>::value) {
        float xh[b], xl[b];
#pragma unroll
        for (int j = 0; j < b; ++j) split_double(x[j], xh[j], xl[j]);
#pragma unroll
        for (int i = 0; i < b; ++i) {
            float hi = 0.f, lo = 0.f;
#pragma unroll
            for (int j = 0; j < b; ++j) {
                const float a = __ldg(M + i * b + j);
                const float pr = __fmul_rn(a, xh[j]);
                const float pe = fmaf(a, xh[j], -pr);   // a xh = pr + pe exactly
                float e;
                hi = two_sum(hi, pr, e);
                lo += e + fmaf(a, xl[j], pe);
            }
            const double z = (double)hi + (double)lo;
            out[i] = z;
            float h, l;
            split_double(z, h, l);
            outSplit[i] = make_float2(h, l);
        }
    } else {
        double z[b];
        prec_row<MT, b>(M, x, z);
#pragma unroll
        for (int i = 0; i < b; ++i) out[i] = z[i];
    }
}

// p = r + beta (p - omega v); ph = Dinv p
template <typename MT, int b>
__global__ void k_bicg_p_prec(int64_t nRows, const double* __restrict__ S, const double* __restrict__ r, const double* __restrict__ v,
                              double* __restrict__ p, const MT* __restrict__ Dinv, double* __restrict__ ph, float2* __restrict__ phs) {
    const int64_t row = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= nRows || S[S_DONE] != 0.0) return;
    const double beta = S[S_BETA], omega = S[S_OMEGA];
    double x[b];
#pragma unroll
    for (int j = 0; j < b; ++j) {
        const int64_t i = row * b + j;
        x[j] = r[i] + beta * (p[i] - omega * v[i]);
        p[i] = x[j];
    }
    prec_row_out<MT, b>(Dinv + row * b * b, x, ph + row * b, phs + row * b);
}

// s = r - alpha v; sh = Dinv s
template <typename MT, int b>
__global__ void k_bicg_s_prec(int64_t nRows, const double* __restrict__ S, const double* __restrict__ r, const double* __restrict__ v,
                              double* __restrict__ sv, const MT* __restrict__ Dinv, double* __restrict__ shv, float2* __restrict__ shs) {
    const int64_t row = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= nRows || S[S_DONE] != 0.0) return;
    const double alpha = S[S_ALPHA];
    double x[b];
#pragma unroll
    for (int j = 0; j < b; ++j) {
        const int64_t i = row * b + j;
        x[j] = r[i] - alpha * v[i];
        sv[i] = x[j];
    }
    prec_row_out<MT, b>(Dinv + row * b * b, x, shv + row * b, shs + row * b);
}

// x += alpha ph + omega sh; r = s - omega t; partials of (r, r) and (r0, r)
// (the grid-stride layout of k_dot_partial, kRedBlocks blocks)

// the scalar updates that follow the reductions (thread 0 of the last block)
__device__ __forceinline__ void bicg_alpha_update(double* S, const double r0v) {
    S[S_R0V] = r0v;
    double alpha = (r0v != 0.0) ? S[S_RHO1] / r0v : 0.0;
    if (r0v == 0.0 || !isfinite(alpha)) { S[S_FLAG] = 1.0; alpha = 0.0; }
    S[S_ALPHA] = alpha;
}
__device__ __forceinline__ void bicg_omega_update(double* S, const double ts, const double tt) {
    S[S_TS] = ts; S[S_TT] = tt;
    const double omega = (tt != 0.0) ? ts / tt : 0.0;
    S[S_OMEGA] = isfinite(omega) ? omega : 0.0;
}

// (r0, v) and alpha in one launch (k_dot_partial's grid and tree, then the last block)
__global__ void __launch_bounds__(kRedThreads) k_bicg_dot_alpha(int64_t n, const double* __restrict__ r0, const double* __restrict__ v,
                                                                 double* __restrict__ partials, unsigned* counter, double* S) {
    if (S[S_DONE] != 0.0) return;
    double d[1] = {0.0};
    for (int64_t i = (int64_t)blockIdx.x * kRedThreads + threadIdx.x; i < n; i += (int64_t)gridDim.x * kRedThreads)
        d[0] += r0[i] * v[i];
    block_partials<1>(d, partials);
    double tot[1];
    if (last_block_sum<1>(partials, counter, tot) && threadIdx.x == 0) bicg_alpha_update(S, tot[0]);
}

// (t, s), (t, t) and omega in one launch
__global__ void __launch_bounds__(kRedThreads) k_bicg_dot_omega(int64_t n, const double* __restrict__ t, const double* __restrict__ sv,
                                                                 double* __restrict__ partials, unsigned* counter, double* S) {
    if (S[S_DONE] != 0.0) return;
    double d[2] = {0.0, 0.0};
    for (int64_t i = (int64_t)blockIdx.x * kRedThreads + threadIdx.x; i < n; i += (int64_t)gridDim.x * kRedThreads) {
        const double ti = t[i];
        d[0] += ti * sv[i];
        d[1] += ti * ti;
    }
    block_partials<2>(d, partials);
    double tot[2];
    if (last_block_sum<2>(partials, counter, tot) && threadIdx.x == 0) bicg_omega_update(S, tot[0], tot[1]);
}

// end of an iteration (thread 0 of the last block of k_bicg_x_end): ||r||^2, the stop
// tests of the host loop (finite, converged, breakdown), then the next iteration's
// rho1 = (r0, r) and beta (as k_bicg_beta)
__device__ __forceinline__ void bicg_end_update(double* S, const double (&v)[2], const double nr0, const double rtol) {
    S[S_NR2] = v[0];
    S[S_RHO] = S[S_RHO1];
    S[S_ITER] += 1.0;
    const double nr = sqrt(v[0]);
    if (!isfinite(nr)) { S[S_DONE] = DONE_NONFINITE; return; }
    if (nr / nr0 < rtol) { S[S_DONE] = DONE_CONVERGED; return; }
    if (S[S_FLAG] != 0.0 || S[S_OMEGA] == 0.0) { S[S_DONE] = DONE_BREAKDOWN; return; }
    S[S_RHO1] = v[1];
    double beta = (v[1] / S[S_RHO]) * (S[S_ALPHA] / S[S_OMEGA]);
    if (v[1] == 0.0 || !isfinite(beta)) { S[S_FLAG] = 1.0; beta = 0.0; }
    S[S_BETA] = beta;
}

// x += alpha ph + omega sh; r = s - omega t; (r, r) and (r0, r) (the grid-stride layout
// of k_dot_partial, kRedBlocks blocks); the last block ends the iteration
__global__ void __launch_bounds__(kRedThreads) k_bicg_x_end(int64_t n, double* S, const double* __restrict__ ph,
                                                             const double* __restrict__ shv, const double* __restrict__ sv,
                                                             const double* __restrict__ t, const double* __restrict__ r0,
                                                             double* __restrict__ x, double* __restrict__ r, double* __restrict__ partials,
                                                             unsigned* counter, double nr0, double rtol) {
    if (S[S_DONE] != 0.0) return;
    const double alpha = S[S_ALPHA], omega = S[S_OMEGA];
    double d[2] = {0.0, 0.0};
    for (int64_t i = (int64_t)blockIdx.x * kRedThreads + threadIdx.x; i < n; i += (int64_t)gridDim.x * kRedThreads) {
        x[i] += alpha * ph[i] + omega * shv[i];
        const double ri = sv[i] - omega * t[i];
        r[i] = ri;
        d[0] += ri * ri;
        d[1] += r0[i] * ri;
    }
    block_partials<2>(d, partials);
    double tot[2];
    if (last_block_sum<2>(partials, counter, tot) && threadIdx.x == 0) bicg_end_update(S, tot, nr0, rtol);
}

template <typename A, typename B>
__global__ void k_convert(int64_t n, const A* __restrict__ a, B* __restrict__ b) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) b[i] = (B)a[i];
}
// b = scale * a (the Newton right-hand side normalised to unit norm before the solve)
template <typename A, typename B>
__global__ void k_convert_scaled(int64_t n, const A* __restrict__ a, B* __restrict__ b, double scale) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) b[i] = (B)(scale * (double)a[i]);
}
template <typename VT>
__global__ void k_fill(int64_t n, VT* a, VT v) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) a[i] = v;
}
// ut = u - lambda du
template <typename VT>
__global__ void k_newton_update(int64_t n, const double* __restrict__ u, const VT* __restrict__ du, double lambda, double* __restrict__ ut) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) ut[i] = u[i] - lambda * (double)du[i];
}
__global__ void k_set_dirichlet(int64_t n, const int32_t* __restrict__ rows, const double* __restrict__ vals, double* u) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) u[rows[i]] = vals[i];
}

// GMRES helpers ---------------------------------------------------------------
// h[k] = (V_k, w) for k < m (one pass over w, partials per block)
template <typename VT>
__global__ void __launch_bounds__(kRedThreads) k_multidot_partial(int64_t n, int m, const VT* __restrict__ V, const VT* __restrict__ w,
                                                                 double* __restrict__ partials) {
    __shared__ double sh[kRedThreads];
    for (int k = 0; k < m; ++k) {
        double acc = 0.0;
        const VT* vk = V + (int64_t)k * n;
        for (int64_t i = (int64_t)blockIdx.x * kRedThreads + threadIdx.x; i < n; i += (int64_t)gridDim.x * kRedThreads)
            acc += (double)vk[i] * (double)w[i];
        sh[threadIdx.x] = acc;
        __syncthreads();
        for (int s = kRedThreads / 2; s > 0; s >>= 1) {
            if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
            __syncthreads();
        }
        if (threadIdx.x == 0) partials[k * gridDim.x + blockIdx.x] = sh[0];
        __syncthreads();
    }
}
__global__ void k_multidot_final(const double* __restrict__ partials, int nb, int m, double* out) {
    __shared__ double sh[kRedThreads];
    for (int k = 0; k < m; ++k) {
        double acc = 0.0;
        for (int i = threadIdx.x; i < nb; i += kRedThreads) acc += partials[k * nb + i];
        sh[threadIdx.x] = acc;
        __syncthreads();
        for (int s = kRedThreads / 2; s > 0; s >>= 1) {
            if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
            __syncthreads();
        }
        if (threadIdx.x == 0) out[k] = sh[0];
        __syncthreads();
    }
}
// w -= sum_k h[k] V_k
template <typename VT>
__global__ void k_multi_axpy(int64_t n, int m, const double* __restrict__ h, const VT* __restrict__ V, VT* __restrict__ w) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double a = (double)w[i];
    for (int k = 0; k < m; ++k) a -= h[k] * (double)V[(int64_t)k * n + i];
    w[i] = (VT)a;
}
// v = w / beta
template <typename VT>
__global__ void k_scale(int64_t n, const VT* __restrict__ w, double inv, VT* __restrict__ v) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) v[i] = (VT)((double)w[i] * inv);
}
// x += sum_k y[k] Z_k   (Z = preconditioned basis)
template <typename VT>
__global__ void k_multi_axpy_add(int64_t n, int m, const double* __restrict__ y, const VT* __restrict__ Z, VT* __restrict__ x) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double a = (double)x[i];
    for (int k = 0; k < m; ++k) a += y[k] * (double)Z[(int64_t)k * n + i];
    x[i] = (VT)a;
}

static inline int grid_for(int64_t n, int t = 256) { return (int)((n + t - 1) / t); }

// Lanes per block row: a row of the FV1 patterns holds 7 (triangles) to 27
// (hexahedra) blocks. With 4 lanes per 3x3-block row each lane takes about two
// blocks and the butterfly over the lanes has two levels instead of three; on a
// 1025^2-row, 7-blocks-per-row FP32 matrix the double-float SpMV went from 112.8
// to 88.2 us (8 -> 4 lanes; 2 lanes: 87.9 us, 1 lane: 105.0 us, loads uncoalesced).
template <int b> constexpr int spmv_lanes() { return b == 4 ? 8 : 4; }

template <typename MT, typename VT>
static cudaError_t spmv(const Disc& D, const MT* vals, const VT* x, VT* y, cudaStream_t s, const double* gate = nullptr) {
    const int64_t nR = D.nNodes;
    const int b = D.dim + 1;
    if (b == 4) {
        constexpr int G = spmv_lanes<4>();
        k_bsr_mv<MT, VT, 4, G><<<grid_for(nR * G), 256, 0, s>>>(nR, D.d_rowPtr, D.d_colIdx, vals, x, y, gate);
    } else {
        constexpr int G = spmv_lanes<3>();
        k_bsr_mv<MT, VT, 3, G><<<grid_for(nR * G), 256, 0, s>>>(nR, D.d_rowPtr, D.d_colIdx, vals, x, y, gate);
    }
    return cudaGetLastError();
}

template <typename MT, typename VT>
static void prec_apply(const Disc& D, const MT* Dinv, const VT* in, VT* out, cudaStream_t s) {
    if (D.dim == 3) k_prec<MT, VT, 4><<<grid_for(D.nNodes), 256, 0, s>>>(D.nNodes, Dinv, in, out);
    else k_prec<MT, VT, 3><<<grid_for(D.nNodes), 256, 0, s>>>(D.nNodes, Dinv, in, out);
}

template <typename VT, int K>
static void dots(int64_t n, const VT* const (&a)[K], const VT* const (&c)[K], double* partials, cudaStream_t s,
                 const double* gate = nullptr) {
    DotArgs<VT, K> A;
    for (int k = 0; k < K; ++k) { A.a[k] = a[k]; A.c[k] = c[k]; }
    k_dot_partial<VT, K><<<kRedBlocks, kRedThreads, 0, s>>>(n, A, partials, gate);
}

// ||x||_2^2 of an FP64 vector into out (device)
static void norm2sq(int64_t n, const double* x, double* partials, double* out, cudaStream_t s) {
    const double* a[1] = {x};
    dots<double, 1>(n, a, a, partials, s);
    k_dot_final<1><<<1, kRedThreads, 0, s>>>(partials, kRedBlocks, out);
}

}  // namespace nsfv1

// ============================================================================
using namespace nsfv1;

namespace nsfv1 {

void Disc::free_workspace() {
    auto f = [](auto*& p) { if (p) cudaFree((void*)p); p = nullptr; };
    f(ws.D); f(ws.Dt); f(ws.Ut); f(ws.du); f(ws.J); f(ws.Dinv); f(ws.vec); f(ws.red); f(ws.scal);
    if (ws.hscal) cudaFreeHost(ws.hscal);
    ws = Workspace();
}

bool Disc::ensure_workspace(int prec, int gmresM) {
    const int b = dim + 1;
    const int64_t n = nNodes * b;
    const int nvec = 10 + 2 * (gmresM + 1);   // BiCGStab: 10 work vectors, then the linear solve's rhs and solution
    if (ws.prec == prec && ws.n == n && ws.nvec >= nvec) return true;
    free_workspace();
    const size_t vt = prec == NSFV1_F64 ? sizeof(double) : sizeof(float);
    auto al = [&](auto*& p, size_t bytes) { return cuda_ok(cudaMalloc((void**)&p, bytes), "workspace alloc"); };
    if (!al(ws.D, n * 8) || !al(ws.Dt, n * 8) || !al(ws.Ut, n * 8) || !al(ws.du, n * 8) ||
        !al(ws.J, colIdx.size() * b * b * vt) || !al(ws.Dinv, (size_t)nNodes * b * b * vt) ||
        !al(ws.vec, (size_t)nvec * n * sizeof(double)) || !al(ws.red, sizeof(double) * kRedBlocks * 80) ||
        !al(ws.scal, sizeof(double) * 256))
        return false;
    if (!cuda_ok(cudaMallocHost((void**)&ws.hscal, sizeof(double) * 256), "pinned alloc")) return false;
    ws.prec = prec; ws.n = n; ws.nvec = nvec; ws.gmresM = gmresM;
    return true;
}

}  // namespace nsfv1

namespace {

// reads k scalars from ws.scal (device) into ws.hscal (pinned) and waits
static bool read_scal(Disc& D, int first, int k, cudaStream_t s) {
    if (!D.cuda_ok(cudaMemcpyAsync(D.ws.hscal + first, D.ws.scal + first, sizeof(double) * k, cudaMemcpyDeviceToHost, s), "read scalars")) return false;
    return D.cuda_ok(cudaStreamSynchronize(s), "sync");
}

// BiCGStab on J x = rhs (right point-block-Jacobi preconditioning), x = 0 start.
// Returns iterations, or -1 on breakdown / failure (D.status set on CUDA errors).
static constexpr int kMaxBicgRestarts = 20;
// Iterations queued between two host reads of the solver state: the stop tests
// run on the device (k_bicg_x_end) and every kernel of a later iteration returns at
// once, so the iterates are those of a test after every iteration.
static constexpr int kBicgBatch = 16;

// the last-block counters of the BiCGStab reductions (unsigned, in the scalar buffer)
static unsigned* bicg_counters(Workspace& W) { return reinterpret_cast<unsigned*>(W.scal + 200); }

template <typename MT, int b>
static void bicg_iteration(Disc& D, const MT* J, const MT* Dinv, double* const (&V)[10], double* x, double nr0, double rtol, cudaStream_t s) {
    Workspace& W = D.ws;
    double *r = V[0], *r0 = V[1], *p = V[2], *v = V[3], *sv = V[4], *t = V[5], *ph = V[6], *shv = V[7];
    float2* phs = reinterpret_cast<float2*>(V[8]);   // split copies of ph and shv (FP32 matrices)
    float2* shs = reinterpret_cast<float2*>(V[9]);
    double* S = W.scal;
    const double* done = S + S_DONE;
    const int64_t nR = D.nNodes, n = W.n;
    const int gn = grid_for(nR);
    auto mv = [&](const double* xd, const float2* xsplit, double* y) {
        if constexpr (std::is_same<MT, float>::value) {
            constexpr int G = spmv_lanes<b>();
            k_bsr_mv_split<b, G><<<grid_for(nR * G), 256, 0, s>>>(nR, D.d_rowPtr, D.d_colIdx, J, xsplit, y, done);
        } else {
            spmv<MT, double>(D, J, xd, y, s, done);
        }
    };
    unsigned* counters = bicg_counters(W);
    k_bicg_p_prec<MT, b><<<gn, 256, 0, s>>>(nR, S, r, v, p, Dinv, ph, phs);
    mv(ph, phs, v);
    k_bicg_dot_alpha<<<kRedBlocks, kRedThreads, 0, s>>>(n, r0, v, W.red, counters + 0, S);
    k_bicg_s_prec<MT, b><<<gn, 256, 0, s>>>(nR, S, r, v, sv, Dinv, shv, shs);
    mv(shv, shs, t);
    k_bicg_dot_omega<<<kRedBlocks, kRedThreads, 0, s>>>(n, t, sv, W.red, counters + 1, S);
    k_bicg_x_end<<<kRedBlocks, kRedThreads, 0, s>>>(n, S, ph, shv, sv, t, r0, x, r, W.red, counters + 2, nr0, rtol);
}

// The Krylov vectors are FP64 whatever the precision MT of the stored Jacobian:
// an FP32 matrix then only perturbs the operator (relative 6e-8 per entry),
// while FP32 vectors would let the recursive residual drift from the true one.
template <typename MT>
static int bicgstab(Disc& D, const MT* J, const MT* Dinv, const double* rhs, double* x, double rtol, int maxit, double* relres, cudaStream_t s,
                    int* restartsOut = nullptr) {
    using VT = double;
    Workspace& W = D.ws;
    const int64_t n = W.n;
    VT* Vb = (VT*)W.vec;
    double* const V[10] = {Vb, Vb + n, Vb + 2 * n, Vb + 3 * n, Vb + 4 * n, Vb + 5 * n, Vb + 6 * n, Vb + 7 * n, Vb + 8 * n, Vb + 9 * n};
    VT *r = V[0], *r0 = V[1], *p = V[2], *v = V[3];
    double* S = W.scal;
    const int g = grid_for(n);
    k_fill<VT><<<g, 256, 0, s>>>(n, x, VT(0));
    cudaMemcpyAsync(r, rhs, n * sizeof(VT), cudaMemcpyDeviceToDevice, s);
    cudaMemcpyAsync(r0, rhs, n * sizeof(VT), cudaMemcpyDeviceToDevice, s);
    k_fill<VT><<<g, 256, 0, s>>>(n, p, VT(0));
    k_fill<VT><<<g, 256, 0, s>>>(n, v, VT(0));
    double init[S_NSCAL] = {0};
    init[S_RHO] = 1.0; init[S_ALPHA] = 1.0; init[S_OMEGA] = 1.0;
    std::memcpy(W.hscal, init, sizeof(init));
    cudaMemcpyAsync(S, W.hscal, sizeof(init), cudaMemcpyHostToDevice, s);
    cudaMemsetAsync(bicg_counters(W), 0, 4 * sizeof(unsigned), s);
    {
        const VT* a[1] = {r};
        dots<VT, 1>(n, a, a, W.red, s);
        k_dot_final<1><<<1, kRedThreads, 0, s>>>(W.red, kRedBlocks, S + S_NR02);
    }
    if (!read_scal(D, S_NR02, 1, s)) return -1;
    const double nr0 = std::sqrt(W.hscal[S_NR02]);
    *relres = 1.0;
    if (nr0 == 0.0) return 0;
    const int b = D.dim + 1;
    int restarts = 0, it = 0;
    struct Report {
        int& n; int* out;
        ~Report() { if (out) *out = n; }
    } report{restarts, restartsOut};
    bool needBeta = true;   // rho1 and beta of the first iteration (later ones come from k_bicg_x_end)
    while (it < maxit) {
        const int K = std::min(kBicgBatch, maxit - it);
        for (int j = 0; j < K; ++j) {
            if (j == 0 && needBeta) {
                const VT* a[1] = {r0}; const VT* c[1] = {r};
                dots<VT, 1>(n, a, c, W.red, s);
                k_bicg_beta<<<1, kRedThreads, 0, s>>>(W.red, kRedBlocks, S);
            }
            if (b == 4) bicg_iteration<MT, 4>(D, J, Dinv, V, x, nr0, rtol, s);
            else bicg_iteration<MT, 3>(D, J, Dinv, V, x, nr0, rtol, s);
        }
        needBeta = false;
        if (!D.cuda_ok(cudaGetLastError(), "bicgstab launch")) return -1;
        if (!read_scal(D, 0, S_NSCAL, s)) return -1;
        it = (int)W.hscal[S_ITER];
        const double nr = std::sqrt(W.hscal[S_NR2]);
        *relres = nr / nr0;
        const int done = (int)W.hscal[S_DONE];
        if (done == DONE_NONFINITE) return -1;   // hard failure: x is not usable
        if (done == DONE_CONVERGED) return it;
        if (done == DONE_BREAKDOWN) {
            // breakdown (rho1 = 0, (r0, v) = 0, a non-finite coefficient, omega = 0): restart
            // with the current residual as the shadow vector; after too many restarts stop
            // with the last finite iterate and let the Newton line search judge it
            if (++restarts > kMaxBicgRestarts) return it;
            cudaMemcpyAsync(r0, r, n * sizeof(VT), cudaMemcpyDeviceToDevice, s);
            k_fill<VT><<<g, 256, 0, s>>>(n, p, VT(0));
            k_fill<VT><<<g, 256, 0, s>>>(n, v, VT(0));
            double re[S_NSCAL];
            std::memcpy(re, W.hscal, sizeof(re));
            re[S_RHO] = 1.0; re[S_ALPHA] = 1.0; re[S_OMEGA] = 1.0; re[S_FLAG] = 0.0; re[S_NR02] = re[S_NR2]; re[S_DONE] = 0.0;
            std::memcpy(W.hscal, re, sizeof(re));
            cudaMemcpyAsync(S, W.hscal, sizeof(re), cudaMemcpyHostToDevice, s);
            needBeta = true;
        }
    }
    return maxit;
}

// restarted GMRES(m), right preconditioned, classical Gram-Schmidt with one
// re-orthogonalisation pass; Hessenberg least squares (Givens) on the host.
template <typename MT>
static int gmres(Disc& D, const MT* J, const MT* Dinv, const double* rhs, double* x, double rtol, int maxit, int m, double* relres, cudaStream_t s) {
    using VT = double;
    Workspace& W = D.ws;
    const int64_t n = W.n;
    VT* base = (VT*)W.vec;
    VT* w = base;                 // work vector
    VT* Vb = base + 1 * n;        // basis V_0..V_m
    VT* Zb = base + (1 + m + 1) * n;   // preconditioned basis Z_0..Z_{m-1}
    double* hdev = W.scal + 32;   // up to 64 + 1 coefficients
    const int g = grid_for(n);
    k_fill<VT><<<g, 256, 0, s>>>(n, x, VT(0));
    std::vector<double> H((m + 1) * m), cs(m), sn(m), gam(m + 1), y(m);
    double beta0 = -1.0;
    int it = 0;
    *relres = 1.0;
    while (it < maxit) {
        // V_0 = rhs - J x
        spmv<MT, VT>(D, J, x, w, s);
        cudaMemcpyAsync(Vb, rhs, n * sizeof(VT), cudaMemcpyDeviceToDevice, s);
        W.hscal[40] = 1.0;
        cudaMemcpyAsync(hdev, W.hscal + 40, sizeof(double), cudaMemcpyHostToDevice, s);
        k_multi_axpy<VT><<<g, 256, 0, s>>>(n, 1, hdev, w, Vb);
        {
            const VT* a[1] = {Vb};
            dots<VT, 1>(n, a, a, W.red, s);
            k_dot_final<1><<<1, kRedThreads, 0, s>>>(W.red, kRedBlocks, W.scal + S_NR2);
        }
        if (!read_scal(D, S_NR2, 1, s)) return -1;
        const double beta = std::sqrt(W.hscal[S_NR2]);
        if (beta0 < 0) beta0 = beta;
        if (beta0 == 0.0) return 0;
        *relres = beta / beta0;
        if (*relres < rtol) return it;
        k_scale<VT><<<g, 256, 0, s>>>(n, Vb, 1.0 / beta, Vb);
        std::fill(gam.begin(), gam.end(), 0.0);
        gam[0] = beta;
        int j = 0;
        for (; j < m && it < maxit; ++j) {
            ++it;
            VT* Zj = Zb + (int64_t)j * n;
            prec_apply<MT, VT>(D, Dinv, Vb + (int64_t)j * n, Zj, s);
            spmv<MT, VT>(D, J, Zj, w, s);
            double hcol[66] = {0};
            for (int pass = 0; pass < 2; ++pass) {
                k_multidot_partial<VT><<<kRedBlocks, kRedThreads, 0, s>>>(n, j + 1, Vb, w, W.red);
                k_multidot_final<<<1, kRedThreads, 0, s>>>(W.red, kRedBlocks, j + 1, hdev);
                k_multi_axpy<VT><<<g, 256, 0, s>>>(n, j + 1, hdev, Vb, w);
                if (!D.cuda_ok(cudaMemcpyAsync(W.hscal + 64, hdev, sizeof(double) * (j + 1), cudaMemcpyDeviceToHost, s), "h")) return -1;
                if (!D.cuda_ok(cudaStreamSynchronize(s), "sync")) return -1;
                for (int k = 0; k <= j; ++k) hcol[k] += W.hscal[64 + k];
            }
            {
                const VT* a[1] = {w};
                dots<VT, 1>(n, a, a, W.red, s);
                k_dot_final<1><<<1, kRedThreads, 0, s>>>(W.red, kRedBlocks, W.scal + S_NR2);
            }
            if (!read_scal(D, S_NR2, 1, s)) return -1;
            const double hn = std::sqrt(W.hscal[S_NR2]);
            hcol[j + 1] = hn;
            if (hn > 0.0) k_scale<VT><<<g, 256, 0, s>>>(n, w, 1.0 / hn, Vb + (int64_t)(j + 1) * n);
            // apply previous Givens rotations, then a new one
            for (int k = 0; k < j; ++k) {
                const double a = hcol[k], b2 = hcol[k + 1];
                hcol[k] = cs[k] * a + sn[k] * b2;
                hcol[k + 1] = -sn[k] * a + cs[k] * b2;
            }
            const double a = hcol[j], b2 = hcol[j + 1];
            const double rr = std::sqrt(a * a + b2 * b2);
            cs[j] = rr > 0 ? a / rr : 1.0; sn[j] = rr > 0 ? b2 / rr : 0.0;
            hcol[j] = rr; hcol[j + 1] = 0.0;
            gam[j + 1] = -sn[j] * gam[j];
            gam[j] = cs[j] * gam[j];
            for (int k = 0; k <= j; ++k) H[k * m + j] = hcol[k];
            *relres = std::fabs(gam[j + 1]) / beta0;
            if (!std::isfinite(*relres)) return -1;
            if (*relres < rtol || hn == 0.0) { ++j; break; }
        }
        // y = H^-1 gam ; x += Z y
        for (int k = j - 1; k >= 0; --k) {
            double acc = gam[k];
            for (int q = k + 1; q < j; ++q) acc -= H[k * m + q] * y[q];
            y[k] = (H[k * m + k] != 0.0) ? acc / H[k * m + k] : 0.0;
        }
        std::memcpy(W.hscal + 64, y.data(), sizeof(double) * j);
        cudaMemcpyAsync(hdev, W.hscal + 64, sizeof(double) * j, cudaMemcpyHostToDevice, s);
        k_multi_axpy_add<VT><<<g, 256, 0, s>>>(n, j, hdev, Zb, x);
        if (!D.cuda_ok(cudaGetLastError(), "gmres launch")) return -1;
        if (*relres < rtol) return it;
    }
    return it;
}

template <typename MT>
static int newton_impl(Disc& D, double* u, const double* u_old, double dt, const nsfv1_newton_params& p, nsfv1_newton_result& res,
                       cudaStream_t s) {
    using VT = double;   // Krylov vectors
    const int prec = std::is_same<MT, double>::value ? NSFV1_F64 : NSFV1_F32;
    const int m = std::min(std::max(p.gmres_restart, 1), 64);
    if (!D.ensure_workspace(prec, p.linear_solver == NSFV1_GMRES ? m : 0)) return D.status;
    Workspace& W = D.ws;
    const int64_t n = W.n;
    const int g = grid_for(n);
    const int b = D.dim + 1;
    MT* J = (MT*)W.J;
    MT* Dinv = (MT*)W.Dinv;
    VT* Vv = (VT*)W.vec;
    VT* rhsV = Vv + (int64_t)(W.nvec - 2) * n;   // rhs of the linear solve (VT)
    VT* xsol = Vv + (int64_t)(W.nvec - 1) * n;   // its solution du (VT)

    if (D.nDir > 0) k_set_dirichlet<<<grid_for(D.nDir), 256, 0, s>>>(D.nDir, D.d_dirRow, D.d_dirVal, u);
    if (!D.assemble_defect(u, u_old, dt, W.D, s)) return D.status;
    norm2sq(n, W.D, W.red, W.scal + 100, s);
    if (!read_scal(D, 100, 1, s)) return D.status;
    double nd = std::sqrt(W.hscal[100]);
    const double nd0 = nd;
    res.initial_defect = nd0; res.final_defect = nd; res.iterations = 0; res.linear_iterations = 0;
    if (!std::isfinite(nd0)) { res.status = NSFV1_ERR_NONFINITE; return res.status; }
    int status = NSFV1_ERR_NOT_CONVERGED;
    if (nd0 == 0.0) status = NSFV1_OK;
    int it = 0;
    while (status == NSFV1_ERR_NOT_CONVERGED && it < p.max_iter) {
        if (nd <= p.rtol * nd0 || nd <= p.atol) { status = NSFV1_OK; break; }
        ++it;
        if (!D.assemble_jacobian(u, u_old, dt, J, prec, s, false)) return D.status;
        cudaMemsetAsync(D.d_err, 0, sizeof(int), s);
        if (b == 4) k_block_inv<MT, MT, 4><<<grid_for(D.nNodes, 128), 128, 0, s>>>(D.nNodes, D.d_diagPos, J, Dinv, D.d_err);
        else k_block_inv<MT, MT, 3><<<grid_for(D.nNodes, 128), 128, 0, s>>>(D.nNodes, D.d_diagPos, J, Dinv, D.d_err);
        int herr = 0;
        cudaMemcpyAsync(&herr, D.d_err, sizeof(int), cudaMemcpyDeviceToHost, s);
        if (!D.cuda_ok(cudaStreamSynchronize(s), "jacobian")) return D.status;
        if (herr & 1) { D.fail(NSFV1_ERR_GEOMETRY, "upwind: cannot find cut side"); cudaMemsetAsync(D.d_err, 0, sizeof(int), s); return D.status; }
        if (herr & 2) { status = NSFV1_ERR_BREAKDOWN; D.fail(NSFV1_ERR_BREAKDOWN, "singular diagonal block"); cudaMemsetAsync(D.d_err, 0, sizeof(int), s); break; }
        // unit-norm right-hand side: the Krylov vectors stay O(1) in FP32 whatever the defect's size
        k_convert_scaled<double, VT><<<g, 256, 0, s>>>(n, W.D, rhsV, 1.0 / nd);
        double rr = 0;
        int li;
        if (p.linear_solver == NSFV1_GMRES) li = gmres<MT>(D, J, Dinv, rhsV, xsol, p.lin_rtol, p.lin_max_iter, m, &rr, s);
        else li = bicgstab<MT>(D, J, Dinv, rhsV, xsol, p.lin_rtol, p.lin_max_iter, &rr, s);
        if (D.status == NSFV1_ERR_CUDA) return D.status;
        if (li < 0) { status = NSFV1_ERR_BREAKDOWN; D.fail(NSFV1_ERR_BREAKDOWN, "linear solver breakdown"); break; }
        res.linear_iterations += li;
        double lambda = 1.0, ndt = 0.0;
        for (int k = 0; k <= p.line_search_steps; ++k) {
            k_newton_update<VT><<<g, 256, 0, s>>>(n, u, xsol, lambda * nd, W.Ut);
            if (!D.assemble_defect(W.Ut, u_old, dt, W.Dt, s)) return D.status;
            norm2sq(n, W.Dt, W.red, W.scal + 100, s);
            if (!read_scal(D, 100, 1, s)) return D.status;
            ndt = std::sqrt(W.hscal[100]);
            if (ndt <= (1.0 - 1e-4 * lambda) * nd || k == p.line_search_steps) break;
            lambda *= 0.5;
        }
        cudaMemcpyAsync(u, W.Ut, n * sizeof(double), cudaMemcpyDeviceToDevice, s);
        std::swap(W.D, W.Dt);
        nd = ndt;
        if (!std::isfinite(nd)) { status = NSFV1_ERR_NONFINITE; break; }
    }
    if (status == NSFV1_ERR_NOT_CONVERGED && (nd <= p.rtol * nd0 || nd <= p.atol)) status = NSFV1_OK;
    if (!D.cuda_ok(cudaStreamSynchronize(s), "newton")) return D.status;
    res.iterations = it; res.final_defect = nd; res.status = status;
    if (status != NSFV1_OK && status != NSFV1_ERR_BREAKDOWN) D.fail(status, status == NSFV1_ERR_NONFINITE ? "non-finite defect" : "Newton did not converge");
    return status;
}

// J x = rhs on the handle's pattern with the Newton loop's linear solver (x = 0 start)
template <typename MT>
static int linear_solve_impl(Disc& D, const MT* J, const double* rhs, double* x, const nsfv1_newton_params& p, int* iterations,
                             double* relres, int* restarts, cudaStream_t s) {
    const int prec = std::is_same<MT, double>::value ? NSFV1_F64 : NSFV1_F32;
    const int m = std::min(std::max(p.gmres_restart, 1), 64);
    if (!D.ensure_workspace(prec, p.linear_solver == NSFV1_GMRES ? m : 0)) return D.status;
    Workspace& W = D.ws;
    MT* Dinv = (MT*)W.Dinv;
    const int b = D.dim + 1;
    cudaMemsetAsync(D.d_err, 0, sizeof(int), s);
    if (b == 4) k_block_inv<MT, MT, 4><<<grid_for(D.nNodes, 128), 128, 0, s>>>(D.nNodes, D.d_diagPos, J, Dinv, D.d_err);
    else k_block_inv<MT, MT, 3><<<grid_for(D.nNodes, 128), 128, 0, s>>>(D.nNodes, D.d_diagPos, J, Dinv, D.d_err);
    int herr = 0;
    cudaMemcpyAsync(&herr, D.d_err, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (!D.cuda_ok(cudaStreamSynchronize(s), "linear solve")) return D.status;
    if (herr & 2) {
        cudaMemsetAsync(D.d_err, 0, sizeof(int), s);
        D.fail(NSFV1_ERR_BREAKDOWN, "singular diagonal block");
        return D.status;
    }
    double rr = 0.0;
    int rs = 0;
    const int li = p.linear_solver == NSFV1_GMRES ? gmres<MT>(D, J, Dinv, rhs, x, p.lin_rtol, p.lin_max_iter, m, &rr, s)
                                                  : bicgstab<MT>(D, J, Dinv, rhs, x, p.lin_rtol, p.lin_max_iter, &rr, s, &rs);
    if (D.status == NSFV1_ERR_CUDA) return D.status;
    if (!D.cuda_ok(cudaStreamSynchronize(s), "linear solve")) return D.status;
    if (iterations) *iterations = li < 0 ? 0 : li;
    if (relres) *relres = rr;
    if (restarts) *restarts = rs;
    if (li < 0) {
        D.fail(NSFV1_ERR_BREAKDOWN, "linear solver: non-finite residual");
        return D.status;
    }
    if (!(rr < p.lin_rtol)) {
        D.fail(NSFV1_ERR_NOT_CONVERGED, "linear solver did not reach the tolerance");
        return D.status;
    }
    return NSFV1_OK;
}

}  // namespace

namespace nsfv1 {
bool Disc::set_dirichlet_values(double* u, cudaStream_t s) {
    if (nDir > 0) k_set_dirichlet<<<grid_for(nDir), 256, 0, s>>>(nDir, d_dirRow, d_dirVal, u);
    return cuda_ok(cudaGetLastError(), "dirichlet values");
}

// point-block Jacobi on a caller's Jacobian: Dinv (FP64 scratch) = inverse
// diagonal blocks, z = Dinv r.
bool block_jacobi_run(Disc& D, const void* vals, int prec, const double* r, double* z, double* Dinv, cudaStream_t s) {
    const int b = D.dim + 1;
    const int64_t nR = D.nNodes;
    if (!D.cuda_ok(cudaMemsetAsync(D.d_err, 0, sizeof(int), s), "block_jacobi")) return false;
    const int g = grid_for(nR, 128);
    if (prec == NSFV1_F64) {
        if (b == 4) k_block_inv<double, double, 4><<<g, 128, 0, s>>>(nR, D.d_diagPos, (const double*)vals, Dinv, D.d_err);
        else k_block_inv<double, double, 3><<<g, 128, 0, s>>>(nR, D.d_diagPos, (const double*)vals, Dinv, D.d_err);
    } else {
        if (b == 4) k_block_inv<float, double, 4><<<g, 128, 0, s>>>(nR, D.d_diagPos, (const float*)vals, Dinv, D.d_err);
        else k_block_inv<float, double, 3><<<g, 128, 0, s>>>(nR, D.d_diagPos, (const float*)vals, Dinv, D.d_err);
    }
    if (b == 4) k_prec<double, double, 4><<<grid_for(nR), 256, 0, s>>>(nR, Dinv, r, z);
    else k_prec<double, double, 3><<<grid_for(nR), 256, 0, s>>>(nR, Dinv, r, z);
    if (!D.cuda_ok(cudaGetLastError(), "block_jacobi launch")) return false;
    int err = 0;
    if (!D.cuda_ok(cudaMemcpyAsync(&err, D.d_err, sizeof(int), cudaMemcpyDeviceToHost, s), "block_jacobi")) return false;
    if (!D.cuda_ok(cudaStreamSynchronize(s), "block_jacobi sync")) return false;
    if (err & 2) return D.fail(NSFV1_ERR_BREAKDOWN, "block_jacobi: singular diagonal block");
    return true;
}
}  // namespace nsfv1

extern "C" {

int nsfv1_bsr_mv(nsfv1_disc* h, const void* vals, int prec, const double* x, double* y, void* stream) {
    Disc* D = reinterpret_cast<Disc*>(h);
    if (!D) return NSFV1_ERR_ARGUMENT;
    D->status = NSFV1_OK;
    if (!D->hasMesh) { D->fail(NSFV1_ERR_STATE, "bsr_mv: no mesh"); return D->status; }
    cudaStream_t s = (cudaStream_t)stream;
    if (prec == NSFV1_F64) {
        if (!D->cuda_ok(spmv<double, double>(*D, (const double*)vals, x, y, s), "bsr_mv")) return D->status;
    } else if (prec == NSFV1_F32) {
        if (!D->cuda_ok(spmv<float, double>(*D, (const float*)vals, x, y, s), "bsr_mv")) return D->status;
    } else {
        D->fail(NSFV1_ERR_ARGUMENT, "bsr_mv: bad precision");
        return D->status;
    }
    return D->cuda_ok(cudaGetLastError(), "bsr_mv") ? NSFV1_OK : D->status;
}

int nsfv1_split_vector(int64_t n, const double* x, float* xs, void* stream) {
    if (n < 0 || (n > 0 && (!x || !xs))) return NSFV1_ERR_ARGUMENT;
    if (n == 0) return NSFV1_OK;
    k_split_vector<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(n, x, reinterpret_cast<float2*>(xs));
    return cudaGetLastError() == cudaSuccess ? NSFV1_OK : NSFV1_ERR_CUDA;
}

int nsfv1_bsr_mv_split(nsfv1_disc* h, const float* vals, const float* xs, double* y, void* stream) {
    Disc* D = reinterpret_cast<Disc*>(h);
    if (!D) return NSFV1_ERR_ARGUMENT;
    D->status = NSFV1_OK;
    if (!D->hasMesh) { D->fail(NSFV1_ERR_STATE, "bsr_mv_split: no mesh"); return D->status; }
    if (!vals || !xs || !y) { D->fail(NSFV1_ERR_ARGUMENT, "bsr_mv_split: null pointer"); return D->status; }
    if (reinterpret_cast<uintptr_t>(xs) & 7) { D->fail(NSFV1_ERR_ARGUMENT, "bsr_mv_split: xs must be 8-byte aligned"); return D->status; }
    const int64_t nR = D->nNodes;
    cudaStream_t s = (cudaStream_t)stream;
    const float2* x2 = reinterpret_cast<const float2*>(xs);
    if (D->dim == 3) {
        constexpr int G = spmv_lanes<4>();
        k_bsr_mv_split<4, G><<<grid_for(nR * G), 256, 0, s>>>(nR, D->d_rowPtr, D->d_colIdx, vals, x2, y, nullptr);
    } else {
        constexpr int G = spmv_lanes<3>();
        k_bsr_mv_split<3, G><<<grid_for(nR * G), 256, 0, s>>>(nR, D->d_rowPtr, D->d_colIdx, vals, x2, y, nullptr);
    }
    return D->cuda_ok(cudaGetLastError(), "bsr_mv_split") ? NSFV1_OK : D->status;
}

int nsfv1_linear_solve(nsfv1_disc* h, const void* vals, const double* rhs, double* x, const nsfv1_newton_params* p, int* iterations,
                       double* relres, int* restarts, void* stream) {
    Disc* D = reinterpret_cast<Disc*>(h);
    if (!D) return NSFV1_ERR_ARGUMENT;
    D->status = NSFV1_OK;
    if (!D->hasMesh) { D->fail(NSFV1_ERR_STATE, "linear_solve: no mesh"); return D->status; }
    if (!vals || !rhs || !x || !p) { D->fail(NSFV1_ERR_ARGUMENT, "linear_solve: null pointer"); return D->status; }
    if (p->lin_max_iter < 1 || !(p->lin_rtol > 0.0)) { D->fail(NSFV1_ERR_ARGUMENT, "linear_solve: lin_max_iter >= 1 and lin_rtol > 0"); return D->status; }
    cudaStream_t s = (cudaStream_t)stream;
    if (p->jacobian_prec == NSFV1_F64) return linear_solve_impl<double>(*D, (const double*)vals, rhs, x, *p, iterations, relres, restarts, s);
    if (p->jacobian_prec == NSFV1_F32) return linear_solve_impl<float>(*D, (const float*)vals, rhs, x, *p, iterations, relres, restarts, s);
    D->fail(NSFV1_ERR_ARGUMENT, "linear_solve: jacobian_prec must be NSFV1_F64 or NSFV1_F32");
    return D->status;
}

int nsfv1_block_jacobi(nsfv1_disc* h, const void* vals, int prec, const double* r, double* z, void* stream) {
    Disc* D = reinterpret_cast<Disc*>(h);
    if (!D) return NSFV1_ERR_ARGUMENT;
    D->status = NSFV1_OK;
    if (!D->hasMesh) { D->fail(NSFV1_ERR_STATE, "block_jacobi: no mesh"); return D->status; }
    if (!vals || !r || !z || (prec != NSFV1_F64 && prec != NSFV1_F32)) { D->fail(NSFV1_ERR_ARGUMENT, "block_jacobi: bad arguments"); return D->status; }
    const int b = D->dim + 1;
    if (!D->d_bjDinv && !D->cuda_ok(cudaMalloc((void**)&D->d_bjDinv, sizeof(double) * D->nNodes * b * b), "block_jacobi scratch"))
        return D->status;
    return block_jacobi_run(*D, vals, prec, r, z, D->d_bjDinv, (cudaStream_t)stream) ? NSFV1_OK : D->status;
}

int nsfv1_newton_solve(nsfv1_disc* h, double* u, const double* u_old, double dt, const nsfv1_newton_params* p,
                       nsfv1_newton_result* r, void* stream) {
    Disc* D = reinterpret_cast<Disc*>(h);
    if (!D) return NSFV1_ERR_ARGUMENT;
    D->status = NSFV1_OK;
    if (!D->hasMesh) { D->fail(NSFV1_ERR_STATE, "newton_solve: no mesh"); return D->status; }
    if (!u || !p || !r) { D->fail(NSFV1_ERR_ARGUMENT, "newton_solve: null argument"); return D->status; }
    nsfv1_newton_result res;
    std::memset(&res, 0, sizeof(res));
    int st;
    if (p->jacobian_prec == NSFV1_F64) st = newton_impl<double>(*D, u, u_old, dt, *p, res, (cudaStream_t)stream);
    else if (p->jacobian_prec == NSFV1_F32) st = newton_impl<float>(*D, u, u_old, dt, *p, res, (cudaStream_t)stream);
    else { D->fail(NSFV1_ERR_ARGUMENT, "newton_solve: bad precision"); return D->status; }
    if (res.status == 0 && st != 0) res.status = st;
    *r = res;
    return st;
}

}  // extern "C"
