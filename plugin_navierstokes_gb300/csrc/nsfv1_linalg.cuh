// Small dense helpers shared by the solver kernels.
#pragma once
#include <cstdint>

namespace nsfv1 {

// Inverse of one b x b block (Gauss-Jordan with partial pivoting, FP64);
// returns false on a zero pivot (O is then set to zero).
template <int b, typename VT, typename OT>
__device__ __forceinline__ bool block_inverse(const VT* __restrict__ A, OT* __restrict__ O) {
    double M[b][2 * b];
#pragma unroll
    for (int i = 0; i < b; ++i)
#pragma unroll
        for (int j = 0; j < b; ++j) { M[i][j] = (double)A[i * b + j]; M[i][b + j] = (i == j) ? 1.0 : 0.0; }
#pragma unroll
    for (int c = 0; c < b; ++c) {
        int p = c;
#pragma unroll
        for (int q = c + 1; q < b; ++q) if (fabs(M[q][c]) > fabs(M[p][c])) p = q;
        if (M[p][c] == 0.0) {
            // singular: a zero block (the caller reports the breakdown; later
            // kernels that still read this block see finite values)
#pragma unroll
            for (int i = 0; i < b * b; ++i) O[i] = (OT)0;
            return false;
        }
        if (p != c) {
#pragma unroll
            for (int j = 0; j < 2 * b; ++j) { const double t = M[p][j]; M[p][j] = M[c][j]; M[c][j] = t; }
        }
        const double piv = 1.0 / M[c][c];
#pragma unroll
        for (int j = 0; j < 2 * b; ++j) M[c][j] *= piv;
#pragma unroll
        for (int q = 0; q < b; ++q) {
            if (q == c) continue;
            const double f = M[q][c];
#pragma unroll
            for (int j = 0; j < 2 * b; ++j) M[q][j] -= f * M[c][j];
        }
    }
#pragma unroll
    for (int i = 0; i < b; ++i)
#pragma unroll
        for (int j = 0; j < b; ++j) O[i * b + j] = (OT)M[i][b + j];
    return true;
}

}  // namespace nsfv1
