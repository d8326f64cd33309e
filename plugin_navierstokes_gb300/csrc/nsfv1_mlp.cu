// Learned warm start: a coordinate MLP that predicts the Newton initial iterate
// (u, v, p) of a lid-driven cavity from (x, y) and the conditioning (log Re, lid).
//
//   features  f(x, y) = [sin(pi k x), cos(pi k x), sin(pi k y), cos(pi k y)]_{k=1..16}  (64)
//   layer l   a_l = W_l h_l ; z_l = gamma_l(c) * (a_l + b_l) + beta_l(c) ; h_{l+1} = silu(z_l)
//             (4 layers of width 256; W_0 is 256 x 64, W_1..3 are 256 x 256)
//   FiLM      gamma_l = 1 + Gw_l c + Gb_l , beta_l = Bw_l c + Bb_l ,
//             c = ((ln Re - ln 100) / ln 10, (lid - 1.25) / 0.75)
//   head      out = Wh h_4 + bh (3), prediction u = lid out_0, v = lid out_1, p = lid^2 out_2
//   loss      mean over points and the 3 channels of (out - target)^2, target = (u/lid, v/lid, p/lid^2)
//
// GEMM operands (h_l, W_l, the output and data gradients) are BF16, every GEMM
// accumulates in FP32 on the tensor cores (tcgen05, nsfv1_tc_gemm.cuh); the
// master weights, the FiLM maps, the elementwise work and Adam are FP32. Points
// are grouped in contiguous "slots" (one instance each) so that the FiLM
// gradients are per-slot sums taken in a fixed order: every result is
// deterministic.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>
#include "nsfv1_gb300.h"
#include "nsfv1_tc_gemm.cuh"

namespace {

using bf16 = __nv_bfloat16;
constexpr int kW = 256;       // width
constexpr int kL = 4;         // hidden layers
constexpr int kF = 16;        // Fourier frequencies
constexpr int kIn0 = 4 * kF;  // 64 input features
constexpr int kOut = 3;
constexpr int kHeadPad = 64;  // head rows padded for the tensor-core tile
constexpr int kRedChunks = 8; // point chunks per slot in the FiLM reductions

__host__ __device__ constexpr int layer_in(int l) { return l == 0 ? kIn0 : kW; }

// flat FP32 parameter layout: per layer [W (256 x in), b, Gw (256 x 2), Gb, Bw (256 x 2), Bb], then Wh (3 x 256), bh (3)
struct Offsets {
    int64_t W[kL], b[kL], Gw[kL], Gb[kL], Bw[kL], Bb[kL], Wh, bh, total;
    Offsets() {
        int64_t o = 0;
        for (int l = 0; l < kL; ++l) {
            W[l] = o; o += (int64_t)kW * layer_in(l);
            b[l] = o; o += kW;
            Gw[l] = o; o += 2 * kW;
            Gb[l] = o; o += kW;
            Bw[l] = o; o += 2 * kW;
            Bb[l] = o; o += kW;
        }
        Wh = o; o += kOut * kW;
        bh = o; o += kOut;
        total = o;
    }
};

uint64_t splitmix(uint64_t& s) {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

__device__ __forceinline__ uint64_t mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

__device__ __forceinline__ float sigmoid(float z) { return 1.0f / (1.0f + expf(-z)); }

// ---- kernels ----------------------------------------------------------------

// features of points [0, P) (rows P..Pp-1 zero): h0 [Pp x 64] and h0T [64 x Pp]
__global__ void k_features(int64_t P, int64_t Pp, const float2* __restrict__ xy, bf16* __restrict__ h0, bf16* __restrict__ h0T) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int k = blockIdx.y;   // frequency index 0..15
    if (i >= Pp) return;
    float v[4] = {0.f, 0.f, 0.f, 0.f};
    if (i < P) {
        const float2 p = xy[i];
        sincospif((float)(k + 1) * p.x, &v[0], &v[1]);
        sincospif((float)(k + 1) * p.y, &v[2], &v[3]);
    }
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        const bf16 h = __float2bfloat16(v[c]);
        h0[i * kIn0 + 4 * k + c] = h;
        h0T[(int64_t)(4 * k + c) * Pp + i] = h;
    }
}

// per-slot FiLM: gb[s][l][0..255] = gamma, gb[s][l][256..511] = beta
__global__ void k_film(int nSlots, const float* __restrict__ cond, const float* __restrict__ prm, Offsets off, float* __restrict__ gb) {
    const int s = blockIdx.x, l = blockIdx.y, j = threadIdx.x;
    if (s >= nSlots) return;
    const float c0 = cond[2 * s], c1 = cond[2 * s + 1];
    const float g = 1.0f + prm[off.Gw[l] + 2 * j] * c0 + prm[off.Gw[l] + 2 * j + 1] * c1 + prm[off.Gb[l] + j];
    const float be = prm[off.Bw[l] + 2 * j] * c0 + prm[off.Bw[l] + 2 * j + 1] * c1 + prm[off.Bb[l] + j];
    gb[((int64_t)s * kL + l) * 2 * kW + j] = g;
    gb[((int64_t)s * kL + l) * 2 * kW + kW + j] = be;
}

// h_{l+1} = silu(gamma (a + b) + beta) for rows < P (0 beyond), row-major and transposed.
// block (32, 8), tile 32 points x 32 features
__global__ void k_act_fwd(int64_t P, int64_t Pp, int l, const float* __restrict__ a, const float* __restrict__ prm, Offsets off,
                          const float* __restrict__ gb, const int32_t* __restrict__ pointSlot, bf16* __restrict__ h,
                          bf16* __restrict__ hT) {
    __shared__ bf16 tile[32][33];
    const int64_t i0 = blockIdx.x * 32ll;
    const int j = blockIdx.y * 32 + threadIdx.x;
    const float bj = prm[off.b[l] + j];
    for (int r = threadIdx.y; r < 32; r += 8) {
        const int64_t i = i0 + r;
        float hv = 0.f;
        if (i < P) {
            const float* g = gb + ((int64_t)pointSlot[i] * kL + l) * 2 * kW;
            const float z = g[j] * (a[i * kW + j] + bj) + g[kW + j];
            hv = z * sigmoid(z);
        }
        const bf16 hb = __float2bfloat16(hv);
        h[i * kW + j] = hb;
        tile[r][threadIdx.x] = hb;
    }
    __syncthreads();
    for (int r = threadIdx.y; r < 32; r += 8) hT[(int64_t)(blockIdx.y * 32 + r) * Pp + i0 + threadIdx.x] = tile[threadIdx.x][r];
}

// da = dh * silu'(z) * gamma (BF16, row-major and transposed; 0 for rows >= P)
__global__ void k_act_bwd(int64_t P, int64_t Pp, int l, const float* __restrict__ a, const float* __restrict__ dh,
                          const float* __restrict__ prm, Offsets off, const float* __restrict__ gb,
                          const int32_t* __restrict__ pointSlot, bf16* __restrict__ da, bf16* __restrict__ daT) {
    __shared__ bf16 tile[32][33];
    const int64_t i0 = blockIdx.x * 32ll;
    const int j = blockIdx.y * 32 + threadIdx.x;
    const float bj = prm[off.b[l] + j];
    for (int r = threadIdx.y; r < 32; r += 8) {
        const int64_t i = i0 + r;
        float v = 0.f;
        if (i < P) {
            const float* g = gb + ((int64_t)pointSlot[i] * kL + l) * 2 * kW;
            const float z = g[j] * (a[i * kW + j] + bj) + g[kW + j];
            const float sg = sigmoid(z);
            v = dh[i * kW + j] * sg * (1.0f + z * (1.0f - sg)) * g[j];
        }
        const bf16 vb = __float2bfloat16(v);
        da[i * kW + j] = vb;
        tile[r][threadIdx.x] = vb;
    }
    __syncthreads();
    for (int r = threadIdx.y; r < 32; r += 8) daT[(int64_t)(blockIdx.y * 32 + r) * Pp + i0 + threadIdx.x] = tile[threadIdx.x][r];
}

// per (slot, chunk) partial sums over the chunk's points of
//   dgamma = dz (a + b), dbeta = dz, db = dz gamma   (dz = dh silu'(z))
__global__ void k_slot_red(int l, const int32_t* __restrict__ slotPtr, const float* __restrict__ a, const float* __restrict__ dh,
                           const float* __restrict__ prm, Offsets off, const float* __restrict__ gb, float* __restrict__ part) {
    const int s = blockIdx.x, c = blockIdx.y, j = threadIdx.x;
    const int64_t p0 = slotPtr[s], p1 = slotPtr[s + 1];
    const int64_t len = p1 - p0;
    const int64_t q0 = p0 + len * c / kRedChunks, q1 = p0 + len * (c + 1) / kRedChunks;
    const float* g = gb + ((int64_t)s * kL + l) * 2 * kW;
    const float gj = g[j], bej = g[kW + j], bj = prm[off.b[l] + j];
    float sg_ = 0.f, sb_ = 0.f, sd_ = 0.f;
    for (int64_t i = q0; i < q1; ++i) {
        const float ab = a[i * kW + j] + bj;
        const float z = gj * ab + bej;
        const float sg = sigmoid(z);
        const float dz = dh[i * kW + j] * sg * (1.0f + z * (1.0f - sg));
        sg_ += dz * ab;
        sb_ += dz;
        sd_ += dz * gj;
    }
    float* o = part + ((int64_t)s * kRedChunks + c) * 3 * kW;
    o[j] = sg_;
    o[kW + j] = sb_;
    o[2 * kW + j] = sd_;
}

// FiLM and bias gradients of layer l from the per-slot partials (fixed order)
__global__ void k_film_grad(int l, int nSlots, const float* __restrict__ cond, const float* __restrict__ part, Offsets off,
                            float* __restrict__ grad) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= kW) return;
    float gw0 = 0.f, gw1 = 0.f, gbs = 0.f, bw0 = 0.f, bw1 = 0.f, bbs = 0.f, db = 0.f;
    for (int s = 0; s < nSlots; ++s) {
        float dg = 0.f, dbe = 0.f;
        for (int c = 0; c < kRedChunks; ++c) {
            const float* o = part + ((int64_t)s * kRedChunks + c) * 3 * kW;
            dg += o[j];
            dbe += o[kW + j];
            db += o[2 * kW + j];
        }
        const float c0 = cond[2 * s], c1 = cond[2 * s + 1];
        gw0 += dg * c0; gw1 += dg * c1; gbs += dg;
        bw0 += dbe * c0; bw1 += dbe * c1; bbs += dbe;
    }
    grad[off.Gw[l] + 2 * j] = gw0;
    grad[off.Gw[l] + 2 * j + 1] = gw1;
    grad[off.Gb[l] + j] = gbs;
    grad[off.Bw[l] + 2 * j] = bw0;
    grad[off.Bw[l] + 2 * j + 1] = bw1;
    grad[off.Bb[l] + j] = bbs;
    grad[off.b[l] + j] = db;
}

// head: residual r = out + bh - target (points < P), dout = 2 r / (3 P) as BF16 [Pp x 64] and [64 x Pp];
// per-block partial sums of r^2 and of dout (the bias gradient), fixed order
__global__ void k_head_loss(int64_t P, int64_t Pp, const float* __restrict__ out, const float* __restrict__ prm, Offsets off,
                            const float* __restrict__ target, bf16* __restrict__ dout, bf16* __restrict__ doutT,
                            double* __restrict__ lossPart, float* __restrict__ dbhPart) {
    __shared__ double sl[256];
    __shared__ float sb[3][256];
    const int64_t i = blockIdx.x * 256ll + threadIdx.x;
    double l2 = 0.0;
    float d[3] = {0.f, 0.f, 0.f};
    if (i < P) {
        const float scale = 2.0f / (3.0f * (float)P);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float r = out[i * kHeadPad + c] + prm[off.bh + c] - target[i * 3 + c];
            l2 += (double)r * r;
            d[c] = scale * r;
        }
    }
    if (i < Pp) {
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const bf16 v = __float2bfloat16(d[c]);
            dout[i * kHeadPad + c] = v;
            doutT[(int64_t)c * Pp + i] = v;
        }
    }
    sl[threadIdx.x] = l2;
    for (int c = 0; c < 3; ++c) sb[c][threadIdx.x] = d[c];
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (threadIdx.x < w) {
            sl[threadIdx.x] += sl[threadIdx.x + w];
            for (int c = 0; c < 3; ++c) sb[c][threadIdx.x] += sb[c][threadIdx.x + w];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        lossPart[blockIdx.x] = sl[0];
        for (int c = 0; c < 3; ++c) dbhPart[blockIdx.x * 3 + c] = sb[c][0];
    }
}

__global__ void k_head_reduce(int nBlocks, int64_t P, const double* __restrict__ lossPart, const float* __restrict__ dbhPart,
                              Offsets off, float* __restrict__ grad, double* __restrict__ loss) {
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int b = 0; b < nBlocks; ++b) s += lossPart[b];
        *loss = s / (3.0 * (double)P);
    }
    if (threadIdx.x < 3) {
        float s = 0.f;
        for (int b = 0; b < nBlocks; ++b) s += dbhPart[b * 3 + threadIdx.x];
        grad[off.bh + threadIdx.x] = s;
    }
}

// sum of split-K partials part[z][M][N] into dst (row-major M x N), fixed order
__global__ void k_sum_splits(int splits, int64_t MN, const float* __restrict__ part, float* __restrict__ dst) {
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= MN) return;
    float s = 0.f;
    for (int z = 0; z < splits; ++z) s += part[z * MN + e];
    dst[e] = s;
}

// head weight gradient from C = dWh^T [256 x 64] partials: grad Wh[c][j] = sum_z C[z][j][c], c < 3
__global__ void k_sum_splits_head(int splits, const float* __restrict__ part, Offsets off, float* __restrict__ grad) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= kOut * kW) return;
    const int c = e / kW, j = e % kW;
    float s = 0.f;
    for (int z = 0; z < splits; ++z) s += part[(int64_t)z * kW * kHeadPad + j * kHeadPad + c];
    grad[off.Wh + e] = s;
}

// BF16 copies of the weights: W_l [256 x in], WT_l [in x 256], Wh [64 x 256] and WhT [256 x 64] (padding zero)
__global__ void k_refresh(const float* __restrict__ prm, Offsets off, bf16* __restrict__ W0, bf16* __restrict__ W1,
                          bf16* __restrict__ W2, bf16* __restrict__ W3, bf16* __restrict__ T0, bf16* __restrict__ T1,
                          bf16* __restrict__ T2, bf16* __restrict__ T3, bf16* __restrict__ Wh, bf16* __restrict__ WhT) {
    const int l = blockIdx.y;
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (l < kL) {
        const int in = layer_in(l);
        if (e >= kW * in) return;
        bf16* W = l == 0 ? W0 : l == 1 ? W1 : l == 2 ? W2 : W3;
        bf16* T = l == 0 ? T0 : l == 1 ? T1 : l == 2 ? T2 : T3;
        const int r = e / in, c = e % in;
        const bf16 v = __float2bfloat16(prm[off.W[l] + e]);
        W[e] = v;
        T[c * kW + r] = v;
    } else {
        if (e >= kHeadPad * kW) return;
        const int r = e / kW, c = e % kW;
        const bf16 v = __float2bfloat16(r < kOut ? prm[off.Wh + r * kW + c] : 0.f);
        Wh[e] = v;
        WhT[c * kHeadPad + r] = v;
    }
}

__global__ void k_adam(int64_t n, float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m, float* __restrict__ v,
                       float lr, float b1, float b2, float eps, float c1, float c2) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

// minibatch: slot s draws training instance k_s, point q of the slot draws node n_{s,q} (counter-based hash)
__global__ void k_sample(int64_t step, uint64_t seed, int nSlots, int Q, int nTrain, int nNodes, const float2* __restrict__ coords,
                         const float* __restrict__ targets, const float* __restrict__ condTrain, float2* __restrict__ xy,
                         float* __restrict__ tgt, float* __restrict__ cond) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= (int64_t)nSlots * Q) return;
    const int s = (int)(i / Q);
    const uint64_t hs = mix64(seed ^ mix64(((uint64_t)step << 20) + (uint64_t)s));
    const int k = (int)(hs % (uint64_t)nTrain);
    const uint64_t hp = mix64(hs + 0x632BE59BD9B4E019ull * (uint64_t)(i + 1));
    const int node = (int)(hp % (uint64_t)nNodes);
    xy[i] = coords[node];
    const float* t = targets + ((int64_t)k * nNodes + node) * 3;
    tgt[i * 3] = t[0];
    tgt[i * 3 + 1] = t[1];
    tgt[i * 3 + 2] = t[2];
    if (i % Q == 0) {
        cond[2 * s] = condTrain[2 * k];
        cond[2 * s + 1] = condTrain[2 * k + 1];
    }
}

__global__ void k_slots_of_points(int nSlots, const int32_t* __restrict__ slotPtr, int32_t* __restrict__ pointSlot) {
    const int s = blockIdx.x;
    if (s >= nSlots) return;
    for (int64_t i = slotPtr[s] + threadIdx.x; i < slotPtr[s + 1]; i += blockDim.x) pointSlot[i] = s;
}

// prediction (points [i0, i0+P) of the full vector): out (+bh) scaled by lid into the FP64 state
__global__ void k_write_state(int64_t P, int64_t i0, const float* __restrict__ out, const float* __restrict__ prm, Offsets off,
                              const int32_t* __restrict__ pointSlot, const float* __restrict__ lid, double* __restrict__ u,
                              float* __restrict__ outF) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= P) return;
    const float o0 = out[i * kHeadPad] + prm[off.bh], o1 = out[i * kHeadPad + 1] + prm[off.bh + 1],
                o2 = out[i * kHeadPad + 2] + prm[off.bh + 2];
    if (outF) {
        outF[(i0 + i) * 3] = o0;
        outF[(i0 + i) * 3 + 1] = o1;
        outF[(i0 + i) * 3 + 2] = o2;
    }
    if (u) {
        const double L = lid[pointSlot[i]];
        u[(i0 + i) * 3] = L * (double)o0;
        u[(i0 + i) * 3 + 1] = L * (double)o1;
        u[(i0 + i) * 3 + 2] = L * L * (double)o2;
    }
}

// normalised training targets of instances that share one mesh: t = (u/lid, v/lid, p/lid^2)
__global__ void k_targets(int64_t n, int nNodes, const double* __restrict__ u, const double* __restrict__ lid, float* __restrict__ t) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double L = lid[i / nNodes];
    t[i * 3] = (float)(u[i * 3] / L);
    t[i * 3 + 1] = (float)(u[i * 3 + 1] / L);
    t[i * 3 + 2] = (float)(u[i * 3 + 2] / (L * L));
}

// ---- tensor-core GEMM launcher ------------------------------------------------

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
    });
    return fn;
}

// K-major BF16 operand [rows x K] (row stride K), box {64, boxRows}, 128-byte swizzle
bool make_map(CUtensorMap* m, const void* ptr, int64_t rows, int64_t K, int boxRows) {
    auto fn = encode_fn();
    if (!fn) return false;
    cuuint64_t dims[2] = {(cuuint64_t)K, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)K * 2};
    cuuint32_t box[2] = {(cuuint32_t)nsfv1::tc::BK, (cuuint32_t)boxRows};
    cuuint32_t es[2] = {1, 1};
    return fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(ptr), dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
              CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int BN, int STAGES>
cudaError_t launch_gemm(const CUtensorMap& a, const CUtensorMap& b, float* C, int M, int N, int K, int splits, int kChunk, int* err,
                        cudaStream_t s) {
    using S = nsfv1::tc::GemmSmem<BN, STAGES>;
    // per launch: the attribute belongs to the current device
    cudaError_t e = cudaFuncSetAttribute(nsfv1::tc::k_gemm_bf16_tn<BN, STAGES>, cudaFuncAttributeMaxDynamicSharedMemorySize, S::kBytes);
    if (e != cudaSuccess) return e;
    dim3 grid(M / nsfv1::tc::BM, N / BN, splits);
    nsfv1::tc::k_gemm_bf16_tn<BN, STAGES><<<grid, 128, S::kBytes, s>>>(a, b, C, M, N, K, kChunk, err);
    return cudaGetLastError();
}

// C[splits][M][N] = A[M x K] * B[N x K]^T (partials per K chunk). Returns the
// number of splits actually used (>= 1), or -1 on an argument / launch error.
int gemm_bf16(const bf16* A, const bf16* B, float* C, int M, int N, int K, int splits, int* err, cudaStream_t s, std::string& why) {
    if (M <= 0 || M % 128 || K <= 0 || K % 64 || !(N == 64 || N == 128 || N % 256 == 0) || splits < 1) {
        why = "gemm: M must be a multiple of 128, K of 64, N 64, 128 or a multiple of 256";
        return -1;
    }
    if (((uintptr_t)A | (uintptr_t)B | (uintptr_t)C) & 15) { why = "gemm: operands must be 16-byte aligned"; return -1; }
    const int kTiles = K / 64;
    splits = std::min(splits, kTiles);
    const int chunkTiles = (kTiles + splits - 1) / splits;
    splits = (kTiles + chunkTiles - 1) / chunkTiles;   // every split gets at least one tile
    const int kChunk = chunkTiles * 64;
    const int BN = N == 64 ? 64 : N == 128 ? 128 : 256;
    CUtensorMap ma, mb;
    if (!make_map(&ma, A, M, K, 128) || !make_map(&mb, B, N, K, BN)) { why = "gemm: tensor map encoding failed"; return -1; }
    cudaError_t e = BN == 64 ? launch_gemm<64, 6>(ma, mb, C, M, N, K, splits, kChunk, err, s)
                  : BN == 128 ? launch_gemm<128, 5>(ma, mb, C, M, N, K, splits, kChunk, err, s)
                              : launch_gemm<256, 4>(ma, mb, C, M, N, K, splits, kChunk, err, s);
    if (e != cudaSuccess) { why = std::string("gemm launch: ") + cudaGetErrorString(e); return -1; }
    return splits;
}

int g_num_sms() {
    int dev = 0, n = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    return n > 0 ? n : 152;
}

}  // namespace

// ---- the handle -------------------------------------------------------------

struct nsfv1_mlp {
    Offsets off;
    int64_t cap = 0;        // point capacity (multiple of 128)
    int maxSlots = 0;
    float *prm = nullptr, *grad = nullptr, *am = nullptr, *av = nullptr;
    bf16 *W[kL] = {}, *WT[kL] = {}, *Wh = nullptr, *WhT = nullptr;
    bf16 *h[kL + 1] = {}, *hT[kL + 1] = {};
    float* a[kL] = {};
    float *out = nullptr, *dh = nullptr, *gb = nullptr, *part = nullptr, *splitBuf = nullptr, *cond = nullptr, *lid = nullptr;
    bf16 *dout = nullptr, *doutT = nullptr, *da = nullptr, *daT = nullptr;
    float *dbhPart = nullptr, *tgt = nullptr;
    float2* xy = nullptr;
    double *lossPart = nullptr, *loss = nullptr;
    int32_t *slotPtr = nullptr, *pointSlot = nullptr;
    int* err = nullptr;
    int64_t adamStep = 0;
    size_t splitCap = 0;
    std::string lastError;

    ~nsfv1_mlp() {
        auto f = [](auto*& p) { if (p) cudaFree((void*)p); p = nullptr; };
        f(prm); f(grad); f(am); f(av); f(Wh); f(WhT);
        for (int l = 0; l < kL; ++l) { f(W[l]); f(WT[l]); f(a[l]); }
        for (int l = 0; l <= kL; ++l) { f(h[l]); f(hT[l]); }
        f(out); f(dh); f(gb); f(part); f(splitBuf); f(cond); f(lid); f(dout); f(doutT); f(da); f(daT); f(dbhPart); f(tgt); f(xy);
        f(lossPart); f(loss); f(slotPtr); f(pointSlot); f(err);
    }
    int fail(int code, const std::string& m) { lastError = m; return code; }
    int cuda(cudaError_t e, const char* where) {
        if (e == cudaSuccess) return NSFV1_OK;
        return fail(NSFV1_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
    }
    int refresh(cudaStream_t s) {
        k_refresh<<<dim3((kW * kW + 255) / 256, kL + 1), 256, 0, s>>>(prm, off, W[0], W[1], W[2], W[3], WT[0], WT[1], WT[2], WT[3], Wh, WhT);
        return cuda(cudaGetLastError(), "mlp weights");
    }
    int gemm(const bf16* A, const bf16* B, float* C, int M, int N, int K, int splits, cudaStream_t s, int* used = nullptr) {
        std::string why;
        if (C == splitBuf && (size_t)nsfv1_gemm_bf16_splits(K, splits) * M * N * 4 > splitCap)
            return fail(NSFV1_ERR_ARGUMENT, "mlp: split-K partials exceed the staging buffer");
        const int u = gemm_bf16(A, B, C, M, N, K, splits, err, s, why);
        if (u < 0) return fail(NSFV1_ERR_ARGUMENT, why);
        if (used) *used = u;
        return NSFV1_OK;
    }
    int check_err(cudaStream_t s) {
        int h = 0;
        int st = cuda(cudaMemcpyAsync(&h, err, sizeof(int), cudaMemcpyDeviceToHost, s), "mlp status");
        if (st) return st;
        if ((st = cuda(cudaStreamSynchronize(s), "mlp"))) return st;
        if (h) {
            cudaMemsetAsync(err, 0, sizeof(int), s);
            return fail(NSFV1_ERR_TIMEOUT, "mlp: a tensor-core GEMM wait timed out");
        }
        return NSFV1_OK;
    }
    // forward of P <= cap points whose xy / pointSlot / gb are in place
    int forward(int64_t P, cudaStream_t s) {
        const int64_t Pp = (P + 127) / 128 * 128;
        k_features<<<dim3((unsigned)((Pp + 255) / 256), kF), 256, 0, s>>>(P, Pp, xy, h[0], hT[0]);
        for (int l = 0; l < kL; ++l) {
            if (int st = gemm(h[l], W[l], a[l], (int)Pp, kW, layer_in(l), 1, s)) return st;
            k_act_fwd<<<dim3((unsigned)(Pp / 32), kW / 32), dim3(32, 8), 0, s>>>(P, Pp, l, a[l], prm, off, gb, pointSlot, h[l + 1], hT[l + 1]);
        }
        if (int st = gemm(h[kL], Wh, out, (int)Pp, kHeadPad, kW, 1, s)) return st;
        return cuda(cudaGetLastError(), "mlp forward");
    }
    int split_count(int64_t Pp, int tilesMN) const {
        const int want = std::max(1, g_num_sms() / std::max(1, tilesMN));
        return (int)std::min<int64_t>(want, Pp / 64);
    }
    // backward after forward(P) and the head loss; fills grad (all entries)
    int backward(int64_t P, int nSlots, cudaStream_t s) {
        const int64_t Pp = (P + 127) / 128 * 128;
        int used = 0;
        // head weights: C = h4^T dout -> [256 x 64]
        if (int st = gemm(hT[kL], doutT, splitBuf, kW, kHeadPad, (int)Pp, split_count(Pp, 2), s, &used)) return st;
        k_sum_splits_head<<<(kOut * kW + 255) / 256, 256, 0, s>>>(used, splitBuf, off, grad);
        // dh4 = dout Wh
        if (int st = gemm(dout, WhT, dh, (int)Pp, kW, kHeadPad, 1, s)) return st;
        for (int l = kL - 1; l >= 0; --l) {
            k_slot_red<<<dim3(nSlots, kRedChunks), kW, 0, s>>>(l, slotPtr, a[l], dh, prm, off, gb, part);
            k_film_grad<<<1, kW, 0, s>>>(l, nSlots, cond, part, off, grad);
            k_act_bwd<<<dim3((unsigned)(Pp / 32), kW / 32), dim3(32, 8), 0, s>>>(P, Pp, l, a[l], dh, prm, off, gb, pointSlot, da, daT);
            const int in = layer_in(l);
            // dW_l = da^T h_l -> [256 x in]
            if (int st = gemm(daT, hT[l], splitBuf, kW, in, (int)Pp, split_count(Pp, 2 * (in / std::min(in, 256))), s, &used)) return st;
            k_sum_splits<<<(kW * in + 255) / 256, 256, 0, s>>>(used, (int64_t)kW * in, splitBuf, grad + off.W[l]);
            // dh_l = da W_l
            if (l > 0)
                if (int st = gemm(da, WT[l], dh, (int)Pp, in, kW, 1, s)) return st;
        }
        return cuda(cudaGetLastError(), "mlp backward");
    }
    int head_loss(int64_t P, cudaStream_t s) {
        const int64_t Pp = (P + 127) / 128 * 128;
        const int nb = (int)((Pp + 255) / 256);
        // rows 3..63 of the transposed output gradient are padding: zero for this row stride
        if (int st = cuda(cudaMemsetAsync(doutT + 3 * Pp, 0, (size_t)(kHeadPad - 3) * Pp * 2, s), "mlp loss")) return st;
        k_head_loss<<<nb, 256, 0, s>>>(P, Pp, out, prm, off, tgt, dout, doutT, lossPart, dbhPart);
        k_head_reduce<<<1, 32, 0, s>>>(nb, P, lossPart, dbhPart, off, grad, loss);
        return cuda(cudaGetLastError(), "mlp loss");
    }
    int upload_slots(int nSlots, const int32_t* slotPtrHost, cudaStream_t s) {
        if (int st = cuda(cudaMemcpyAsync(slotPtr, slotPtrHost, (nSlots + 1) * 4, cudaMemcpyHostToDevice, s), "mlp slots")) return st;
        k_slots_of_points<<<nSlots, 256, 0, s>>>(nSlots, slotPtr, pointSlot);
        return cuda(cudaGetLastError(), "mlp slots");
    }
};

namespace {
int check_slots(nsfv1_mlp* m, int64_t P, int nSlots, const int32_t* slotPtr) {
    if (P <= 0 || P > m->cap) return m->fail(NSFV1_ERR_ARGUMENT, "mlp: number of points outside (0, capacity]");
    if (nSlots <= 0 || nSlots > m->maxSlots) return m->fail(NSFV1_ERR_ARGUMENT, "mlp: number of slots outside (0, max_slots]");
    if (!slotPtr || slotPtr[0] != 0 || slotPtr[nSlots] != P) return m->fail(NSFV1_ERR_ARGUMENT, "mlp: slot_ptr must run from 0 to n_points");
    for (int s = 0; s < nSlots; ++s)
        if (slotPtr[s + 1] <= slotPtr[s]) return m->fail(NSFV1_ERR_ARGUMENT, "mlp: every slot needs at least one point");
    return NSFV1_OK;
}
}  // namespace

extern "C" {

int nsfv1_mlp_create(const nsfv1_mlp_config* cfg, nsfv1_mlp** out) {
    if (!out) return NSFV1_ERR_ARGUMENT;
    *out = nullptr;
    if (!cfg || cfg->max_points <= 0 || cfg->max_slots <= 0) return NSFV1_ERR_ARGUMENT;
    if (!encode_fn()) return NSFV1_ERR_CUDA;
    auto* m = new nsfv1_mlp();
    m->cap = ((int64_t)cfg->max_points + 127) / 128 * 128;
    m->maxSlots = cfg->max_slots;
    const int64_t P = m->cap, np = m->off.total;
    bool ok = true;
    auto al = [&](auto*& p, size_t bytes) { if (ok && cudaMalloc((void**)&p, bytes) != cudaSuccess) ok = false; };
    al(m->prm, np * 4); al(m->grad, np * 4); al(m->am, np * 4); al(m->av, np * 4);
    for (int l = 0; l < kL; ++l) { al(m->W[l], (size_t)kW * layer_in(l) * 2); al(m->WT[l], (size_t)kW * layer_in(l) * 2); al(m->a[l], (size_t)P * kW * 4); }
    al(m->Wh, kHeadPad * kW * 2); al(m->WhT, kHeadPad * kW * 2);
    for (int l = 0; l <= kL; ++l) { al(m->h[l], (size_t)P * layer_in(l) * 2); al(m->hT[l], (size_t)P * layer_in(l) * 2); }
    al(m->out, (size_t)P * kHeadPad * 4); al(m->dh, (size_t)P * kW * 4);
    al(m->gb, (size_t)m->maxSlots * kL * 2 * kW * 4);
    al(m->part, (size_t)m->maxSlots * kRedChunks * 3 * kW * 4);
    m->splitCap = (size_t)2 * g_num_sms() * kW * kW * 4;
    al(m->splitBuf, m->splitCap);
    al(m->cond, (size_t)m->maxSlots * 2 * 4); al(m->lid, (size_t)m->maxSlots * 4);
    al(m->dout, (size_t)P * kHeadPad * 2); al(m->doutT, (size_t)P * kHeadPad * 2);
    al(m->da, (size_t)P * kW * 2); al(m->daT, (size_t)P * kW * 2);
    al(m->dbhPart, (size_t)(P / 256 + 1) * 3 * 4); al(m->lossPart, (size_t)(P / 256 + 1) * 8); al(m->loss, 8);
    al(m->tgt, (size_t)P * 3 * 4); al(m->xy, (size_t)P * 8);
    al(m->slotPtr, (size_t)(m->maxSlots + 1) * 4); al(m->pointSlot, (size_t)P * 4); al(m->err, 4);
    if (ok) ok = cudaMemset(m->dout, 0, (size_t)P * kHeadPad * 2) == cudaSuccess && cudaMemset(m->doutT, 0, (size_t)P * kHeadPad * 2) == cudaSuccess &&
                 cudaMemset(m->err, 0, 4) == cudaSuccess && cudaMemset(m->am, 0, np * 4) == cudaSuccess &&
                 cudaMemset(m->av, 0, np * 4) == cudaSuccess && cudaMemset(m->grad, 0, np * 4) == cudaSuccess;
    if (!ok) { delete m; return NSFV1_ERR_CUDA; }
    *out = m;
    return NSFV1_OK;
}

void nsfv1_mlp_destroy(nsfv1_mlp* m) { delete m; }

const char* nsfv1_mlp_last_error(const nsfv1_mlp* m) { return m ? m->lastError.c_str() : "null handle"; }

int64_t nsfv1_mlp_num_params(const nsfv1_mlp* m) { return m ? m->off.total : 0; }

int nsfv1_mlp_init(nsfv1_mlp* m, uint64_t seed) {
    if (!m) return NSFV1_ERR_ARGUMENT;
    std::vector<float> p(m->off.total, 0.0f);
    uint64_t st = seed;
    auto uni = [&](float bound) { return (float)(((splitmix(st) >> 11) * (1.0 / 9007199254740992.0)) * 2.0 - 1.0) * bound; };
    for (int l = 0; l < kL; ++l) {
        const float bound = std::sqrt(6.0f / (float)layer_in(l));
        for (int64_t e = 0; e < (int64_t)kW * layer_in(l); ++e) p[m->off.W[l] + e] = uni(bound);
    }
    const float hb = std::sqrt(3.0f / (float)kW);
    for (int e = 0; e < kOut * kW; ++e) p[m->off.Wh + e] = uni(hb);
    m->adamStep = 0;
    if (int st2 = m->cuda(cudaMemcpy(m->prm, p.data(), p.size() * 4, cudaMemcpyHostToDevice), "mlp init")) return st2;
    cudaMemset(m->am, 0, p.size() * 4);
    cudaMemset(m->av, 0, p.size() * 4);
    if (int st3 = m->refresh(0)) return st3;
    return m->cuda(cudaDeviceSynchronize(), "mlp init");
}

int nsfv1_mlp_get_params(nsfv1_mlp* m, float* host, int64_t n) {
    if (!m || !host || n != m->off.total) return NSFV1_ERR_ARGUMENT;
    return m->cuda(cudaMemcpy(host, m->prm, n * 4, cudaMemcpyDeviceToHost), "mlp get params");
}

int nsfv1_mlp_set_params(nsfv1_mlp* m, const float* host, int64_t n) {
    if (!m || !host || n != m->off.total) return NSFV1_ERR_ARGUMENT;
    if (int st = m->cuda(cudaMemcpy(m->prm, host, n * 4, cudaMemcpyHostToDevice), "mlp set params")) return st;
    if (int st = m->refresh(0)) return st;
    return m->cuda(cudaDeviceSynchronize(), "mlp set params");
}

int nsfv1_mlp_forward(nsfv1_mlp* m, int64_t n_points, const float* xy, int n_slots, const int32_t* slot_ptr, const float* cond,
                      float* out, void* stream) {
    if (!m || !xy || !cond || !out) return NSFV1_ERR_ARGUMENT;
    if (int st = check_slots(m, n_points, n_slots, slot_ptr)) return st;
    cudaStream_t s = (cudaStream_t)stream;
    if (int st = m->cuda(cudaMemcpyAsync(m->cond, cond, n_slots * 8, cudaMemcpyHostToDevice, s), "mlp cond")) return st;
    if (int st = m->upload_slots(n_slots, slot_ptr, s)) return st;
    k_film<<<dim3(n_slots, kL), kW, 0, s>>>(n_slots, m->cond, m->prm, m->off, m->gb);
    if (int st = m->cuda(cudaMemcpyAsync(m->xy, xy, n_points * 8, cudaMemcpyDeviceToDevice, s), "mlp xy")) return st;
    if (int st = m->forward(n_points, s)) return st;
    k_write_state<<<(unsigned)((n_points + 255) / 256), 256, 0, s>>>(n_points, 0, m->out, m->prm, m->off, m->pointSlot, nullptr, nullptr, out);
    if (int st = m->cuda(cudaGetLastError(), "mlp forward")) return st;
    return m->check_err(s);
}

int nsfv1_mlp_loss_grad(nsfv1_mlp* m, int64_t n_points, const float* xy, int n_slots, const int32_t* slot_ptr, const float* cond,
                        const float* target, double* loss, float* grad, void* stream) {
    if (!m || !xy || !cond || !target || !grad) return NSFV1_ERR_ARGUMENT;
    if (int st = check_slots(m, n_points, n_slots, slot_ptr)) return st;
    cudaStream_t s = (cudaStream_t)stream;
    if (int st = m->cuda(cudaMemcpyAsync(m->cond, cond, n_slots * 8, cudaMemcpyHostToDevice, s), "mlp cond")) return st;
    if (int st = m->upload_slots(n_slots, slot_ptr, s)) return st;
    k_film<<<dim3(n_slots, kL), kW, 0, s>>>(n_slots, m->cond, m->prm, m->off, m->gb);
    if (int st = m->cuda(cudaMemcpyAsync(m->xy, xy, n_points * 8, cudaMemcpyDeviceToDevice, s), "mlp xy")) return st;
    if (int st = m->cuda(cudaMemcpyAsync(m->tgt, target, n_points * 12, cudaMemcpyDeviceToDevice, s), "mlp target")) return st;
    if (int st = m->forward(n_points, s)) return st;
    if (int st = m->head_loss(n_points, s)) return st;
    if (int st = m->backward(n_points, n_slots, s)) return st;
    if (int st = m->cuda(cudaMemcpyAsync(grad, m->grad, m->off.total * 4, cudaMemcpyDeviceToDevice, s), "mlp grad")) return st;
    if (loss)
        if (int st = m->cuda(cudaMemcpyAsync(loss, m->loss, 8, cudaMemcpyDeviceToHost, s), "mlp loss")) return st;
    return m->check_err(s);
}

int nsfv1_mlp_train(nsfv1_mlp* m, const nsfv1_mlp_dataset* data, const nsfv1_mlp_train_params* tp, float* loss_history, void* stream) {
    if (!m || !data || !tp || !data->coords || !data->targets || !data->cond) return NSFV1_ERR_ARGUMENT;
    if (data->n_train <= 0 || data->n_nodes <= 0 || tp->steps <= 0 || tp->slots <= 0 || tp->points_per_slot <= 0)
        return m->fail(NSFV1_ERR_ARGUMENT, "mlp train: empty dataset or schedule");
    const int64_t P = (int64_t)tp->slots * tp->points_per_slot;
    if (P > m->cap || tp->slots > m->maxSlots) return m->fail(NSFV1_ERR_ARGUMENT, "mlp train: slots x points_per_slot above capacity");
    cudaStream_t s = (cudaStream_t)stream;
    std::vector<int32_t> sp(tp->slots + 1);
    for (int i = 0; i <= tp->slots; ++i) sp[i] = i * tp->points_per_slot;
    if (int st = m->upload_slots(tp->slots, sp.data(), s)) return st;
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    for (int it = 0; it < tp->steps; ++it) {
        k_sample<<<(unsigned)((P + 255) / 256), 256, 0, s>>>(it + tp->step_offset, tp->seed, tp->slots, tp->points_per_slot, data->n_train,
                                                         data->n_nodes, (const float2*)data->coords, data->targets, data->cond, m->xy, m->tgt, m->cond);
        k_film<<<dim3(tp->slots, kL), kW, 0, s>>>(tp->slots, m->cond, m->prm, m->off, m->gb);
        if (int st = m->forward(P, s)) return st;
        if (int st = m->head_loss(P, s)) return st;
        if (int st = m->backward(P, tp->slots, s)) return st;
        // cosine schedule from lr to lr_final
        const double fr = tp->steps > 1 ? (double)it / (tp->steps - 1) : 1.0;
        const float lr = (float)(tp->lr_final + 0.5 * (tp->lr - tp->lr_final) * (1.0 + std::cos(M_PI * fr)));
        ++m->adamStep;
        const float c1 = 1.0f - std::pow(b1, (float)m->adamStep), c2 = 1.0f - std::pow(b2, (float)m->adamStep);
        k_adam<<<(unsigned)((m->off.total + 255) / 256), 256, 0, s>>>(m->off.total, m->prm, m->grad, m->am, m->av, lr, b1, b2, eps, c1, c2);
        if (int st = m->refresh(s)) return st;
        if (loss_history) {
            double l = 0.0;
            if (int st = m->cuda(cudaMemcpyAsync(&l, m->loss, 8, cudaMemcpyDeviceToHost, s), "mlp loss")) return st;
            if (int st = m->cuda(cudaStreamSynchronize(s), "mlp train")) return st;
            loss_history[it] = (float)l;
        }
    }
    return m->check_err(s);
}

void nsfv1_mlp_condition(double re, double lid, float* c2) {
    c2[0] = (float)((std::log(re) - std::log(100.0)) / std::log(10.0));
    c2[1] = (float)((lid - 1.25) / 0.75);
}

int nsfv1_mlp_targets(int64_t n_instances, int64_t n_nodes, const double* u, const double* lid, float* targets, void* stream) {
    if (n_instances <= 0 || n_nodes <= 0 || !u || !lid || !targets) return NSFV1_ERR_ARGUMENT;
    const int64_t n = n_instances * n_nodes;
    k_targets<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(n, (int)n_nodes, u, lid, targets);
    return cudaGetLastError() == cudaSuccess ? NSFV1_OK : NSFV1_ERR_CUDA;
}

int nsfv1_mlp_predict(nsfv1_mlp* m, int64_t n_points, const float* xy, int n_slots, const int32_t* slot_ptr, const float* cond,
                      const float* lid, double* u, void* stream) {
    if (!m || !xy || !cond || !lid || !u || !slot_ptr || n_slots <= 0 || n_points <= 0) return NSFV1_ERR_ARGUMENT;
    if (slot_ptr[0] != 0 || slot_ptr[n_slots] != n_points) return m->fail(NSFV1_ERR_ARGUMENT, "mlp: slot_ptr must run from 0 to n_points");
    cudaStream_t s = (cudaStream_t)stream;
    // chunks of whole slots that fit the capacity
    int s0 = 0;
    while (s0 < n_slots) {
        int s1 = s0;
        while (s1 < n_slots && (int64_t)slot_ptr[s1 + 1] - slot_ptr[s0] <= m->cap && s1 - s0 < m->maxSlots) ++s1;
        if (s1 == s0) return m->fail(NSFV1_ERR_ARGUMENT, "mlp predict: one slot exceeds the point capacity");
        const int ns = s1 - s0;
        const int64_t p0 = slot_ptr[s0], P = (int64_t)slot_ptr[s1] - p0;
        std::vector<int32_t> sp(ns + 1);
        for (int i = 0; i <= ns; ++i) sp[i] = slot_ptr[s0 + i] - (int32_t)p0;
        if (int st = m->cuda(cudaMemcpyAsync(m->cond, cond + 2 * s0, ns * 8, cudaMemcpyHostToDevice, s), "mlp cond")) return st;
        if (int st = m->cuda(cudaMemcpyAsync(m->lid, lid + s0, ns * 4, cudaMemcpyHostToDevice, s), "mlp lid")) return st;
        if (int st = m->upload_slots(ns, sp.data(), s)) return st;
        k_film<<<dim3(ns, kL), kW, 0, s>>>(ns, m->cond, m->prm, m->off, m->gb);
        if (int st = m->cuda(cudaMemcpyAsync(m->xy, xy + 2 * p0, P * 8, cudaMemcpyDeviceToDevice, s), "mlp xy")) return st;
        if (int st = m->forward(P, s)) return st;
        k_write_state<<<(unsigned)((P + 255) / 256), 256, 0, s>>>(P, p0, m->out, m->prm, m->off, m->pointSlot, m->lid, u, nullptr);
        if (int st = m->cuda(cudaGetLastError(), "mlp predict")) return st;
        // the staging buffers are reused by the next chunk
        if (int st = m->cuda(cudaStreamSynchronize(s), "mlp predict")) return st;
        s0 = s1;
    }
    return m->check_err(s);
}

int nsfv1_gemm_bf16(int M, int N, int K, const void* A, const void* B, float* C, int splits, void* stream) {
    // status word of the bounded waits, one per device
    static int* errs[64] = {nullptr};
    static std::mutex mu;
    std::lock_guard<std::mutex> g(mu);
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64) return NSFV1_ERR_ARGUMENT;
    int*& err = errs[dev];
    if (!err && cudaMalloc(&err, 4) != cudaSuccess) return NSFV1_ERR_CUDA;
    cudaStream_t s = (cudaStream_t)stream;
    cudaMemsetAsync(err, 0, 4, s);
    std::string why;
    const int used = gemm_bf16((const bf16*)A, (const bf16*)B, C, M, N, K, splits, err, s, why);
    if (used < 0) return NSFV1_ERR_ARGUMENT;
    int h = 0;
    if (cudaMemcpyAsync(&h, err, 4, cudaMemcpyDeviceToHost, s) != cudaSuccess || cudaStreamSynchronize(s) != cudaSuccess)
        return NSFV1_ERR_CUDA;
    return h ? NSFV1_ERR_TIMEOUT : NSFV1_OK;
}

int nsfv1_gemm_bf16_splits(int K, int splits) {
    if (K <= 0 || K % 64 || splits < 1) return 0;
    const int kTiles = K / 64;
    splits = std::min(splits, kTiles);
    const int chunkTiles = (kTiles + splits - 1) / splits;
    return (kTiles + chunkTiles - 1) / chunkTiles;
}

}  // extern "C"
