// Many independent instances (e.g. lid-driven cavities of uneven size) solved
// together: the instances are disjoint node ranges of one mesh, assembled by
// the colour kernels in one pass (per-element viscosity, converged instances
// skipped), and every Newton step runs ONE persistent launch of a
// cluster-per-instance restarted GMRES (right point-block-Jacobi
// preconditioning): each thread-block cluster takes instances from a queue
// (largest first), keeps the Hessenberg state in the shared memory of every
// CTA of the cluster (computed redundantly, so no broadcast is needed), and
// reduces dot products over the cluster through distributed shared memory in a
// fixed order. Cluster barriers are hardware barriers; the kernel has no
// spin-wait. Results do not depend on which cluster runs an instance.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <numeric>
#include <vector>
#include <cooperative_groups.h>
#include "nsfv1_internal.h"
#include "nsfv1_host.h"
#include "nsfv1_linalg.cuh"
#include "../../include/nsfv1_gb300.h"

namespace cg = cooperative_groups;

namespace nsfv1 {

static constexpr int kGT = 512;      // threads per CTA of the GMRES kernel (16 warps per SM hide the latency of the instance-local loops)
static constexpr int kMaxM = 32;     // largest restart length
static constexpr int kWarps = kGT / 32;

static constexpr int kMaxLevels = 8;
static constexpr int64_t kLocalRows = 289;   // multigrid levels up to 16 x 16 cells run on one CTA

// one level of the geometric multigrid hierarchy (level 0 = the fine mesh)
template <typename VT>
struct MgLevel {
    const int32_t* rowPtr;
    const int32_t* colIdx;
    const VT* vals;
    const VT* Dinv;
    const int32_t* node0;   // [nInst] first node of each instance on this level, -1 if absent
    const uint8_t* mask;    // [dofs] 1 = free row, 0 = Dirichlet row
    VT* x;                  // level correction
    VT* r;                  // level right-hand side
    VT* s;                  // residual scratch
    VT* x2;                 // second correction buffer (smoother sweeps alternate between x and x2)
};

template <typename VT>
struct MgArgs {
    int nLevels;            // 0: point-block Jacobi preconditioner
    const int32_t* cells0;  // [nInst] cells per side on level 0
    int nu;                 // pre/post smoothing sweeps
    int nuCoarse;           // sweeps on the coarsest level
    double omega;           // damping of the point-block Jacobi smoother
    MgLevel<VT> lv[kMaxLevels];
};

template <typename VT>
struct GmresBatchArgs {
    const int32_t* queue;      // instance ids, largest first
    int nQueue;
    int* head;                 // queue position (zeroed before the launch)
    const int32_t* instNode0;  // [nInst + 1] node ranges
    const int32_t* rowPtr;
    const int32_t* colIdx;
    const VT* vals;
    const VT* Dinv;            // inverted diagonal blocks
    const double* rhs;         // FP64 right-hand side (the defect)
    VT* x;                     // solution
    VT* V;                     // basis [m + 1][nTot]
    VT* t;                     // preconditioned vector [nTot]
    int64_t nTot;
    int m;
    double rtol;
    int maxit;
    int* itersOut;
    double* relresOut;
    VT* q;                     // extra vector [nTot] (V y before the final preconditioning)
    MgArgs<VT> mg;
    const int* nQueueDev;      // if set: queue length read from device memory (graph replays)
    const double* rtolInst;    // if set: per-instance relative tolerance (adaptive forcing)
};

// warp-level part of a reduction: the warp sum of v goes to wred[warp][k]
struct ClusterRed {
    __device__ __forceinline__ static void block_part(double v, int k, double (*wred)[kMaxM + 2]) {
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
        if ((threadIdx.x & 31) == 0) wred[threadIdx.x >> 5][k] = v;
    }
};

// acc += the block row [q0, q1) of (vals, colIdx) applied to x (x indexed by
// global column minus xoff): lane takes blocks lane, lane+G, ...; one fused
// multiply-add per matrix entry
template <typename VT, int b, int G>
__device__ __forceinline__ void block_row_acc(const VT* __restrict__ vals, const int32_t* __restrict__ colIdx, int64_t q0, int64_t q1,
                                              int lane, const VT* __restrict__ x, int64_t xoff, VT (&acc)[b]) {
    for (int64_t q = q0 + lane; q < q1; q += G) {
        const VT* blk = vals + q * (b * b);
        const VT* xc = x + (int64_t)colIdx[q] * b - xoff;
        VT xv[b];
#pragma unroll
        for (int j = 0; j < b; ++j) xv[j] = xc[j];
#pragma unroll
        for (int i = 0; i < b; ++i)
#pragma unroll
            for (int j = 0; j < b; ++j) acc[i] = fma(blk[i * b + j], xv[j], acc[i]);
    }
}

// rows [0, nn) of a block-CSR slice (global row = row0 + local row), U rows per
// lane group and trip: the row pointers, column indices, blocks and x entries of
// U rows (two blocks per lane unrolled, predicated) are all requested before the
// first is used, so each trip pays one memory latency instead of U; longer rows
// finish in a remainder loop. epi(local row, component c, acc) runs on lane c < b
// of the group with the row sums (spreading the epilogue over b lanes).
template <typename VT, int b, int G, int U, typename Epi>
__device__ __forceinline__ void rows_spmv(const int32_t* __restrict__ rowPtr, const int32_t* __restrict__ colIdx,
                                          const VT* __restrict__ vals, int64_t row0, int64_t nn, const VT* __restrict__ xin,
                                          int64_t xoff, int ctid, int cth, Epi&& epi) {
    constexpr int KB = 2;
    const int lane = ctid % G;
    const int64_t groups = cth / G;
    const int64_t per = groups * U;
    const int64_t trips = (nn + per - 1) / per;
    for (int64_t it = 0; it < trips; ++it) {
        int64_t q0[U], q1[U];
        VT acc[U][b];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int64_t lr = ctid / G + (it * U + u) * groups;
            const bool valid = lr < nn;
            q0[u] = valid ? rowPtr[row0 + lr] : 0;
            q1[u] = valid ? rowPtr[row0 + lr + 1] : 0;
#pragma unroll
            for (int i = 0; i < b; ++i) acc[u][i] = VT(0);
        }
#pragma unroll
        for (int k = 0; k < KB; ++k)
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const int64_t q = q0[u] + lane + k * G;
                if (q < q1[u]) {
                    const VT* blk = vals + q * (b * b);
                    const VT* xc = xin + (int64_t)colIdx[q] * b - xoff;
                    VT xv[b];
#pragma unroll
                    for (int j = 0; j < b; ++j) xv[j] = xc[j];
#pragma unroll
                    for (int i = 0; i < b; ++i)
#pragma unroll
                        for (int j = 0; j < b; ++j) acc[u][i] = fma(blk[i * b + j], xv[j], acc[u][i]);
                }
            }
#pragma unroll
        for (int u = 0; u < U; ++u)
            if (q1[u] - q0[u] > KB * G) block_row_acc<VT, b, G>(vals, colIdx, q0[u] + KB * G, q1[u], lane, xin, xoff, acc[u]);
#pragma unroll
        for (int u = 0; u < U; ++u) {
            // butterfly: every lane of the group gets the row sums; lane c < b handles component c
#pragma unroll
            for (int off = G / 2; off > 0; off >>= 1)
#pragma unroll
                for (int r = 0; r < b; ++r) acc[u][r] += __shfl_xor_sync(0xffffffffu, acc[u][r], off, G);
            const int64_t lr = ctid / G + (it * U + u) * groups;
            if (lr < nn && lane < b) epi(lr, lane, acc[u]);
        }
    }
}

template <typename VT, int b, int G>
__global__ void __launch_bounds__(kGT) k_gmres_batch(const GmresBatchArgs<VT> A) {
    cg::cluster_group cl = cg::this_cluster();
    const int crank = (int)cl.block_rank();
    const int csize = (int)cl.num_blocks();
    __shared__ double wred[kWarps][kMaxM + 2];
    __shared__ double red[kMaxM + 2];
    __shared__ double sum[kMaxM + 2];
    __shared__ double H[(kMaxM + 1) * kMaxM];
    __shared__ double hcol[kMaxM + 2];
    __shared__ double cs[kMaxM], sn[kMaxM], gvec[kMaxM + 1], yv[kMaxM];
    __shared__ int s_item;
    const int tid = threadIdx.x;
    const int ctid = crank * kGT + tid;
    const int cth = csize * kGT;
    const int m = A.m;
    const int nQueue = A.nQueueDev ? *A.nQueueDev : A.nQueue;

    // sum over the cluster of K values that each thread deposited in wred[warp][k]
    auto cluster_sum = [&](int K) {
        __syncthreads();
        if (tid < K) {
            double s = 0.0;
#pragma unroll
            for (int w = 0; w < kWarps; ++w) s += wred[w][tid];
            red[tid] = s;
        }
        cl.sync();
        if (tid < K) {
            double s = 0.0;
            for (int r = 0; r < csize; ++r) s += cl.map_shared_rank(red, r)[tid];
            sum[tid] = s;
        }
        cl.sync();   // red may be reused afterwards; sum is visible to this CTA
    };

    for (;;) {
        if (crank == 0 && tid == 0) s_item = atomicAdd(A.head, 1);
        cl.sync();
        const int item = *cl.map_shared_rank(&s_item, 0);
        cl.sync();
        if (item >= nQueue) break;
        const int inst = A.queue[item];
        const double rtol = A.rtolInst ? A.rtolInst[inst] : A.rtol;
        const int64_t node0 = A.instNode0[inst], nNode = A.instNode0[inst + 1] - node0;
        const int64_t o = node0 * b, n = nNode * b;
        VT* __restrict__ x = A.x + o;
        const double* __restrict__ rhs = A.rhs + o;
        auto Vk = [&](int k) { return A.V + (int64_t)k * A.nTot + o; };
        VT* __restrict__ t = A.t + o;
        const VT* __restrict__ Dinv = A.Dinv + node0 * b * b;

        // y = M t  (rows of this instance; G lanes per block row, uniform trip count)
        auto spmv = [&](const VT* __restrict__ xin, VT* __restrict__ yout) {
            rows_spmv<VT, b, G, 4>(A.rowPtr, A.colIdx, A.vals, node0, nNode, xin, o, ctid, cth, [&](int64_t lr, int c, const VT (&acc)[b]) {
                VT v = acc[0];
#pragma unroll
                for (int r = 1; r < b; ++r) v = (c == r) ? acc[r] : v;
                yout[lr * b + c] = v;
            });
        };
        // point-block Jacobi: out = Dm (in) (per node, optionally damped / accumulated)
        // coarse multigrid levels run on CTA 0 alone with block barriers ("local"
        // mode); everything else on the whole cluster with cluster barriers
        bool loc = false;
        auto me = [&]() { return loc ? tid : ctid; };
        auto nth = [&]() { return loc ? kGT : cth; };
        auto bar = [&]() {
            if (loc) __syncthreads();
            else cl.sync();
        };
        auto jacobi = [&](const VT* __restrict__ Dm, int64_t nn, const VT* __restrict__ in, VT* __restrict__ out, VT w, bool accumulate) {
            const int64_t t0 = me(), tn = nth();
#pragma unroll 2
            for (int64_t nd = t0; nd < nn; nd += tn) {
                VT xi[b];
#pragma unroll
                for (int j = 0; j < b; ++j) xi[j] = in[nd * b + j];
#pragma unroll
                for (int i = 0; i < b; ++i) {
                    VT a = VT(0);
#pragma unroll
                    for (int j = 0; j < b; ++j) a += Dm[nd * b * b + i * b + j] * xi[j];
                    out[nd * b + i] = accumulate ? out[nd * b + i] + w * a : w * a;
                }
            }
        };
        // level SpMV with residual epilogue: res = rhs - M_l x  (rhs == nullptr: res = M_l x)
        auto lspmv = [&](const MgLevel<VT>& L, int64_t n0, int64_t nn, const VT* __restrict__ xin, const VT* __restrict__ rhsl,
                         VT* __restrict__ res) {
            rows_spmv<VT, b, G, 4>(L.rowPtr, L.colIdx, L.vals, n0, nn, xin, n0 * b, me(), nth(), [&](int64_t lr, int c, const VT (&acc)[b]) {
                VT v = acc[0];
#pragma unroll
                for (int r = 1; r < b; ++r) v = (c == r) ? acc[r] : v;
                res[lr * b + c] = rhsl ? rhsl[lr * b + c] - v : v;
            });
        };
        // instance levels: cells per side, first node on each level
        const int nLev = A.mg.nLevels;
        int myLev = 0;
        int64_t ln0[kMaxLevels];
        int lcell[kMaxLevels];
        for (int l = 0; l < nLev; ++l) {
            const int32_t v = A.mg.lv[l].node0[inst];
            if (v < 0) break;
            ln0[l] = v;
            lcell[l] = A.mg.cells0[inst] >> l;
            myLev = l + 1;
        }
        // V-cycle: out = M^-1 in on level 0 (in/out instance-local); point-block
        // Jacobi when the instance has no coarse level
        auto precond = [&](const VT* __restrict__ in, VT* __restrict__ out) {
            if (myLev <= 1) { jacobi(Dinv, nNode, in, out, VT(1), false); return; }
            const VT om = (VT)A.mg.omega;
            // the correction of each level lives in one of two buffers; a smoother sweep
            // reads the current one and writes the other
            auto prim = [&](int l) { return l == 0 ? out : A.mg.lv[l].x + ln0[l] * b; };
            auto sec = [&](int l) { return A.mg.lv[l].x2 + ln0[l] * b; };
            bool inSec[kMaxLevels];
#pragma unroll 1
            for (int l = 0; l < kMaxLevels; ++l) inSec[l] = false;
            auto lx = [&](int l) { return inSec[l] ? sec(l) : prim(l); };
            auto lr = [&](int l) { return l == 0 ? in : (const VT*)(A.mg.lv[l].r + ln0[l] * b); };
            auto ls = [&](int l) { return A.mg.lv[l].s + ln0[l] * b; };
            auto lD = [&](int l) { return A.mg.lv[l].Dinv + ln0[l] * b * b; };
            auto lnn = [&](int l) { return (int64_t)(lcell[l] + 1) * (lcell[l] + 1); };
            // one damped point-block Jacobi sweep in a single pass:
            //   x_new = x + omega Dinv (r - M x)    (row-local; neighbours read from x)
            auto fsweep = [&](int l) {
                const MgLevel<VT>& L = A.mg.lv[l];
                const VT* xc = lx(l);
                VT* xn = inSec[l] ? prim(l) : sec(l);
                const VT* rl = lr(l);
                const VT* Dm = lD(l);
                rows_spmv<VT, b, G, 4>(L.rowPtr, L.colIdx, L.vals, ln0[l], lnn(l), xc, ln0[l] * b, me(), nth(),
                                       [&](int64_t r0, int c, const VT (&acc)[b]) {
                                           VT sv[b];
#pragma unroll
                                           for (int j = 0; j < b; ++j) sv[j] = rl[r0 * b + j] - acc[j];
                                           VT a = VT(0);
#pragma unroll
                                           for (int j = 0; j < b; ++j) a += Dm[r0 * b * b + c * b + j] * sv[j];
                                           xn[r0 * b + c] = xc[r0 * b + c] + om * a;
                                       });
                inSec[l] = !inSec[l];
                bar();
            };
            // pre-smoothing on level l, then (above the coarsest) residual and restriction into l + 1
            auto down = [&](int l) {
                const MgLevel<VT>& L = A.mg.lv[l];
                const int64_t nn = lnn(l);
                const int sweeps = (l == myLev - 1) ? A.mg.nuCoarse : A.mg.nu;
                jacobi(lD(l), nn, lr(l), lx(l), om, false);
                bar();
                for (int k = 1; k < sweeps; ++k) fsweep(l);
                if (l == myLev - 1) return;
                lspmv(L, ln0[l], nn, lx(l), lr(l), ls(l));
                bar();
                // restriction (transpose of bilinear interpolation), masked on both levels
                const int nf = lcell[l], nc = lcell[l + 1];
                const int64_t mf = nf + 1, mc = nc + 1;
                const uint8_t* mkf = L.mask + ln0[l] * b;
                const uint8_t* mkc = A.mg.lv[l + 1].mask + ln0[l + 1] * b;
                VT* rc = A.mg.lv[l + 1].r + ln0[l + 1] * b;
                const VT* sf = ls(l);
                for (int64_t c = me(); c < mc * mc; c += nth()) {
                    const int64_t I = c % mc, J = c / mc;
                    VT acc[b];
#pragma unroll
                    for (int f = 0; f < b; ++f) acc[f] = VT(0);
#pragma unroll
                    for (int dj = -1; dj <= 1; ++dj)
#pragma unroll
                        for (int di = -1; di <= 1; ++di) {
                            const int64_t fi = 2 * I + di, fj = 2 * J + dj;
                            if (fi < 0 || fj < 0 || fi >= mf || fj >= mf) continue;
                            const VT w = (di == 0 ? VT(1) : VT(0.5)) * (dj == 0 ? VT(1) : VT(0.5));
                            const int64_t fn = fj * mf + fi;
#pragma unroll
                            for (int f = 0; f < b; ++f)
                                if (mkf[fn * b + f]) acc[f] += w * sf[fn * b + f];
                        }
#pragma unroll
                    for (int f = 0; f < b; ++f) rc[c * b + f] = mkc[c * b + f] ? acc[f] : VT(0);
                }
                bar();
            };
            // prolongation of the correction of level l + 1 into level l, then post-smoothing on l
            auto up = [&](int l) {
                const MgLevel<VT>& L = A.mg.lv[l];
                const int64_t nn = lnn(l);
                const int nf = lcell[l];
                const int64_t mf = nf + 1, mc = lcell[l + 1] + 1;
                const uint8_t* mkf = L.mask + ln0[l] * b;
                const VT* xc = lx(l + 1);
                VT* xf = lx(l);
                for (int64_t fnode = me(); fnode < mf * mf; fnode += nth()) {
                    const int64_t I = fnode % mf, J = fnode / mf;
                    const int64_t i0 = I / 2, j0 = J / 2;
                    const int64_t i1 = (I & 1) ? i0 + 1 : i0, j1 = (J & 1) ? j0 + 1 : j0;
                    const VT wi = (I & 1) ? VT(0.5) : VT(1), wj = (J & 1) ? VT(0.5) : VT(1);
#pragma unroll
                    for (int f = 0; f < b; ++f) {
                        VT v = wi * wj * xc[(j0 * mc + i0) * b + f];
                        if (I & 1) v += wi * wj * xc[(j0 * mc + i1) * b + f];
                        if (J & 1) v += wi * wj * xc[(j1 * mc + i0) * b + f];
                        if ((I & 1) && (J & 1)) v += wi * wj * xc[(j1 * mc + i1) * b + f];
                        if (mkf[fnode * b + f]) xf[fnode * b + f] += v;
                    }
                }
                bar();
                for (int k = 0; k < A.mg.nu; ++k) fsweep(l);
                (void)nn;
            };
            // the first level (below the instance's own) with at most kLocalRows nodes starts the
            // part of the cycle that CTA 0 runs alone
            int lsm = myLev;
            for (int l = 1; l < myLev; ++l)
                if (lnn(l) <= kLocalRows) { lsm = l; break; }
            for (int l = 0; l < lsm; ++l) down(l);
            if (lsm < myLev) {
                if (crank == 0) {
                    loc = true;
                    for (int l = lsm; l < myLev; ++l) down(l);
                    for (int l = myLev - 2; l >= lsm; --l) up(l);
                    loc = false;
                }
                cl.sync();
                // which buffer holds level lsm's correction now (every CTA agrees; CTA 0 got
                // there by running the sweeps: sweeps - 1 fused ones down, nu up)
                const int sw = (lsm == myLev - 1) ? A.mg.nuCoarse : A.mg.nu;
                inSec[lsm] = (((sw - 1) + (lsm < myLev - 1 ? A.mg.nu : 0)) & 1) != 0;
            }
            for (int l = min(lsm, myLev - 1) - 1; l >= 0; --l) up(l);
            if (inSec[0]) {
                const VT* src = sec(0);
#pragma unroll 4
                for (int64_t e = ctid; e < n; e += cth) out[e] = src[e];
            }
        };
        // ||v||^2 over the cluster
        auto norm2 = [&](const VT* __restrict__ v) {
            VT acc = VT(0);
            for (int64_t e = ctid; e < n; e += cth) acc += v[e] * v[e];
            ClusterRed::block_part((double)acc, 0, wred);
            cluster_sum(1);
            return sum[0];
        };

        // r0 = rhs (x0 = 0)
        VT* v0 = Vk(0);
        for (int64_t e = ctid; e < n; e += cth) { v0[e] = (VT)rhs[e]; x[e] = VT(0); }
        cl.sync();
        double beta = sqrt(norm2(v0));
        const double beta0 = beta;
        double relres = 0.0;
        int total = 0;
        if (beta0 > 0.0 && isfinite(beta0)) {
            relres = 1.0;
            for (;;) {
                const VT ib = (VT)(1.0 / beta);
                for (int64_t e = ctid; e < n; e += cth) v0[e] *= ib;
                if (tid == 0) { gvec[0] = beta; for (int k = 1; k <= m; ++k) gvec[k] = 0.0; }
                cl.sync();
                int j = 0;
                bool done = false;
                for (; j < m && total < A.maxit; ++j) {
                    ++total;
                    precond(Vk(j), t);
                    cl.sync();
                    VT* w = Vk(j + 1);
                    spmv(t, w);
                    cl.sync();
                    if (tid <= j) hcol[tid] = 0.0;
                    // classical Gram-Schmidt, two passes
                    for (int pass = 0; pass < 2; ++pass) {
                        // four basis vectors per pass over w (each dot keeps its own
                        // summation order, so the results do not change)
                        for (int k0 = 0; k0 <= j; k0 += 4) {
                            const int nk = min(4, j + 1 - k0);
                            const VT* v0k = Vk(k0);
                            const VT* v1k = Vk(min(k0 + 1, j));
                            const VT* v2k = Vk(min(k0 + 2, j));
                            const VT* v3k = Vk(min(k0 + 3, j));
                            VT a0 = VT(0), a1 = VT(0), a2 = VT(0), a3 = VT(0);
#pragma unroll 2
                            for (int64_t e = ctid; e < n; e += cth) {
                                const VT we = w[e];
                                a0 += v0k[e] * we;
                                if (nk > 1) a1 += v1k[e] * we;
                                if (nk > 2) a2 += v2k[e] * we;
                                if (nk > 3) a3 += v3k[e] * we;
                            }
                            ClusterRed::block_part((double)a0, k0, wred);
                            if (nk > 1) ClusterRed::block_part((double)a1, k0 + 1, wred);
                            if (nk > 2) ClusterRed::block_part((double)a2, k0 + 2, wred);
                            if (nk > 3) ClusterRed::block_part((double)a3, k0 + 3, wred);
                        }
                        cluster_sum(j + 1);
                        if (tid <= j) hcol[tid] += sum[tid];
                        // the second pass also sums ||w||^2 of the result (norm2's order: each
                        // thread its own entries in turn, then the cluster sum)
                        VT nacc = VT(0);
#pragma unroll 2
                        for (int64_t e = ctid; e < n; e += cth) {
                            VT a = w[e];
                            for (int k = 0; k <= j; ++k) a -= (VT)sum[k] * Vk(k)[e];
                            w[e] = a;
                            if (pass == 1) nacc += a * a;
                        }
                        if (pass == 0) {
                            cl.sync();
                        } else {
                            ClusterRed::block_part((double)nacc, 0, wred);
                            cluster_sum(1);
                        }
                    }
                    const double hn = sqrt(sum[0]);
                    if (hn > 0.0) {
                        const VT ih = (VT)(1.0 / hn);
                        for (int64_t e = ctid; e < n; e += cth) w[e] *= ih;
                    }
                    // Givens rotations (redundantly in every CTA; thread 0)
                    if (tid == 0) {
                        hcol[j + 1] = hn;
                        for (int k = 0; k < j; ++k) {
                            const double a = hcol[k], c = hcol[k + 1];
                            hcol[k] = cs[k] * a + sn[k] * c;
                            hcol[k + 1] = -sn[k] * a + cs[k] * c;
                        }
                        const double a = hcol[j], c = hcol[j + 1];
                        const double rr = sqrt(a * a + c * c);
                        cs[j] = rr > 0.0 ? a / rr : 1.0;
                        sn[j] = rr > 0.0 ? c / rr : 0.0;
                        hcol[j] = rr;
                        gvec[j + 1] = -sn[j] * gvec[j];
                        gvec[j] = cs[j] * gvec[j];
                        for (int k = 0; k <= j; ++k) H[k * kMaxM + j] = hcol[k];
                        red[kMaxM + 1] = fabs(gvec[j + 1]) / beta0;   // scratch slot for the estimate
                    }
                    cl.sync();
                    relres = red[kMaxM + 1];
                    if (!(relres >= rtol) || hn == 0.0) { ++j; done = true; break; }   // converged (or NaN: stop)
                }
                // y = H^-1 g ; x += Dinv (V y)
                if (tid == 0) {
                    for (int k = j - 1; k >= 0; --k) {
                        double acc = gvec[k];
                        for (int q = k + 1; q < j; ++q) acc -= H[k * kMaxM + q] * yv[q];
                        yv[k] = (H[k * kMaxM + k] != 0.0) ? acc / H[k * kMaxM + k] : 0.0;
                    }
                }
                __syncthreads();
                VT* qv = A.q + o;
                for (int64_t e = ctid; e < n; e += cth) {
                    VT a = VT(0);
                    for (int k = 0; k < j; ++k) a += (VT)yv[k] * Vk(k)[e];
                    qv[e] = a;
                }
                cl.sync();
                precond(qv, t);
                cl.sync();
                for (int64_t e = ctid; e < n; e += cth) x[e] += t[e];
                cl.sync();
                if (done || total >= A.maxit || !isfinite(relres)) break;
                // restart: V_0 = rhs - M x
                spmv(x, v0);
                cl.sync();
                for (int64_t e = ctid; e < n; e += cth) v0[e] = (VT)(rhs[e] - (double)v0[e]);
                cl.sync();
                beta = sqrt(norm2(v0));
                relres = beta / beta0;
                if (!(relres >= rtol) || beta == 0.0) break;
            }
        }
        if (crank == 0 && tid == 0) { A.itersOut[inst] = total; A.relresOut[inst] = relres; }
        cl.sync();
    }
}

// ---- small batch kernels ----------------------------------------------------------

// per-instance ||v||^2 over its node range (one CTA per instance, fixed order)
__global__ void __launch_bounds__(256) k_inst_norm2(const int32_t* __restrict__ instNode0, int b, const double* __restrict__ v,
                                                    double* __restrict__ out) {
    __shared__ double sh[256];
    const int inst = blockIdx.x;
    const int64_t e0 = (int64_t)instNode0[inst] * b, e1 = (int64_t)instNode0[inst + 1] * b;
    double acc = 0.0;
    for (int64_t e = e0 + threadIdx.x; e < e1; e += 256) acc += v[e] * v[e];
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (int s = 128; s > 0; s >>= 1) {
        if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[inst] = sh[0];
}

// point-block Jacobi setup for the nodes of active instances
template <typename VT, int b>
__global__ void k_block_inv_active(int64_t nRows, const int32_t* __restrict__ diagPos, const int32_t* __restrict__ nodeInst,
                                   const int32_t* __restrict__ active, const VT* __restrict__ vals, VT* __restrict__ Dinv, int* err) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nRows || !active[nodeInst[r]]) return;
    if (!block_inverse<b>(vals + (int64_t)diagPos[r] * b * b, Dinv + r * b * b)) atomicOr(err, 2);
}

template <typename VT, int b>
__global__ void k_block_inv_all(int64_t nRows, const int32_t* __restrict__ diagPos, const VT* __restrict__ vals, VT* __restrict__ Dinv, int* err) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nRows) return;
    if (!block_inverse<b>(vals + (int64_t)diagPos[r] * b * b, Dinv + r * b * b)) atomicOr(err, 2);
}

// trial iterate: ut = u - lambda[inst] du on the nodes of pending instances
template <typename VT>
__global__ void k_batch_trial(int64_t n, int b, const int32_t* __restrict__ nodeInst, const int32_t* __restrict__ pending,
                              const double* __restrict__ lambda, const double* __restrict__ u, const VT* __restrict__ du,
                              double* __restrict__ ut) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n) return;
    const int inst = nodeInst[e / b];
    if (pending[inst]) ut[e] = u[e] - lambda[inst] * (double)du[e];
}

// state of a coarse level: u_c[node] = u_f[inj[node]]
__global__ void k_inject(int64_t nc, int b, const int32_t* __restrict__ inj, const double* __restrict__ uf, double* __restrict__ uc) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e < nc * b) uc[e] = uf[(int64_t)inj[e / b] * b + e % b];
}

// copy the rows of flagged instances: dst[e] = src[e]
__global__ void k_batch_copy(int64_t n, int b, const int32_t* __restrict__ nodeInst, const int32_t* __restrict__ flag,
                             const double* __restrict__ src, double* __restrict__ dst) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e < n && flag[nodeInst[e / b]]) dst[e] = src[e];
}

template <typename VT, int b>
static cudaError_t launch_gmres_batch(const GmresBatchArgs<VT>& a, int clusterSize, int nClusters, cudaStream_t s) {
    constexpr int G = (b == 4) ? 16 : 8;
    auto kern = k_gmres_batch<VT, b, G>;
    if (clusterSize > 8) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
        if (e != cudaSuccess) return e;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(clusterSize * nClusters, 1, 1);
    cfg.blockDim = dim3(kGT, 1, 1);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = clusterSize;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kern, a);
}

// most clusters of this size that can be resident at once
template <typename VT, int b>
static int max_clusters(int clusterSize) {
    constexpr int G = (b == 4) ? 16 : 8;
    auto kern = k_gmres_batch<VT, b, G>;
    if (clusterSize > 8) cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(clusterSize, 1, 1);
    cfg.blockDim = dim3(kGT, 1, 1);
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = clusterSize;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int n = 0;
    if (cudaOccupancyMaxActiveClusters(&n, kern, &cfg) != cudaSuccess || n <= 0) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

// ---- the batched Newton driver -----------------------------------------------------

struct BatchWs {
    int prec = -1, m = 0, nInst = 0;
    int64_t n = 0, nnzb = 0;   // every buffer is sized by (prec, n, m, nInst, nnzb)
    double *D = nullptr, *Dt = nullptr, *Ut = nullptr, *nrm = nullptr, *lambda = nullptr, *relres = nullptr;
    void *J = nullptr, *Dinv = nullptr, *V = nullptr, *t = nullptr, *x = nullptr, *q = nullptr, *s = nullptr, *x2 = nullptr;
    int32_t *queue = nullptr, *head = nullptr, *pending = nullptr, *accepted = nullptr, *iters = nullptr, *nQueue = nullptr;
    double* rtolInst = nullptr;
    ~BatchWs() { release(); }
    void release() {
        auto f = [](auto*& p) { if (p) cudaFree((void*)p); p = nullptr; };
        f(D); f(Dt); f(Ut); f(nrm); f(lambda); f(relres); f(J); f(Dinv); f(V); f(t); f(x); f(q); f(s); f(x2);
        f(queue); f(head); f(pending); f(accepted); f(iters); f(nQueue); f(rtolInst);
        prec = -1;
    }
};

}  // namespace nsfv1

using namespace nsfv1;

namespace {
struct BatchState;
}

namespace nsfv1 {
void batch_free(void* p);
}

namespace {

// a coarse level of the structured-instance hierarchy
struct Level {
    Disc* disc = nullptr;          // the level mesh (all instances that have this level)
    std::vector<int32_t> node0;    // [nInst] first node of each instance on this level, -1 if absent
    int32_t* d_node0 = nullptr;
    int32_t* d_inj = nullptr;      // [level nodes] node of the next finer level at the same point
    uint8_t* d_mask = nullptr;     // [level dofs] 1 = free row
    double* d_u = nullptr;         // injected state
    void *J = nullptr, *Dinv = nullptr, *x = nullptr, *r = nullptr, *s = nullptr, *x2 = nullptr;
    int prec = -1;
    void release() {
        auto f = [](auto*& p) { if (p) cudaFree((void*)p); p = nullptr; };
        f(d_node0); f(d_inj); f(d_mask); f(d_u); f(J); f(Dinv); f(x); f(r); f(s); f(x2);
        delete disc; disc = nullptr;
        prec = -1;
    }
};

struct BatchState {
    BatchWs ws;
    std::vector<Level> levels;     // levels[0] unused (the handle's own mesh); levels[l], l >= 1
    uint8_t* d_mask0 = nullptr;    // Dirichlet mask of the fine level
    int32_t* d_cells = nullptr;    // [nInst] cells per side
    // CUDA graph of one Newton step's fixed device work (Jacobians, block inverses, GMRES launch)
    cudaStream_t gs = nullptr;
    cudaEvent_t evIn = nullptr, evOut = nullptr;
    std::vector<std::pair<int, cudaGraphExec_t>> graphs;   // one per cluster size in use
    // timing of the last solve (ms): [steps, step work (Jacobians + GMRES), line search, wall]
    double stats[8] = {0};
    ~BatchState() {
        clear_levels();
        drop_graph();
        if (evIn) cudaEventDestroy(evIn);
        if (evOut) cudaEventDestroy(evOut);
        if (gs) cudaStreamDestroy(gs);
    }
    void drop_graph() {
        for (auto& g : graphs) cudaGraphExecDestroy(g.second);
        graphs.clear();
    }
    cudaGraphExec_t* graph_for(int cs) {
        for (auto& g : graphs) if (g.first == cs) return &g.second;
        return nullptr;
    }
    void clear_levels() {
        for (auto& L : levels) L.release();
        levels.clear();
        if (d_mask0) cudaFree(d_mask0);
        if (d_cells) cudaFree(d_cells);
        d_mask0 = nullptr; d_cells = nullptr;
    }
};

BatchState* batch_state(Disc& D) {
    if (!D.batch) D.batch = new BatchState();
    return static_cast<BatchState*>(D.batch);
}

// Eisenstat-Walker forcing term ("choice 2", gamma 0.9, alpha 2) with the usual
// safeguards: no sharp decrease while the previous term was large, at most
// etaMax, at least etaMin, and no oversolving below half the remaining distance
// to the Newton target.
double ew_forcing(double nd, double ndPrev, double etaPrev, double etaMin, double etaMax, double target) {
    const double gamma = 0.9;
    double eta = gamma * (nd / ndPrev) * (nd / ndPrev);
    const double keep = gamma * etaPrev * etaPrev;
    if (keep > 0.1) eta = std::max(eta, keep);
    eta = std::min(eta, etaMax);
    eta = std::max(eta, 0.5 * target / nd);
    eta = std::min(eta, etaMax);
    return std::max(eta, etaMin);
}

template <typename VT>
int batched_newton(Disc& D, double* u, const double* u_old, double dt, const nsfv1_newton_params& p, const nsfv1_batch_options& opt,
                   nsfv1_newton_result* res, cudaStream_t s) {
    const int b = D.dim + 1;
    const int nInst = D.nInst;
    const int64_t n = D.nNodes * b;
    const int prec = std::is_same<VT, double>::value ? NSFV1_F64 : NSFV1_F32;
    const int m = std::min(std::max(p.gmres_restart, 2), kMaxM);
    BatchState* BS = batch_state(D);
    BatchWs& W = BS->ws;
    BS->drop_graph();
    for (double& x : BS->stats) x = 0.0;
    const auto wall0 = std::chrono::steady_clock::now();
    struct Ev {
        cudaEvent_t e = nullptr;
        Ev() { cudaEventCreate(&e); }
        ~Ev() { if (e) cudaEventDestroy(e); }
    } eA, eB, eC;
    cudaEvent_t evA = eA.e, evB = eB.e, evC = eC.e;
    const int64_t nnzb = (int64_t)D.colIdx.size();
    if (W.prec != prec || W.n != n || W.m != m || W.nInst != nInst || W.nnzb != nnzb) {
        W.release();
        const size_t vt = sizeof(VT);
        auto al = [&](auto*& ptr, size_t bytes) { return D.cuda_ok(cudaMalloc((void**)&ptr, bytes), "batch workspace"); };
        if (!al(W.D, n * 8) || !al(W.Dt, n * 8) || !al(W.Ut, n * 8) || !al(W.nrm, nInst * 8) || !al(W.lambda, nInst * 8) ||
            !al(W.relres, nInst * 8) || !al(W.J, D.colIdx.size() * b * b * vt) || !al(W.Dinv, (size_t)D.nNodes * b * b * vt) ||
            !al(W.V, (size_t)(m + 1) * n * vt) || !al(W.t, n * vt) || !al(W.x, n * vt) || !al(W.q, n * vt) || !al(W.s, n * vt) ||
            !al(W.x2, n * vt) ||
            !al(W.queue, nInst * 4) || !al(W.head, 4) || !al(W.nQueue, 4) || !al(W.rtolInst, nInst * 8) ||
            !al(W.pending, nInst * 4) || !al(W.accepted, nInst * 4) || !al(W.iters, nInst * 4))
            return D.status;
        W.prec = prec; W.n = n; W.m = m; W.nInst = nInst; W.nnzb = nnzb;
    }
    const int baseCluster = opt.cluster_size > 0 ? opt.cluster_size : 4;
    int numSMs = 0;
    {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&numSMs, cudaDevAttrMultiProcessorCount, dev);
    }
    // resident clusters per cluster size (computed on first use)
    int clustersFor[17] = {0};
    auto clusters_of = [&](int cs) {
        if (!clustersFor[cs]) {
            int nc = (b == 4) ? max_clusters<VT, 4>(cs) : max_clusters<VT, 3>(cs);
            if (opt.max_clusters > 0) nc = std::min(nc, opt.max_clusters);
            clustersFor[cs] = std::min(std::max(nc, 0), nInst);
        }
        return clustersFor[cs];
    };
    if (clusters_of(baseCluster) <= 0) { D.fail(NSFV1_ERR_ARGUMENT, "batched solve: cluster size not launchable"); return D.status; }
    int clusterSize = baseCluster, nClusters = clusters_of(baseCluster);
    const bool useMG = opt.mg_levels != 0 && BS->levels.size() > 1;
    const bool adaptive = opt.forcing_max > 0.0;
    const bool useGraph = opt.graph != 0;

    // coarse-level buffers of this precision (before any graph capture)
    if (useMG) {
        for (size_t l = 1; l < BS->levels.size(); ++l) {
            Level& L = BS->levels[l];
            if (L.prec == prec) continue;
            Disc& C = *L.disc;
            const int64_t nc = C.nNodes;
            auto f = [](auto*& q) { if (q) cudaFree((void*)q); q = nullptr; };
            f(L.J); f(L.Dinv); f(L.x); f(L.r); f(L.s); f(L.x2);
            const size_t vt = sizeof(VT);
            if (!D.cuda_ok(cudaMalloc(&L.J, C.colIdx.size() * b * b * vt), "level J") ||
                !D.cuda_ok(cudaMalloc(&L.Dinv, (size_t)nc * b * b * vt), "level Dinv") ||
                !D.cuda_ok(cudaMalloc(&L.x, (size_t)nc * b * vt), "level x") ||
                !D.cuda_ok(cudaMalloc(&L.r, (size_t)nc * b * vt), "level r") ||
                !D.cuda_ok(cudaMalloc(&L.s, (size_t)nc * b * vt), "level s") ||
                !D.cuda_ok(cudaMalloc(&L.x2, (size_t)nc * b * vt), "level x2"))
                return D.status;
            L.prec = prec;
        }
    }

    std::vector<int32_t> active(nInst, 1), pend(nInst, 0), acc(nInst, 0), iters(nInst, 0);
    std::vector<double> nd0(nInst, 0.0), nd(nInst, 0.0), ndt(nInst, 0.0), lam(nInst, 1.0), rr(nInst, 0.0);
    std::vector<double> eta(nInst, adaptive ? opt.forcing_max : p.lin_rtol), ndPrev(nInst, 0.0);
    std::vector<int64_t> size(nInst);
    for (int i = 0; i < nInst; ++i) size[i] = D.instNode0[i + 1] - D.instNode0[i];
    for (int i = 0; i < nInst; ++i) { res[i] = nsfv1_newton_result{}; res[i].status = NSFV1_ERR_NOT_CONVERGED; }

    auto upload_flags = [&](const std::vector<int32_t>& f, int32_t* dst) {
        return D.cuda_ok(cudaMemcpyAsync(dst, f.data(), nInst * 4, cudaMemcpyHostToDevice, s), "flags");
    };
    auto norms = [&](const double* v, std::vector<double>& out) {
        k_inst_norm2<<<nInst, 256, 0, s>>>(D.d_instNode0, b, v, W.nrm);
        if (!D.cuda_ok(cudaMemcpyAsync(out.data(), W.nrm, nInst * 8, cudaMemcpyDeviceToHost, s), "norms")) return false;
        if (!D.cuda_ok(cudaStreamSynchronize(s), "norms")) return false;
        for (auto& x : out) x = std::sqrt(x);
        return true;
    };

    // GMRES arguments (fixed for the whole solve: every pointer stays put)
    GmresBatchArgs<VT> ga{W.queue, 0, W.head, D.d_instNode0, D.d_rowPtr, D.d_colIdx, (const VT*)W.J, (const VT*)W.Dinv,
                          W.D, (VT*)W.x, (VT*)W.V, (VT*)W.t, n, m, p.lin_rtol, p.lin_max_iter, W.iters, W.relres, (VT*)W.q, {},
                          W.nQueue, W.rtolInst};
    ga.mg.nLevels = 0;
    if (useMG) {
        ga.mg.nLevels = (int)BS->levels.size();
        ga.mg.cells0 = BS->d_cells;
        ga.mg.nu = opt.smooth_steps > 0 ? opt.smooth_steps : 2;
        ga.mg.nuCoarse = opt.coarse_steps > 0 ? opt.coarse_steps : 20;
        ga.mg.omega = opt.smooth_omega > 0.0 ? opt.smooth_omega : 0.7;
        ga.mg.lv[0] = MgLevel<VT>{D.d_rowPtr, D.d_colIdx, (const VT*)W.J, (const VT*)W.Dinv, D.d_instNode0, BS->d_mask0,
                                  (VT*)W.t, nullptr, (VT*)W.s, (VT*)W.x2};
        for (size_t l = 1; l < BS->levels.size(); ++l) {
            Level& L = BS->levels[l];
            ga.mg.lv[l] = MgLevel<VT>{L.disc->d_rowPtr, L.disc->d_colIdx, (const VT*)L.J, (const VT*)L.Dinv, L.d_node0, L.d_mask,
                                      (VT*)L.x, (VT*)L.r, (VT*)L.s, (VT*)L.x2};
        }
    }

    // the fixed device work of one Newton step, enqueued on stream q: Jacobians of
    // the active instances on every level, inverted diagonal blocks, one GMRES launch
    auto enqueue_step = [&](cudaStream_t q) -> bool {
        if (!D.assemble_jacobian(u, u_old, dt, W.J, prec, q, false)) return false;
        cudaMemsetAsync(D.d_err, 0, sizeof(int), q);
        if (b == 4) k_block_inv_active<VT, 4><<<(int)((D.nNodes + 127) / 128), 128, 0, q>>>(D.nNodes, D.d_diagPos, D.d_nodeInst, D.d_instActive, (VT*)W.J, (VT*)W.Dinv, D.d_err);
        else k_block_inv_active<VT, 3><<<(int)((D.nNodes + 127) / 128), 128, 0, q>>>(D.nNodes, D.d_diagPos, D.d_nodeInst, D.d_instActive, (VT*)W.J, (VT*)W.Dinv, D.d_err);
        if (useMG) {
            const double* uf = u;
            for (size_t l = 1; l < BS->levels.size(); ++l) {
                Level& L = BS->levels[l];
                Disc& C = *L.disc;
                const int64_t nc = C.nNodes;
                k_inject<<<(int)((nc * b + 255) / 256), 256, 0, q>>>(nc, b, L.d_inj, uf, L.d_u);
                if (!C.assemble_jacobian(L.d_u, nullptr, dt, L.J, prec, q, false)) { D.fail(C.status, C.lastError); return false; }
                if (b == 4) k_block_inv_all<VT, 4><<<(int)((nc + 127) / 128), 128, 0, q>>>(nc, C.d_diagPos, (VT*)L.J, (VT*)L.Dinv, D.d_err);
                else k_block_inv_all<VT, 3><<<(int)((nc + 127) / 128), 128, 0, q>>>(nc, C.d_diagPos, (VT*)L.J, (VT*)L.Dinv, D.d_err);
                uf = L.d_u;
            }
        }
        cudaMemsetAsync(W.head, 0, 4, q);
        cudaError_t le = (b == 4) ? launch_gmres_batch<VT, 4>(ga, clusterSize, nClusters, q) : launch_gmres_batch<VT, 3>(ga, clusterSize, nClusters, q);
        return D.cuda_ok(le, "batched GMRES launch");
    };
    auto run_step = [&]() -> bool {
        if (!useGraph) return enqueue_step(s);
        if (!BS->gs) {
            if (!D.cuda_ok(cudaStreamCreateWithFlags(&BS->gs, cudaStreamNonBlocking), "graph stream") ||
                !D.cuda_ok(cudaEventCreateWithFlags(&BS->evIn, cudaEventDisableTiming), "graph event") ||
                !D.cuda_ok(cudaEventCreateWithFlags(&BS->evOut, cudaEventDisableTiming), "graph event"))
                return false;
        }
        cudaGraphExec_t* ge = BS->graph_for(clusterSize);
        if (!ge) {
            cudaGraph_t g = nullptr;
            cudaGraphExec_t exec = nullptr;
            if (!D.cuda_ok(cudaStreamBeginCapture(BS->gs, cudaStreamCaptureModeRelaxed), "graph capture")) return false;
            const bool ok = enqueue_step(BS->gs);
            const cudaError_t ce = cudaStreamEndCapture(BS->gs, &g);
            if (!ok) { if (g) cudaGraphDestroy(g); return false; }
            if (!D.cuda_ok(ce, "graph capture")) return false;
            const cudaError_t ie = cudaGraphInstantiate(&exec, g, 0);
            cudaGraphDestroy(g);
            if (!D.cuda_ok(ie, "graph instantiate")) return false;
            BS->graphs.emplace_back(clusterSize, exec);
            ge = BS->graph_for(clusterSize);
        }
        return D.cuda_ok(cudaEventRecord(BS->evIn, s), "graph event") && D.cuda_ok(cudaStreamWaitEvent(BS->gs, BS->evIn, 0), "graph event") &&
               D.cuda_ok(cudaGraphLaunch(*ge, BS->gs), "graph launch") && D.cuda_ok(cudaEventRecord(BS->evOut, BS->gs), "graph event") &&
               D.cuda_ok(cudaStreamWaitEvent(s, BS->evOut, 0), "graph event");
    };

    const int g = (int)((n + 255) / 256);
    D.instSkip = false;
    if (!upload_flags(active, D.d_instActive)) return D.status;
    if (!D.set_dirichlet_values(u, s)) return D.status;
    if (!D.assemble_defect(u, u_old, dt, W.D, s)) return D.status;
    if (!norms(W.D, nd0)) return D.status;
    nd = nd0;
    if (opt.defect_reference == 1) {
        // reference defect of the zero iterate (Dirichlet values, 0 elsewhere)
        std::vector<double> ndz(nInst, 0.0);
        cudaMemsetAsync(W.Ut, 0, n * 8, s);
        if (!D.set_dirichlet_values(W.Ut, s)) return D.status;
        if (!D.assemble_defect(W.Ut, u_old, dt, W.Dt, s)) return D.status;
        if (!norms(W.Dt, ndz)) return D.status;
        if (opt.zero_fallback) {
            for (int i = 0; i < nInst; ++i) acc[i] = !(nd0[i] <= ndz[i]);   // also restarts a non-finite iterate
            if (!upload_flags(acc, W.accepted)) return D.status;
            k_batch_copy<<<g, 256, 0, s>>>(n, b, D.d_nodeInst, W.accepted, W.Ut, u);
            k_batch_copy<<<g, 256, 0, s>>>(n, b, D.d_nodeInst, W.accepted, W.Dt, W.D);
            for (int i = 0; i < nInst; ++i) if (acc[i]) nd[i] = ndz[i];
            std::fill(acc.begin(), acc.end(), 0);
        }
        for (int i = 0; i < nInst; ++i) {
            res[i].initial_defect = nd[i];
            nd0[i] = ndz[i];
        }
    } else {
        for (int i = 0; i < nInst; ++i) res[i].initial_defect = nd0[i];
    }
    for (int i = 0; i < nInst; ++i) {
        res[i].final_defect = nd[i];
        if (!std::isfinite(nd[i]) || !std::isfinite(nd0[i])) { active[i] = 0; res[i].status = NSFV1_ERR_NONFINITE; }
        else if (nd[i] == 0.0) { active[i] = 0; res[i].status = NSFV1_OK; }
    }
    for (int it = 0; it < p.max_iter; ++it) {
        int nAct = 0;
        for (int i = 0; i < nInst; ++i) {
            if (!active[i]) continue;
            if (nd[i] <= p.rtol * nd0[i] || nd[i] <= p.atol) { active[i] = 0; res[i].status = NSFV1_OK; continue; }
            ++nAct;
        }
        if (nAct == 0) break;
        // linear tolerances of this step
        for (int i = 0; i < nInst; ++i) {
            if (!active[i]) continue;
            if (adaptive && it > 0) eta[i] = ew_forcing(nd[i], ndPrev[i], eta[i], p.lin_rtol, opt.forcing_max, std::max(p.rtol * nd0[i], p.atol));
            else if (!adaptive) eta[i] = p.lin_rtol;
            ndPrev[i] = nd[i];
        }
        // queue: active instances, largest first
        std::vector<int32_t> q;
        for (int i = 0; i < nInst; ++i) if (active[i]) q.push_back(i);
        std::stable_sort(q.begin(), q.end(), [&](int a, int c) { return size[a] > size[c]; });
        const int nq = (int)q.size();
        // tail: with few active instances grow the clusters (up to 16 CTAs) so
        // that the instances still being solved keep the SMs busy
        clusterSize = baseCluster;
        if (opt.tail_clusters)
            while (clusterSize < 16 && (int64_t)nq * clusterSize * 2 <= numSMs && clusters_of(clusterSize * 2) > 0) clusterSize *= 2;
        nClusters = clusters_of(clusterSize);
        D.instSkip = true;
        if (!upload_flags(active, D.d_instActive) ||
            !D.cuda_ok(cudaMemcpyAsync(W.queue, q.data(), q.size() * 4, cudaMemcpyHostToDevice, s), "queue") ||
            !D.cuda_ok(cudaMemcpyAsync(W.nQueue, &nq, 4, cudaMemcpyHostToDevice, s), "queue") ||
            !D.cuda_ok(cudaMemcpyAsync(W.rtolInst, eta.data(), nInst * 8, cudaMemcpyHostToDevice, s), "tolerances"))
            return D.status;
        cudaEventRecord(evA, s);
        if (!run_step()) return D.status;
        cudaEventRecord(evB, s);
        int herr = 0;
        cudaMemcpyAsync(&herr, D.d_err, sizeof(int), cudaMemcpyDeviceToHost, s);
        cudaMemcpyAsync(iters.data(), W.iters, nInst * 4, cudaMemcpyDeviceToHost, s);
        cudaMemcpyAsync(rr.data(), W.relres, nInst * 8, cudaMemcpyDeviceToHost, s);
        if (!D.cuda_ok(cudaStreamSynchronize(s), "batched GMRES")) return D.status;
        if (herr & 1) { D.fail(NSFV1_ERR_GEOMETRY, "upwind: cannot find cut side"); cudaMemsetAsync(D.d_err, 0, sizeof(int), s); return D.status; }
        for (int i : q) {
            res[i].iterations = it + 1;
            res[i].linear_iterations += iters[i];
            if (!std::isfinite(rr[i])) { active[i] = 0; res[i].status = NSFV1_ERR_NONFINITE; }
        }
        if (herr & 2) {
            // a singular diagonal block: report it on every active instance
            for (int i : q) if (active[i]) { active[i] = 0; res[i].status = NSFV1_ERR_BREAKDOWN; }
            cudaMemsetAsync(D.d_err, 0, sizeof(int), s);
            break;
        }
        // per-instance backtracking line search on ||d||_2
        for (int i = 0; i < nInst; ++i) { pend[i] = active[i]; lam[i] = 1.0; acc[i] = 0; }
        cudaMemcpyAsync(W.Ut, u, n * 8, cudaMemcpyDeviceToDevice, s);
        for (int k = 0; k <= p.line_search_steps; ++k) {
            if (!D.cuda_ok(cudaMemcpyAsync(W.lambda, lam.data(), nInst * 8, cudaMemcpyHostToDevice, s), "lambda") ||
                !upload_flags(pend, W.pending))
                return D.status;
            k_batch_trial<VT><<<g, 256, 0, s>>>(n, b, D.d_nodeInst, W.pending, W.lambda, u, (const VT*)W.x, W.Ut);
            if (!upload_flags(pend, D.d_instActive)) return D.status;
            if (!D.assemble_defect(W.Ut, u_old, dt, W.Dt, s)) return D.status;
            if (!norms(W.Dt, ndt)) return D.status;
            bool any = false;
            std::fill(acc.begin(), acc.end(), 0);
            for (int i = 0; i < nInst; ++i) {
                if (!pend[i]) continue;
                if (ndt[i] <= (1.0 - 1e-4 * lam[i]) * nd[i] || k == p.line_search_steps || !std::isfinite(ndt[i])) {
                    acc[i] = 1; pend[i] = 0; nd[i] = ndt[i];
                } else {
                    lam[i] *= 0.5; any = true;
                }
            }
            if (!upload_flags(acc, W.accepted)) return D.status;
            k_batch_copy<<<g, 256, 0, s>>>(n, b, D.d_nodeInst, W.accepted, W.Dt, W.D);
            if (!any) break;
        }
        cudaEventRecord(evC, s);
        {
            float a = 0.f, c = 0.f;
            cudaEventSynchronize(evC);
            cudaEventElapsedTime(&a, evA, evB);
            cudaEventElapsedTime(&c, evB, evC);
            BS->stats[0] += 1.0; BS->stats[1] += a; BS->stats[2] += c;
        }
        // u <- Ut on the active instances
        if (!upload_flags(active, W.accepted)) return D.status;
        k_batch_copy<<<g, 256, 0, s>>>(n, b, D.d_nodeInst, W.accepted, W.Ut, u);
        for (int i = 0; i < nInst; ++i) {
            if (!active[i]) continue;
            res[i].final_defect = nd[i];
            if (!std::isfinite(nd[i])) { active[i] = 0; res[i].status = NSFV1_ERR_NONFINITE; }
        }
    }
    for (int i = 0; i < nInst; ++i) {
        res[i].final_defect = nd[i];
        if (active[i] && (nd[i] <= p.rtol * nd0[i] || nd[i] <= p.atol)) res[i].status = NSFV1_OK;
    }
    D.instSkip = false;
    std::vector<int32_t> all(nInst, 1);
    upload_flags(all, D.d_instActive);
    if (!D.cuda_ok(cudaStreamSynchronize(s), "batched newton")) return D.status;
    BS->stats[3] = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - wall0).count();
    int worst = NSFV1_OK;
    for (int i = 0; i < nInst; ++i) if (res[i].status != NSFV1_OK) worst = res[i].status;
    if (worst != NSFV1_OK) D.fail(worst, "batched Newton: some instances did not converge (see the per-instance results)");
    return worst;
}

}  // namespace

namespace nsfv1 {
void batch_free(void* p) { delete static_cast<BatchState*>(p); }
}  // namespace nsfv1

extern "C" {

int nsfv1_set_elem_viscosity(nsfv1_disc* h, const double* nu) {
    Disc* D = reinterpret_cast<Disc*>(h);
    if (!D) return NSFV1_ERR_ARGUMENT;
    D->status = NSFV1_OK;
    if (!D->hasMesh) { D->fail(NSFV1_ERR_STATE, "set_elem_viscosity: no mesh"); return D->status; }
    if (D->d_nuElem) { cudaFree(D->d_nuElem); D->d_nuElem = nullptr; }
    D->nuElemHost.clear();
    if (!nu) return NSFV1_OK;
    for (int64_t e = 0; e < D->nElems; ++e)
        if (!(nu[e] > 0.0) || !std::isfinite(nu[e])) { D->fail(NSFV1_ERR_ARGUMENT, "set_elem_viscosity: viscosity must be positive"); return D->status; }
    if (!D->cuda_ok(cudaMalloc((void**)&D->d_nuElem, sizeof(double) * D->nElems), "alloc viscosity") ||
        !D->cuda_ok(cudaMemcpy(D->d_nuElem, nu, sizeof(double) * D->nElems, cudaMemcpyHostToDevice), "upload viscosity"))
        return D->status;
    D->nuElemHost.assign(nu, nu + D->nElems);
    D->viscoSet = true;
    return NSFV1_OK;
}

int nsfv1_set_instances(nsfv1_disc* h, int n_inst, const int32_t* node_offsets) {
    Disc* D = reinterpret_cast<Disc*>(h);
    if (!D) return NSFV1_ERR_ARGUMENT;
    D->status = NSFV1_OK;
    if (!D->hasMesh) { D->fail(NSFV1_ERR_STATE, "set_instances: no mesh"); return D->status; }
    if (n_inst <= 0 || !node_offsets || node_offsets[0] != 0 || node_offsets[n_inst] != D->nNodes) {
        D->fail(NSFV1_ERR_ARGUMENT, "set_instances: offsets must start at 0 and end at the node count");
        return D->status;
    }
    std::vector<int32_t> nodeInst(D->nNodes), elemInst(D->nElems);
    for (int i = 0; i < n_inst; ++i) {
        if (node_offsets[i + 1] <= node_offsets[i]) { D->fail(NSFV1_ERR_ARGUMENT, "set_instances: empty or decreasing range"); return D->status; }
        for (int32_t v = node_offsets[i]; v < node_offsets[i + 1]; ++v) nodeInst[v] = i;
    }
    const int nsh = D->nsh;
    std::vector<int32_t> conn;   // host copy of the connectivity is needed for the check
    conn.resize((size_t)D->nElems * nsh);
    if (!D->cuda_ok(cudaMemcpy(conn.data(), D->d_conn, conn.size() * 4, cudaMemcpyDeviceToHost), "read conn")) return D->status;
    for (int64_t e = 0; e < D->nElems; ++e) {
        const int i = nodeInst[conn[e * nsh]];
        for (int k = 1; k < nsh; ++k)
            if (nodeInst[conn[e * nsh + k]] != i) { D->fail(NSFV1_ERR_ARGUMENT, "set_instances: an element spans two instances"); return D->status; }
        elemInst[e] = i;
    }
    auto up = [&](int32_t*& dst, const int32_t* src, size_t cnt) {
        if (dst) cudaFree(dst);
        dst = nullptr;
        return D->cuda_ok(cudaMalloc((void**)&dst, cnt * 4), "alloc instances") &&
               D->cuda_ok(cudaMemcpy(dst, src, cnt * 4, cudaMemcpyHostToDevice), "upload instances");
    };
    std::vector<int32_t> ones(n_inst, 1);
    if (!up(D->d_instNode0, node_offsets, n_inst + 1) || !up(D->d_nodeInst, nodeInst.data(), nodeInst.size()) ||
        !up(D->d_elemInst, elemInst.data(), elemInst.size()) || !up(D->d_instActive, ones.data(), n_inst))
        return D->status;
    // multigrid levels, graphs and solver buffers of the previous partition no longer apply
    if (D->batch) { batch_free(D->batch); D->batch = nullptr; }
    D->instCells.clear();
    D->nInst = n_inst;
    D->instNode0.assign(node_offsets, node_offsets + n_inst + 1);
    D->instSkip = false;
    return NSFV1_OK;
}

int nsfv1_set_instance_grids(nsfv1_disc* h, const int32_t* cells) {
    Disc* D = reinterpret_cast<Disc*>(h);
    if (!D) return NSFV1_ERR_ARGUMENT;
    D->status = NSFV1_OK;
    if (!D->hasMesh || D->nInst <= 0) { D->fail(NSFV1_ERR_STATE, "set_instance_grids: set the mesh and the instances first"); return D->status; }
    if (D->roid != ROID_QUADRILATERAL) { D->fail(NSFV1_ERR_ARGUMENT, "set_instance_grids: structured quadrilateral instances only"); return D->status; }
    const int nInst = D->nInst, b = D->dim + 1;
    for (int i = 0; i < nInst; ++i) {
        const int64_t m = (int64_t)cells[i] + 1;
        if (cells[i] <= 0 || m * m != D->instNode0[i + 1] - D->instNode0[i]) {
            D->fail(NSFV1_ERR_ARGUMENT, "set_instance_grids: node count of an instance is not (cells+1)^2");
            return D->status;
        }
    }
    BatchState* BS = batch_state(*D);
    BS->clear_levels();
    D->instCells.assign(cells, cells + nInst);
    // fine-level Dirichlet mask and the cells per side
    std::vector<uint8_t> mask0((size_t)D->nNodes * b, 1);
    for (int32_t r : D->dirRowHost) mask0[r] = 0;
    if (!D->cuda_ok(cudaMalloc((void**)&BS->d_mask0, mask0.size()), "mg mask") ||
        !D->cuda_ok(cudaMemcpy(BS->d_mask0, mask0.data(), mask0.size(), cudaMemcpyHostToDevice), "mg mask") ||
        !D->cuda_ok(cudaMalloc((void**)&BS->d_cells, nInst * 4), "mg cells") ||
        !D->cuda_ok(cudaMemcpy(BS->d_cells, cells, nInst * 4, cudaMemcpyHostToDevice), "mg cells"))
        return D->status;
    BS->levels.resize(1);
    // finer-level data of the current step (level 0 = this handle)
    std::vector<double> fCoords = D->coordsHost;
    std::vector<int32_t> fNode0(D->instNode0.begin(), D->instNode0.end() - 1);
    std::vector<int> fCells(cells, cells + nInst);
    std::vector<uint8_t> fDir(mask0.size());
    std::vector<double> fDirVal(mask0.size(), 0.0);
    for (size_t k = 0; k < D->dirRowHost.size(); ++k) { fDir[D->dirRowHost[k]] = 1; fDirVal[D->dirRowHost[k]] = D->dirValHost[k]; }
    std::vector<double> instNu(nInst, D->nu);
    if (!D->nuElemHost.empty()) {
        std::vector<int32_t> firstElem(nInst, -1);
        for (int64_t e = D->nElems - 1; e >= 0; --e) {
            const int32_t nd = D->connHost[e * D->nsh];
            const int i = (int)(std::upper_bound(D->instNode0.begin(), D->instNode0.end(), nd) - D->instNode0.begin()) - 1;
            firstElem[i] = (int32_t)e;
        }
        for (int i = 0; i < nInst; ++i) instNu[i] = D->nuElemHost[firstElem[i]];
    }
    for (int l = 1; l < kMaxLevels; ++l) {
        // instances that coarsen once more (even cells, at least 4 coarse cells)
        std::vector<int32_t> cNode0(nInst, -1);
        std::vector<double> coords;
        std::vector<int32_t> conn, inj, dirRow;
        std::vector<double> dirVal, nuE;
        std::vector<int32_t> instOff{0};
        int32_t nn = 0;
        for (int i = 0; i < nInst; ++i) {
            if (fNode0[i] < 0 || fCells[i] % 2 != 0 || fCells[i] / 2 < 4) continue;
            const int nc = fCells[i] / 2, mc = nc + 1, mf = fCells[i] + 1;
            cNode0[i] = nn;
            for (int J = 0; J < mc; ++J)
                for (int I = 0; I < mc; ++I) {
                    const int64_t fnode = fNode0[i] + (int64_t)(2 * J) * mf + 2 * I;
                    coords.push_back(fCoords[fnode * 2]); coords.push_back(fCoords[fnode * 2 + 1]);
                    inj.push_back((int32_t)fnode);
                    for (int f = 0; f < b; ++f)
                        if (fDir[fnode * b + f]) { dirRow.push_back((nn + J * mc + I) * b + f); dirVal.push_back(fDirVal[fnode * b + f]); }
                }
            for (int J = 0; J < nc; ++J)
                for (int I = 0; I < nc; ++I) {
                    const int32_t n0 = nn + J * mc + I;
                    conn.push_back(n0); conn.push_back(n0 + 1); conn.push_back(n0 + mc + 1); conn.push_back(n0 + mc);
                    nuE.push_back(instNu[i]);
                }
            nn += mc * mc;
            instOff.push_back(nn);
        }
        if (nn == 0) break;
        Level L;
        L.disc = new Disc();
        Disc& C = *L.disc;
        C.dim = D->dim; C.nu = D->nu; C.rho = D->rho; C.fullNewton = D->fullNewton;
        for (int d = 0; d < 3; ++d) C.src[d] = D->src[d];
        C.hasSource = D->hasSource; C.stokes = D->stokes; C.laplace = D->laplace; C.peclet = D->peclet;
        C.viscoSet = D->viscoSet; C.stabSet = D->stabSet; C.convUpwindSet = D->convUpwindSet; C.stabSharesConv = D->stabSharesConv;
        C.convUpwindType = D->convUpwindType; C.stabUpwindType = D->stabUpwindType; C.stabType = D->stabType; C.diffLen = D->diffLen;
        nsfv1_disc* ch = reinterpret_cast<nsfv1_disc*>(&C);
        C.pac = D->pac;
        int st = C.ensure_ipws() ? NSFV1_OK : C.status;
        if (st == NSFV1_OK) st = nsfv1_set_mesh(ch, ROID_QUADRILATERAL, nn, coords.data(), (int64_t)conn.size() / 4, conn.data());
        if (st == NSFV1_OK) st = nsfv1_set_elem_viscosity(ch, nuE.data());
        if (st == NSFV1_OK) st = nsfv1_set_dirichlet(ch, (int64_t)dirRow.size(), dirRow.data(), dirVal.data());
        if (st != NSFV1_OK) { D->fail(st, "multigrid level " + std::to_string(l) + ": " + C.lastError); L.release(); return D->status; }
        std::vector<uint8_t> mask((size_t)nn * b, 1);
        for (int32_t r : dirRow) mask[r] = 0;
        if (!D->cuda_ok(cudaMalloc((void**)&L.d_node0, nInst * 4), "level") ||
            !D->cuda_ok(cudaMemcpy(L.d_node0, cNode0.data(), nInst * 4, cudaMemcpyHostToDevice), "level") ||
            !D->cuda_ok(cudaMalloc((void**)&L.d_inj, inj.size() * 4), "level") ||
            !D->cuda_ok(cudaMemcpy(L.d_inj, inj.data(), inj.size() * 4, cudaMemcpyHostToDevice), "level") ||
            !D->cuda_ok(cudaMalloc((void**)&L.d_mask, mask.size()), "level") ||
            !D->cuda_ok(cudaMemcpy(L.d_mask, mask.data(), mask.size(), cudaMemcpyHostToDevice), "level") ||
            !D->cuda_ok(cudaMalloc((void**)&L.d_u, (size_t)nn * b * 8), "level")) {
            L.release();
            return D->status;
        }
        L.node0 = cNode0;
        BS->levels.push_back(std::move(L));
        // this level becomes the finer level of the next one
        fCoords = coords;
        std::vector<int> nCells(nInst, 0);
        for (int i = 0; i < nInst; ++i) nCells[i] = cNode0[i] >= 0 ? fCells[i] / 2 : 0;
        std::vector<uint8_t> nDir((size_t)nn * b, 0);
        std::vector<double> nDirVal((size_t)nn * b, 0.0);
        for (size_t k = 0; k < dirRow.size(); ++k) { nDir[dirRow[k]] = 1; nDirVal[dirRow[k]] = dirVal[k]; }
        fNode0 = cNode0; fCells = nCells; fDir = nDir; fDirVal = nDirVal;
    }
    return NSFV1_OK;
}

int nsfv1_batch_autotune(nsfv1_disc* h, const double* u, const double* u_old, double dt, const nsfv1_newton_params* p,
                         nsfv1_batch_options* opt, const int* candidates, int n_candidates, double* ms, void* stream) {
    Disc* D = reinterpret_cast<Disc*>(h);
    if (!D) return NSFV1_ERR_ARGUMENT;
    D->status = NSFV1_OK;
    if (!D->hasMesh || D->nInst <= 0) { D->fail(NSFV1_ERR_STATE, "batch_autotune: no mesh or no instances"); return D->status; }
    if (!u || !p || !opt || !candidates || n_candidates <= 0) { D->fail(NSFV1_ERR_ARGUMENT, "batch_autotune: null argument"); return D->status; }
    for (int c = 0; c < n_candidates; ++c)
        if (candidates[c] < 1 || candidates[c] > 16) { D->fail(NSFV1_ERR_ARGUMENT, "batch_autotune: cluster sizes must be 1..16"); return D->status; }
    if (p->jacobian_prec != NSFV1_F64 && p->jacobian_prec != NSFV1_F32) { D->fail(NSFV1_ERR_ARGUMENT, "batch_autotune: bad precision"); return D->status; }
    cudaStream_t s = (cudaStream_t)stream;
    const int64_t n = D->nNodes * (D->dim + 1);
    double* tu = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (!D->cuda_ok(cudaMalloc(&tu, n * 8), "autotune") || !D->cuda_ok(cudaEventCreate(&e0), "autotune") ||
        !D->cuda_ok(cudaEventCreate(&e1), "autotune")) {
        if (tu) cudaFree(tu);
        return D->status;
    }
    nsfv1_newton_params q = *p;
    q.max_iter = 1;
    std::vector<nsfv1_newton_result> r(D->nInst);
    std::vector<double> t(n_candidates, 0.0);
    int st = NSFV1_OK;
    for (int pass = 0; pass < 2 && st == NSFV1_OK; ++pass) {
        for (int c = 0; c < n_candidates && st == NSFV1_OK; ++c) {
            nsfv1_batch_options o = *opt;
            o.cluster_size = candidates[c];
            cudaMemcpyAsync(tu, u, n * 8, cudaMemcpyDeviceToDevice, s);
            cudaEventRecord(e0, s);
            const int rs = q.jacobian_prec == NSFV1_F64 ? batched_newton<double>(*D, tu, u_old, dt, q, o, r.data(), s)
                                                        : batched_newton<float>(*D, tu, u_old, dt, q, o, r.data(), s);
            cudaEventRecord(e1, s);
            if (rs == NSFV1_ERR_CUDA || rs == NSFV1_ERR_ARGUMENT || rs == NSFV1_ERR_STATE || rs == NSFV1_ERR_GEOMETRY) { st = rs; break; }
            float msec = 0.f;
            if (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&msec, e0, e1) != cudaSuccess) {
                D->fail(NSFV1_ERR_CUDA, "autotune timing");
                st = NSFV1_ERR_CUDA;
                break;
            }
            t[c] = msec;
        }
    }
    cudaFree(tu);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (st != NSFV1_OK) return st;
    int best = 0;
    for (int c = 1; c < n_candidates; ++c) if (t[c] < t[best]) best = c;
    opt->cluster_size = candidates[best];
    if (ms) for (int c = 0; c < n_candidates; ++c) ms[c] = t[c];
    D->status = NSFV1_OK;
    D->lastError.clear();
    return NSFV1_OK;
}

int nsfv1_batch_stats(const nsfv1_disc* h, double* out, int n) {
    const Disc* D = reinterpret_cast<const Disc*>(h);
    if (!D || !out || n <= 0) return NSFV1_ERR_ARGUMENT;
    const BatchState* BS = static_cast<const BatchState*>(D->batch);
    for (int i = 0; i < n; ++i) out[i] = (BS && i < 8) ? BS->stats[i] : 0.0;
    return NSFV1_OK;
}

int nsfv1_newton_solve_batched(nsfv1_disc* h, double* u, const double* u_old, double dt, const nsfv1_newton_params* p,
                               const nsfv1_batch_options* opt, nsfv1_newton_result* results, void* stream) {
    Disc* D = reinterpret_cast<Disc*>(h);
    if (!D) return NSFV1_ERR_ARGUMENT;
    D->status = NSFV1_OK;
    if (!D->hasMesh || D->nInst <= 0) { D->fail(NSFV1_ERR_STATE, "newton_solve_batched: no mesh or no instances"); return D->status; }
    if (!u || !p || !results) { D->fail(NSFV1_ERR_ARGUMENT, "newton_solve_batched: null argument"); return D->status; }
    nsfv1_batch_options o{};
    if (opt) o = *opt;
    if (o.cluster_size < 0 || o.cluster_size > 16) { D->fail(NSFV1_ERR_ARGUMENT, "newton_solve_batched: cluster size must be 1..16"); return D->status; }
    if (p->jacobian_prec == NSFV1_F64) return batched_newton<double>(*D, u, u_old, dt, *p, o, results, (cudaStream_t)stream);
    if (p->jacobian_prec == NSFV1_F32) return batched_newton<float>(*D, u, u_old, dt, *p, o, results, (cudaStream_t)stream);
    D->fail(NSFV1_ERR_ARGUMENT, "newton_solve_batched: bad precision");
    return D->status;
}

}  // extern "C"
