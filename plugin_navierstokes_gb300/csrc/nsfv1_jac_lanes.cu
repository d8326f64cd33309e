// nsfv1_jac_lanes.cu -- the FP32 Jacobian assembly (the Newton loop's FP32-matrix
// mode) with one lane group per element: one lane per corner of the element.
//
// With one thread per element (the structure of the FP64 k_jacobian) one colour
// of a 64^3 hexahedral mesh is 1024 warps (6.7 per SM), latency-bound, and each
// SCVF's blocks go straight into the matrix: three reductions per block and
// element, spread over the whole kernel, so the colour's 134 MB of blocks cycle
// through L2 three times. Here every element of a colour gets nsh lanes:
//  0. lane k converts corner k (coordinates, state) into the element's shared-
//     memory record, and one lane computes the element geometry there;
//  1. lane k evaluates SCVFs k, k + nsh, ... (geometry, upwinds, stabilisation,
//     the per-SCVF factors of add_jac_A_elem, navier_stokes_fv1.cpp:250-595) and
//     leaves the factors in shared memory;
//  2. lane k forms column k of the element matrix: for every SCVF the block of
//     corner k (jac_block_col, the same block algebra as the FP64 path) added to
//     row 'from' and subtracted from row 'to', summed in registers in SCVF order;
//  3. a row is reduced into the matrix once its last SCVF is in: one
//     red.global.add per block row and element (a quarter of the reductions).
// Determinism is unchanged: within a colour no other lane touches these blocks,
// every block of an element is summed in a fixed order by one lane, and the
// colours run in order.
#include <utility>
#include "nsfv1_asm_common.cuh"

namespace nsfv1 {
namespace {

template <int ROID>
struct Lanes {
    using R = Ref<ROID>;
    static constexpr int L = R::nsh;                        // lanes per element
    static constexpr int EPW = 32 / L;                      // elements per warp
    static constexpr int ROUNDS = (R::nip + L - 1) / L;     // SCVF rounds of the factor phase
    static constexpr int FS = 28 + ((3 * R::nsh + 3) / 4) * 4;   // floats per SCVF slot
    static constexpr int WARPS = 4;
    static constexpr int THREADS = 32 * WARPS;
    static constexpr int EPC = WARPS * EPW;                 // elements per CTA
};

// Shared memory of one CTA (dynamic): the SCVF factor slots, then per element its
// geometry (Elem, filled by the group) and states, then the reference tables.
template <int ROID, bool PAC>
struct LaneSmem {
    using R = Ref<ROID>;
    using C = Lanes<ROID>;
    static constexpr size_t slots = sizeof(float) * C::EPC * R::nip * C::FS;
    static constexpr size_t elemBytes = (sizeof(Elem<ROID, float>) + 15) / 16 * 16;
    static constexpr size_t elems = elemBytes * C::EPC;
    static constexpr size_t uFloats = R::b * R::nsh + (PAC ? R::dim * R::nsh : 0);   // u [b][nsh], then uo [dim][nsh]
    static constexpr size_t us = (sizeof(float) * uFloats * C::EPC + 15) / 16 * 16;
    static constexpr size_t tab = sizeof(float4) * R::nip * R::nsh;
    static constexpr size_t bytes = slots + elems + us + tab;
};

// slot layout: the scalar factors of JacIp, then its per-corner shapes
enum : int {
    F_N = 0, F_IDIAG = 3, F_JT = 4, F_VEL = 13, F_UPV = 16, F_NUL = 19, F_NSVCL = 20, F_NSVDL = 21,
    F_PW = 22, F_PPE = 23, F_W = 24, F_RIVN = 25, F_ARR = 28
};

// the scalar factors of one SCVF as jac_block_col reads them
struct LaneFactors {
    float n[3], JtInv[3][3], StdVel[3], UpwindVel[3];
    float nuL, nsvcl, nsvdl, idiag, pw, ppe, w, riVn;
};

// first / last SCVF (reference order) with corner i as 'from' or 'to'
template <int ROID>
__host__ __device__ constexpr int first_ip(const int i) {
    for (int ip = 0; ip < Ref<ROID>::nip; ++ip)
        if (Ref<ROID>::edge(ip, 0) == i || Ref<ROID>::edge(ip, 1) == i) return ip;
    return -1;
}
template <int ROID>
__host__ __device__ constexpr int last_ip(const int i) {
    int l = -1;
    for (int ip = 0; ip < Ref<ROID>::nip; ++ip)
        if (Ref<ROID>::edge(ip, 0) == i || Ref<ROID>::edge(ip, 1) == i) l = ip;
    return l;
}

template <class F, int... I>
__device__ __forceinline__ void for_each_const(F&& f, std::integer_sequence<int, I...>) {
    (f(std::integral_constant<int, I>{}), ...);
}

template <int ROID>
__device__ __forceinline__ void store_factors(float* __restrict__ sl, const JacIp<ROID, float>& J) {
    constexpr int nsh = Ref<ROID>::nsh;
    float4* q = reinterpret_cast<float4*>(sl);
    q[0] = make_float4(J.n[0], J.n[1], J.n[2], J.idiag);
    q[1] = make_float4(J.JtInv[0][0], J.JtInv[0][1], J.JtInv[0][2], J.JtInv[1][0]);
    q[2] = make_float4(J.JtInv[1][1], J.JtInv[1][2], J.JtInv[2][0], J.JtInv[2][1]);
    q[3] = make_float4(J.JtInv[2][2], J.StdVel[0], J.StdVel[1], J.StdVel[2]);
    q[4] = make_float4(J.UpwindVel[0], J.UpwindVel[1], J.UpwindVel[2], J.nuL);
    q[5] = make_float4(J.nsvcl, J.nsvdl, J.pw, J.ppe);
    q[6] = make_float4(J.w, J.riVn, 0.f, 0.f);
#pragma unroll
    for (int s = 0; s < nsh; ++s) {
        sl[F_ARR + s] = J.upC[s];
        sl[F_ARR + nsh + s] = J.upS[s];
        sl[F_ARR + 2 * nsh + s] = J.dnS[s];
    }
}

__device__ __forceinline__ void load_factors(const float* __restrict__ sl, LaneFactors& F) {
    const float4* q = reinterpret_cast<const float4*>(sl);
    const float4 a0 = q[0], a1 = q[1], a2 = q[2], a3 = q[3], a4 = q[4], a5 = q[5], a6 = q[6];
    F.n[0] = a0.x; F.n[1] = a0.y; F.n[2] = a0.z; F.idiag = a0.w;
    F.JtInv[0][0] = a1.x; F.JtInv[0][1] = a1.y; F.JtInv[0][2] = a1.z; F.JtInv[1][0] = a1.w;
    F.JtInv[1][1] = a2.x; F.JtInv[1][2] = a2.y; F.JtInv[2][0] = a2.z; F.JtInv[2][1] = a2.w;
    F.JtInv[2][2] = a3.x; F.StdVel[0] = a3.y; F.StdVel[1] = a3.z; F.StdVel[2] = a3.w;
    F.UpwindVel[0] = a4.x; F.UpwindVel[1] = a4.y; F.UpwindVel[2] = a4.z; F.nuL = a4.w;
    F.nsvcl = a5.x; F.nsvdl = a5.y; F.pw = a5.z; F.ppe = a5.w;
    F.w = a6.x; F.riVn = a6.y;
}

// SPEC fixes flags at compile time (the common configurations, much smaller
// unrolled column loop): 0 = none, 1 = FLOW, 2 = FIELDS, both without Stokes,
// Laplace or Peclet blend
enum : int { SPEC_GENERIC = 0, SPEC_FLOW = 1, SPEC_FIELDS = 2 };

inline int lanes_spec(const DiscParams& P) {
    if (P.stokes || P.laplace || P.peclet) return SPEC_GENERIC;
    return P.stab == STAB_FLOW ? SPEC_FLOW : P.stab == STAB_FIELDS ? SPEC_FIELDS : SPEC_GENERIC;
}

template <int ROID, bool PAC, int SPEC>
__global__ void __launch_bounds__(Lanes<ROID>::THREADS, 3) k_jacobian_lanes(const DiscParams Pin, const AsmArgs A) {
    // a local copy whose fixed members the compiler folds into the element code
    DiscParams P = Pin;
    if constexpr (SPEC != SPEC_GENERIC) {
        P.stokes = 0; P.laplace = 0; P.peclet = 0;
        P.stab = SPEC == SPEC_FLOW ? STAB_FLOW : STAB_FIELDS;
    }
    using R = Ref<ROID>;
    using C = Lanes<ROID>;
    constexpr int dim = R::dim, nsh = R::nsh, nip = R::nip, b = R::b;
    constexpr int L = C::L, EPW = C::EPW, FS = C::FS;
    using M = LaneSmem<ROID, PAC>;
    extern __shared__ __align__(16) unsigned char smem[];
    float* sSlots = reinterpret_cast<float*>(smem);
    unsigned char* sElems = smem + M::slots;
    float* sU = reinterpret_cast<float*>(smem + M::slots + M::elems);
    float4* sTab = reinterpret_cast<float4*>(smem + M::slots + M::elems + M::us);   // (reference gradient, value) of shape k at SCVF ip
    {
        const auto& tb = tab<ROID, float>();
        for (int j = threadIdx.x; j < nip * nsh; j += blockDim.x) {
            const int ip = j / nsh, k = j - ip * nsh;
            sTab[j] = make_float4(tb.ipLGrad[ip][k][0], tb.ipLGrad[ip][k][1], tb.ipLGrad[ip][k][2], tb.ipShape[ip][k]);
        }
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int grp = lane / L, k = lane - grp * L;
    if (grp >= EPW) return;   // the lanes left over when nsh does not divide 32
    const int64_t t = ((int64_t)blockIdx.x * C::WARPS + warp) * EPW + grp;
    if (t >= A.count) return;
    const int32_t e = __ldg(A.elems + t);
    if (A.elemInst && !__ldg(A.instActive + __ldg(A.elemInst + e))) return;
    // the lanes of this element (the whole group returns together above)
    const unsigned mask = ((1u << L) - 1u) << (grp * L);
    const float nuEl = (float)(A.nuElem ? __ldg(A.nuElem + e) : P.nu);
    // ---- gather: lane k converts corner k (coordinates relative to corner 0, in
    // FP64 before the rounding, and the states) once for the whole group
    const int32_t node0 = __ldg(A.conn + (int64_t)e * nsh);
    const int32_t nodek = __ldg(A.conn + (int64_t)e * nsh + k);
#ifdef NSFV1_BOUNDS_CHECK
    // the group leaves together (the syncs below wait for all of its lanes)
    const bool inRange = NSFV1_IN_RANGE(node0, A.nNodes, A.err) && NSFV1_IN_RANGE(nodek, A.nNodes, A.err);
    if (!__all_sync(mask, inRange)) return;
#endif
    const bool withOld = PAC && P.transient && P.pac && P.fullNewton != 0.0;
    const int slot = warp * EPW + grp;
    Elem<ROID, float>& E = *reinterpret_cast<Elem<ROID, float>*>(sElems + slot * M::elemBytes);
    float (&u)[b][nsh] = *reinterpret_cast<float(*)[b][nsh]>(sU + slot * M::uFloats);
    // the old state (PAC with the exact-Jacobian terms only; otherwise any array, unread)
    float (&uo)[dim][nsh] = *reinterpret_cast<float(*)[dim][nsh]>(sU + slot * M::uFloats + (PAC ? b * nsh : 0));
    {
#pragma unroll
        for (int d = 0; d < dim; ++d)
            E.x[k][d] = (float)(__ldg(A.coords + (int64_t)nodek * dim + d) - __ldg(A.coords + (int64_t)node0 * dim + d));
#pragma unroll
        for (int f = 0; f < b; ++f) u[f][k] = (float)__ldg(A.U + (int64_t)nodek * b + f);
        if constexpr (PAC) {
#pragma unroll
            for (int f = 0; f < dim; ++f) uo[f][k] = withOld ? (float)__ldg(A.Uold + (int64_t)nodek * b + f) : 0.f;
        }
    }
    __syncwarp(mask);
    // the element geometry once per group, in shared memory (read by every lane's SCVFs)
    if (k == 0) elem_setup<ROID, float>(E);
    __syncwarp(mask);
    float* mySlots = sSlots + slot * nip * FS;
    const float volk = E.vol[k];
    bool ok = true;
    {
        // ---- phase 1: the factors of SCVFs k, k + nsh, ...
        float corMinN = 0.f, corMinD = 0.f, corAvgN = 1.f;
        if (P.stab != STAB_WITHOUT && P.diffLen == DL_COR) cor_data<ROID, float>(E, corMinN, corMinD, corAvgN);
#pragma unroll 1
        for (int r = 0; r < C::ROUNDS; ++r) {
            const int ip = k + r * L;
            if (ip >= nip) break;
            IpGeo<float> G;
            ip_geom<ROID, float>(E, ip, G);
            IpState<ROID, float> S;
            ip_state<ROID, float>(P, E, G, ip, u, corMinN, corMinD, corAvgN, nuEl, S);
            ok &= S.ok;
            JacIp<ROID, float> J;
            jac_ip_factors<ROID, float, PAC>(P, G, S, ip, u, uo, nuEl, J);
            store_factors<ROID>(mySlots + ip * FS, J);
        }
    }
    if (!ok) atomicOr(A.err, 1);
    __syncwarp(mask);
    // ---- phase 2: column k of the element matrix, rows reduced as they complete
    int32_t q[nsh];
#pragma unroll
    for (int i = 0; i < nsh; ++i) q[i] = __ldg(A.elemBlk + (int64_t)e * nsh * nsh + i * nsh + k);
    const float scale = P.transient ? (float)P.dt : 1.f;
    const float mass = volk * (float)P.rho;
    float* __restrict__ vals = reinterpret_cast<float*>(A.vals);
    float acc[nsh][b][b];
    auto flush = [&](auto ic) {
        constexpr int i = decltype(ic)::value;
        if (!NSFV1_IN_RANGE(q[i], A.nnzb, A.err)) return;
        float v[b][b];
#pragma unroll
        for (int r = 0; r < b; ++r)
#pragma unroll
            for (int c = 0; c < b; ++c) v[r][c] = acc[i][r][c] * scale;
        if (P.transient && i == k) {
#pragma unroll
            for (int d = 0; d < dim; ++d) v[d][d] += mass;
        }
        float* p = vals + (int64_t)q[i] * (b * b);
        if constexpr (b == 4) {
#pragma unroll
            for (int r = 0; r < 4; ++r)
                asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(p + r * 4), "f"(v[r][0]), "f"(v[r][1]),
                             "f"(v[r][2]), "f"(v[r][3])
                             : "memory");
        } else {
#pragma unroll
            for (int r = 0; r < b; ++r)
#pragma unroll
                for (int c = 0; c < b; ++c) atomicAdd(p + r * b + c, v[r][c]);
        }
    };
    auto step = [&](auto ipc) {
        constexpr int ip = decltype(ipc)::value;
        constexpr int fr = R::edge(ip, 0), to = R::edge(ip, 1);
        const float* sl = mySlots + ip * FS;
        LaneFactors F;
        load_factors(sl, F);
        const float4 tk = sTab[ip * nsh + k];
        const float lg[3] = {tk.x, tk.y, tk.z};
        float B[b][b];
        jac_block_col<ROID, float, PAC>(P, F, lg, tk.w, sl[F_ARR + k], sl[F_ARR + nsh + k], sl[F_ARR + 2 * nsh + k], nuEl, B);
#pragma unroll
        for (int r = 0; r < b; ++r)
#pragma unroll
            for (int c = 0; c < b; ++c) {
                if constexpr (first_ip<ROID>(fr) == ip) acc[fr][r][c] = B[r][c];
                else acc[fr][r][c] += B[r][c];
                if constexpr (first_ip<ROID>(to) == ip) acc[to][r][c] = -B[r][c];
                else acc[to][r][c] -= B[r][c];
            }
        if constexpr (last_ip<ROID>(fr) == ip) flush(std::integral_constant<int, fr>{});
        if constexpr (last_ip<ROID>(to) == ip) flush(std::integral_constant<int, to>{});
    };
    for_each_const(step, std::make_integer_sequence<int, nip>{});
}

template <class F>
cudaError_t dispatch_roid_lanes(int roid, F&& f) {
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

cudaError_t launch_jacobian_lanes(int roid, const DiscParams& P, const AsmArgs& a, cudaStream_t s) {
    if (a.count <= 0) return cudaSuccess;
    return dispatch_roid_lanes(roid, [&](auto r) {
        constexpr int RO = decltype(r)::value;
        using C = Lanes<RO>;
        const int grid = (a.count + C::EPC - 1) / C::EPC;
        const int spec = lanes_spec(P);
        auto go = [&](auto kern, size_t bytes) {
            // dynamic shared memory above 48 KB needs the per-kernel opt-in (set once)
            static bool attr = false;
            if (!attr && bytes > 48 * 1024) {
                if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) != cudaSuccess) return;
                attr = true;
            }
            kern<<<grid, C::THREADS, bytes, s>>>(P, a);
        };
        if (P.pac && !P.stokes) go(k_jacobian_lanes<RO, true, SPEC_GENERIC>, LaneSmem<RO, true>::bytes);
        else if (spec == SPEC_FLOW) go(k_jacobian_lanes<RO, false, SPEC_FLOW>, LaneSmem<RO, false>::bytes);
        else if (spec == SPEC_FIELDS) go(k_jacobian_lanes<RO, false, SPEC_FIELDS>, LaneSmem<RO, false>::bytes);
        else go(k_jacobian_lanes<RO, false, SPEC_GENERIC>, LaneSmem<RO, false>::bytes);
    });
}

}  // namespace nsfv1
