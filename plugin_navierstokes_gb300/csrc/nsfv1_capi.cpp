// Host side of the C ABI (include/nsfv1_gb300.h): the element-disc handle,
// its setters (same names, string ids and error behaviour as the reference's
// NavierStokesFV1 / NavierStokesBase / IncompressibleNavierStokesBase), the
// mesh set-up (block-CSR pattern, element colouring, device upload) and the
// assembly dispatch.
#include <algorithm>
#include <cctype>
#include <cstring>
#include <exception>
#include <stdexcept>
#include <string>
#include <vector>
#include "nsfv1_internal.h"
#include "nsfv1_refelem.cuh"
#include "nsfv1_host.h"
#include "../../include/nsfv1_gb300.h"

using namespace nsfv1;

namespace nsfv1 {

std::string lower_trim(const char* s) {
    std::string n = s ? s : "";
    const size_t a = n.find_first_not_of(" \t\n\r"), z = n.find_last_not_of(" \t\n\r");
    n = (a == std::string::npos) ? std::string() : n.substr(a, z - a + 1);
    std::transform(n.begin(), n.end(), n.begin(), [](unsigned char c) { return (char)std::tolower(c); });
    return n;
}

// CreateNavierStokesUpwind (upwind_interface.cpp:43-62), FV1 upwinds of this path
static int upwind_id(const char* name) {
    const std::string n = lower_trim(name);
    if (n == "no") return UPW_NO;
    if (n == "full") return UPW_FULL;
    if (n == "skewed") return UPW_SKEWED;
    if (n == "linearprofileskewed" || n == "lps") return UPW_LPS;
    if (n == "positive" || n == "pos") return UPW_POS;
    return -1;
}
// CreateNavierStokesStabilization (stabilization.cpp:46-57) + the "without" variant
static int stab_id(const char* name) {
    const std::string n = lower_trim(name);
    if (n == "fields") return STAB_FIELDS;
    if (n == "flow") return STAB_FLOW;
    if (n == "without" || n == "none") return STAB_WITHOUT;
    return -1;
}
// set_diffusion_length (stabilization.cpp:86-100)
static int difflen_id(const char* name) {
    const std::string n = lower_trim(name);
    if (n == "raw") return DL_RAW;
    if (n == "fivepoint") return DL_FIVEPOINT;
    if (n == "cor") return DL_COR;
    return -1;
}

int ref_dim(int roid) {
    return (roid == ROID_TRIANGLE || roid == ROID_QUADRILATERAL) ? 2 : (roid == ROID_TETRAHEDRON || roid == ROID_PRISM || roid == ROID_HEXAHEDRON) ? 3 : 0;
}
int ref_nsh(int roid) {
    switch (roid) {
        case ROID_TRIANGLE: return 3;
        case ROID_QUADRILATERAL: return 4;
        case ROID_TETRAHEDRON: return 4;
        case ROID_PRISM: return 6;
        case ROID_HEXAHEDRON: return 8;
    }
    return 0;
}

template <class T> static void dfree(T*& p) { if (p) cudaFree((void*)p); p = nullptr; }

template <class T> static cudaError_t dupload(T*& dst, const T* src, size_t n) {
    dfree(dst);
    if (n == 0) return cudaSuccess;
    cudaError_t e = cudaMalloc((void**)&dst, n * sizeof(T));
    if (e != cudaSuccess) { dst = nullptr; return e; }
    return cudaMemcpy((void*)dst, src, n * sizeof(T), cudaMemcpyHostToDevice);
}

void Disc::free_mesh() {
    dfree(d_coords); dfree(d_conn); dfree(d_elemBlk); dfree(d_colorElems); dfree(d_rowPtr); dfree(d_colIdx);
    dfree(d_dirRow); dfree(d_dirVal); dfree(d_diagPos); dfree(d_bjDinv); dfree(d_nuElem); dfree(d_bndFlux); dfree(d_nodeVol);
    free_outflow();
    outflowHost.clear();
    bndFluxHost.clear();
    dfree(d_instNode0); dfree(d_elemInst); dfree(d_nodeInst); dfree(d_instActive);
    nInst = 0; instNode0.clear(); instSkip = false;
    // the batched solver's levels, graphs and buffers belong to this mesh
    if (batch) { batch_free(batch); batch = nullptr; }
}

void Disc::free_outflow() {
    dfree(d_ofSeg); dfree(d_ofElem); dfree(d_ofLocal); dfree(d_ofXi); dfree(d_ofN);
    nOfSeg = 0;
}

// the outflow faces' terms (after the element loop, before the Dirichlet rows)
bool Disc::outflow_terms(const DiscParams& P, const double* u, double* d, void* vals, int prec, cudaStream_t s) {
    if (nOfSeg <= 0) return true;
    AsmArgs a{d_coords, d_conn, d_elemBlk, nullptr, 0, d_err, u, nullptr, d, vals, d_nuElem, nullptr, nullptr, nNodes, (int64_t)colIdx.size()};
    OutflowArgs o{nOfSeg, d_ofSeg, d_ofElem, d_ofLocal, d_ofXi, d_ofN};
    return cuda_ok(launch_outflow(roid, P, a, o, prec, s), "outflow boundary");
}

Disc::~Disc() {
    free_mesh();
    free_workspace();
    if (batch) { batch_free(batch); batch = nullptr; }
    dfree(d_err);
    dfree(d_ipws);
}

// The positive upwind's element path keeps the state of every SCVF of an element
// in a per-thread workspace: one slice per thread of a fixed launch width (one
// 64-thread CTA per SM), sized for the largest element type of the dimension.
// Allocated when such an upwind is set, so that no assembly call allocates.
bool Disc::ensure_ipws(bool force) {
    const bool need = force || convUpwindType == UPW_POS || stabUpwindType == UPW_POS;
    if (!need || d_ipws) return true;
    int dev = 0, sms = 0;
    if (!cuda_ok(cudaGetDevice(&dev), "device")) return false;
    if (!cuda_ok(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "SM count")) return false;
    const int64_t threads = (int64_t)sms * kIpwsCtaThreads;
    if (!cuda_ok(cudaMalloc(&d_ipws, sizeof(double) * (size_t)threads * ipws_doubles_host(dim)), "positive-upwind workspace")) {
        d_ipws = nullptr;
        return false;
    }
    ipwsThreads = threads;
    return true;
}

// Disc parameters for a launch; validates like prep_elem_loop (navier_stokes_fv1.cpp:136-199)
bool Disc::params(DiscParams& P, bool transient, double dt) {
    if (!stabSet) return fail(NSFV1_ERR_STATE, "Stabilization has not been set.");
    if (!stokes && !convUpwindSet) return fail(NSFV1_ERR_STATE, "Upwinding for convective Term in Momentum eq. not set.");
    if (!viscoSet) return fail(NSFV1_ERR_STATE, "NavierStokes::prep_elem_loop: Kinematic Viscosity has not been set, but is required.");
    if (!stokes && stabUpwindType < 0) return fail(NSFV1_ERR_STATE, "No upwind object");
    std::memset(&P, 0, sizeof(P));
    P.nu = nu; P.rho = rho; P.fullNewton = fullNewton; P.dt = dt;
    for (int d = 0; d < 3; ++d) P.src[d] = src[d];
    P.convUpwind = convUpwindType;
    P.stabUpwind = stabUpwindType < 0 ? convUpwindType : stabUpwindType;
    P.sameUpwind = stabSharesConv ? 1 : 0;
    P.stab = stabType; P.diffLen = diffLen;
    P.stokes = stokes; P.laplace = laplace; P.peclet = peclet; P.hasSource = hasSource; P.transient = transient ? 1 : 0;
    P.pac = pac ? 1 : 0;
    P.ipws = d_ipws;
    P.ipwsStride = ipwsThreads;
    return true;
}

// the positive-upwind workspace of a launch (allocated here at the latest)
bool Disc::bind_ipws(DiscParams& P) {
    if (!uses_ipshape(P) || P.ipws) return true;
    if (!ensure_ipws()) return false;
    P.ipws = d_ipws;
    P.ipwsStride = ipwsThreads;
    return true;
}

bool Disc::fail(int code, const std::string& msg) {
    status = code;
    lastError = msg;
    return false;
}

bool Disc::cuda_ok(cudaError_t e, const char* where) {
    if (e == cudaSuccess) return true;
    return fail(NSFV1_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

bool Disc::check_err_word(cudaStream_t s) {
    int err = 0;
    if (!cuda_ok(cudaMemcpyAsync(&err, d_err, sizeof(int), cudaMemcpyDeviceToHost, s), "error word")) return false;
    if (!cuda_ok(cudaStreamSynchronize(s), "sync")) return false;
    if (err & 4) {
        cudaMemsetAsync(d_err, 0, sizeof(int), s);
        return fail(NSFV1_ERR_ARGUMENT, "an index out of range was skipped (bounds-checked build)");
    }
    if (err & 1) {
        cudaMemsetAsync(d_err, 0, sizeof(int), s);
        return fail(NSFV1_ERR_GEOMETRY, "GetLinearProfileSkewedUpwindShapes: Cannot find cut side.");
    }
    if (err & 8) {
        // the non-diagonal stabilisation's ip-ip system (stabilization.cpp:299, 641)
        cudaMemsetAsync(d_err, 0, sizeof(int), s);
        return fail(NSFV1_ERR_BREAKDOWN, "Could not compute inverse.");
    }
    return true;
}

// block-CSR pattern: every node pair sharing an element, columns sorted
static void build_pattern(int nsh, int64_t nNodes, int64_t nElems, const int32_t* conn, std::vector<int32_t>& rowPtr,
                          std::vector<int32_t>& colIdx, std::vector<int32_t>& elemBlk) {
    // node -> incident elements
    std::vector<int64_t> nptr(nNodes + 1, 0);
    for (int64_t k = 0; k < nElems * nsh; ++k) nptr[conn[k] + 1]++;
    for (int64_t r = 0; r < nNodes; ++r) nptr[r + 1] += nptr[r];
    std::vector<int32_t> nel(nptr[nNodes]);
    {
        std::vector<int64_t> fill(nptr.begin(), nptr.end() - 1);
        for (int64_t e = 0; e < nElems; ++e)
            for (int i = 0; i < nsh; ++i) nel[fill[conn[e * nsh + i]]++] = (int32_t)e;
    }
    rowPtr.assign(nNodes + 1, 0);
    std::vector<int32_t> scratch;
    colIdx.clear();
    colIdx.reserve((size_t)nNodes * (nsh == 8 ? 27 : 9));
    for (int64_t r = 0; r < nNodes; ++r) {
        scratch.clear();
        for (int64_t k = nptr[r]; k < nptr[r + 1]; ++k) {
            const int64_t e = nel[k];
            for (int j = 0; j < nsh; ++j) scratch.push_back(conn[e * nsh + j]);
        }
        std::sort(scratch.begin(), scratch.end());
        scratch.erase(std::unique(scratch.begin(), scratch.end()), scratch.end());
        colIdx.insert(colIdx.end(), scratch.begin(), scratch.end());
        rowPtr[r + 1] = (int32_t)colIdx.size();
    }
    elemBlk.resize((size_t)nElems * nsh * nsh);
    for (int64_t e = 0; e < nElems; ++e)
        for (int i = 0; i < nsh; ++i) {
            const int32_t r = conn[e * nsh + i];
            const int32_t* b0 = colIdx.data() + rowPtr[r];
            const int32_t* b1 = colIdx.data() + rowPtr[r + 1];
            for (int j = 0; j < nsh; ++j)
                elemBlk[(e * nsh + i) * nsh + j] = (int32_t)(std::lower_bound(b0, b1, conn[e * nsh + j]) - colIdx.data());
        }
}

// Connectivity check of a mesh: every index in range and every node referenced
// by at least one element (an unreferenced node would get an empty block row
// without a diagonal block). Returns the error text, or nullptr.
static const char* check_connectivity(int nsh, int64_t nNodes, int64_t nElems, const int32_t* conn) {
    std::vector<uint8_t> used(nNodes, 0);
    for (int64_t k = 0; k < nElems * nsh; ++k) {
        if (conn[k] < 0 || conn[k] >= nNodes) return "connectivity out of range";
        used[conn[k]] = 1;
    }
    for (int64_t r = 0; r < nNodes; ++r)
        if (!used[r]) return "a node belongs to no element (its matrix row would have no diagonal block)";
    return nullptr;
}

// greedy colouring in element order: the smallest colour not used by an
// earlier element that shares a node
static int build_coloring(int nsh, int64_t nNodes, int64_t nElems, const int32_t* conn, std::vector<int32_t>& color) {
    std::vector<int64_t> nptr(nNodes + 1, 0);
    for (int64_t k = 0; k < nElems * nsh; ++k) nptr[conn[k] + 1]++;
    for (int64_t r = 0; r < nNodes; ++r) nptr[r + 1] += nptr[r];
    std::vector<int32_t> nel(nptr[nNodes]);
    {
        std::vector<int64_t> fill(nptr.begin(), nptr.end() - 1);
        for (int64_t e = 0; e < nElems; ++e)
            for (int i = 0; i < nsh; ++i) nel[fill[conn[e * nsh + i]]++] = (int32_t)e;
    }
    color.assign(nElems, -1);
    std::vector<int64_t> mark(256, -1);
    int nc = 0;
    for (int64_t e = 0; e < nElems; ++e) {
        for (int i = 0; i < nsh; ++i) {
            const int32_t n = conn[e * nsh + i];
            for (int64_t k = nptr[n]; k < nptr[n + 1]; ++k) {
                const int32_t o = nel[k];
                if (o < e && color[o] >= 0) mark[color[o]] = e;
            }
        }
        int c = 0;
        while (mark[c] == e) ++c;
        if (c >= 255) return -1;
        color[e] = c;
        nc = std::max(nc, c + 1);
    }
    return nc;
}

}  // namespace nsfv1

// ============================================================================
// C ABI
// ============================================================================
extern "C" {

int nsfv1_create(int dim, nsfv1_disc** out) {
    if (!out || (dim != 2 && dim != 3)) return NSFV1_ERR_ARGUMENT;
    try {
        Disc* h = new Disc();
        h->dim = dim;
        *out = reinterpret_cast<nsfv1_disc*>(h);
        return NSFV1_OK;
    } catch (...) { return NSFV1_ERR_ARGUMENT; }
}

int nsfv1_destroy(nsfv1_disc* h) {
    delete reinterpret_cast<Disc*>(h);
    return NSFV1_OK;
}

const char* nsfv1_last_error(const nsfv1_disc* h) {
    return h ? reinterpret_cast<const Disc*>(h)->lastError.c_str() : "null handle";
}

const char* nsfv1_disc_type(const nsfv1_disc*) { return "fv1"; }

#define NSFV1_H Disc* D = reinterpret_cast<Disc*>(h); if (!D) return NSFV1_ERR_ARGUMENT; D->status = NSFV1_OK

int nsfv1_set_kinematic_viscosity(nsfv1_disc* h, double nu) { NSFV1_H; D->nu = nu; D->viscoSet = true; return NSFV1_OK; }
int nsfv1_set_density(nsfv1_disc* h, double rho) { NSFV1_H; D->rho = rho; return NSFV1_OK; }
int nsfv1_set_source(nsfv1_disc* h, const double* f, int n) {
    NSFV1_H;
    if (!f || n != D->dim) { D->fail(NSFV1_ERR_ARGUMENT, "set_source: need exactly dim components"); return D->status; }
    D->hasSource = 1;
    for (int d = 0; d < 3; ++d) D->src[d] = d < n ? f[d] : 0.0;
    return NSFV1_OK;
}
int nsfv1_set_exact_jacobian(nsfv1_disc* h, double factor) { NSFV1_H; D->fullNewton = factor; return NSFV1_OK; }
int nsfv1_set_stokes(nsfv1_disc* h, int on) { NSFV1_H; D->stokes = on ? 1 : 0; return NSFV1_OK; }
int nsfv1_set_laplace(nsfv1_disc* h, int on) { NSFV1_H; D->laplace = on ? 1 : 0; return NSFV1_OK; }
int nsfv1_set_peclet_blend(nsfv1_disc* h, int on) { NSFV1_H; D->peclet = on ? 1 : 0; return NSFV1_OK; }

int nsfv1_set_upwind(nsfv1_disc* h, const char* name) {
    NSFV1_H;
    const int t = upwind_id(name);
    if (t < 0) {
        D->fail(NSFV1_ERR_ARGUMENT, std::string("NavierStokes: upwind type '") + (name ? name : "") +
                "' not found. Options are: no, full, skewed, LinearProfileSkewed (lps), positive (pos)");
        return D->status;
    }
    D->pac = false;   // set_upwind(name) clears the stabilisation-as-upwind (m_spConvStab = SPNULL)
    // navier_stokes_fv1.h:213-215: a new upwind object for the convection; a
    // stabilisation without an upwind gets this object, one that already has an
    // upwind keeps its (possibly previously shared) object and type
    D->convUpwindType = t; D->convUpwindSet = true;
    if (D->stabSet && D->stabUpwindType < 0) { D->stabUpwindType = t; D->stabSharesConv = true; }
    else D->stabSharesConv = false;
    if (D->d_err && !D->ensure_ipws()) return D->status;   // the device is in use: allocate now
    return NSFV1_OK;
}

int nsfv1_set_stabilization(nsfv1_disc* h, const char* name, const char* diff_length) {
    NSFV1_H;
    const int t = stab_id(name);
    if (t < 0) {
        D->fail(NSFV1_ERR_ARGUMENT, std::string("NavierStokes: stabilization type '") + (name ? name : "") +
                "' not a valid name of a Schneider-Raw stabilization. Options are: fields, flow");
        return D->status;
    }
    const int dl = diff_length ? difflen_id(diff_length) : DL_RAW;
    if (dl < 0) {
        D->fail(NSFV1_ERR_ARGUMENT, "Diffusion Length calculation method not found. Use one of [Raw, Fivepoint, Cor].");
        return D->status;
    }
    D->stabType = t; D->diffLen = dl; D->stabSet = true;
    // a new stabilisation object: it takes the convection upwind if one is set (navier_stokes_fv1.h:192,199)
    if (D->convUpwindSet) { D->stabUpwindType = D->convUpwindType; D->stabSharesConv = true; }
    else { D->stabUpwindType = -1; D->stabSharesConv = false; }
    return NSFV1_OK;
}

int nsfv1_set_pac_upwind(nsfv1_disc* h, int on) {
    NSFV1_H;
    if (!on) return NSFV1_OK;   // the reference's set_pac_upwind(false) changes nothing
    if (!D->convUpwindSet) { D->fail(NSFV1_ERR_STATE, "Upwind must be specified previously.\n"); return D->status; }
    if (!D->stabSet) { D->fail(NSFV1_ERR_STATE, "Stabilization must be specified previously.\n"); return D->status; }
    // navier_stokes_fv1.h:217-225: the stabilisation takes the convection upwind object and
    // becomes the convective upwind
    D->stabUpwindType = D->convUpwindType;
    D->stabSharesConv = true;
    D->pac = true;
    return NSFV1_OK;
}

int nsfv1_set_stabilization_upwind(nsfv1_disc* h, const char* name) {
    NSFV1_H;
    const int t = upwind_id(name);
    if (t < 0) { D->fail(NSFV1_ERR_ARGUMENT, std::string("NavierStokes: upwind type '") + (name ? name : "") + "' not found."); return D->status; }
    if (!D->stabSet) { D->fail(NSFV1_ERR_STATE, "Stabilization has not been set."); return D->status; }
    D->stabUpwindType = t; D->stabSharesConv = false;
    if (D->d_err && !D->ensure_ipws()) return D->status;   // the device is in use: allocate now
    return NSFV1_OK;
}

int nsfv1_set_mesh(nsfv1_disc* h, int elem_type, int64_t n_nodes, const double* coords, int64_t n_elems, const int32_t* conn) {
    NSFV1_H;
    try {
        const int dim = ref_dim(elem_type), nsh = ref_nsh(elem_type);
        if (dim == 0) { D->fail(NSFV1_ERR_ARGUMENT, "unsupported element type"); return D->status; }
        if (dim != D->dim) { D->fail(NSFV1_ERR_ARGUMENT, "element dimension does not match the disc"); return D->status; }
        if (n_nodes <= 0 || n_elems <= 0 || !coords || !conn) { D->fail(NSFV1_ERR_ARGUMENT, "empty mesh"); return D->status; }
        if (n_nodes >= (int64_t(1) << 31) / 4 || n_elems * nsh * nsh >= (int64_t(1) << 31)) { D->fail(NSFV1_ERR_ARGUMENT, "mesh too large for 32-bit indices"); return D->status; }
        if (const char* bad = check_connectivity(nsh, n_nodes, n_elems, conn)) { D->fail(NSFV1_ERR_ARGUMENT, bad); return D->status; }
        D->free_mesh();
        D->hasMesh = false;
        D->roid = elem_type; D->nsh = nsh; D->nNodes = n_nodes; D->nElems = n_elems;
        D->coordsHost.assign(coords, coords + n_nodes * dim);
        D->connHost.assign(conn, conn + n_elems * nsh);
        D->nuElemHost.clear(); D->dirRowHost.clear(); D->dirValHost.clear(); D->instCells.clear();
        build_pattern(nsh, n_nodes, n_elems, conn, D->rowPtr, D->colIdx, D->elemBlk);
        D->nColors = build_coloring(nsh, n_nodes, n_elems, conn, D->color);
        if (D->nColors < 0) { D->fail(NSFV1_ERR_ARGUMENT, "too many element colours"); return D->status; }
        D->colorPtr.assign(D->nColors + 1, 0);
        for (int64_t e = 0; e < n_elems; ++e) D->colorPtr[D->color[e] + 1]++;
        for (int c = 0; c < D->nColors; ++c) D->colorPtr[c + 1] += D->colorPtr[c];
        D->colorElems.resize(n_elems);
        {
            std::vector<int32_t> f(D->colorPtr.begin(), D->colorPtr.end() - 1);
            for (int64_t e = 0; e < n_elems; ++e) D->colorElems[f[D->color[e]]++] = (int32_t)e;
        }
        if (!D->cuda_ok(dupload(D->d_coords, coords, (size_t)n_nodes * dim), "upload coords") ||
            !D->cuda_ok(dupload(D->d_conn, conn, (size_t)n_elems * nsh), "upload conn") ||
            !D->cuda_ok(dupload(D->d_elemBlk, D->elemBlk.data(), D->elemBlk.size()), "upload elemBlk") ||
            !D->cuda_ok(dupload(D->d_colorElems, D->colorElems.data(), D->colorElems.size()), "upload colours") ||
            !D->cuda_ok(dupload(D->d_rowPtr, D->rowPtr.data(), D->rowPtr.size()), "upload rowPtr") ||
            !D->cuda_ok(dupload(D->d_colIdx, D->colIdx.data(), D->colIdx.size()), "upload colIdx"))
            return D->status;
        {
            std::vector<int32_t> dp(n_nodes);
            for (int64_t r = 0; r < n_nodes; ++r) {
                int32_t q = D->rowPtr[r];
                while (q < D->rowPtr[r + 1] && D->colIdx[q] != r) ++q;
                if (q == D->rowPtr[r + 1]) { D->fail(NSFV1_ERR_ARGUMENT, "a matrix row has no diagonal block"); return D->status; }
                dp[r] = q;
            }
            if (!D->cuda_ok(dupload(D->d_diagPos, dp.data(), dp.size()), "upload diagPos")) return D->status;
        }
        if (!D->d_err) {
            if (!D->cuda_ok(cudaMalloc((void**)&D->d_err, sizeof(int)), "alloc err")) return D->status;
        }
        if (!D->cuda_ok(cudaMemset(D->d_err, 0, sizeof(int)), "memset err")) return D->status;
        if (!D->ensure_ipws()) return D->status;
        D->nDir = 0;
        D->free_workspace();
        D->hasMesh = true;
        return NSFV1_OK;
    } catch (std::exception& ex) {
        D->fail(NSFV1_ERR_ARGUMENT, ex.what());
        return D->status;
    }
}

int nsfv1_pattern_info(const nsfv1_disc* h, int64_t* n_rows, int64_t* nnz_blocks, int* block_size, int* n_colors) {
    const Disc* D = reinterpret_cast<const Disc*>(h);
    if (!D || !D->hasMesh) return NSFV1_ERR_STATE;
    if (n_rows) *n_rows = D->nNodes;
    if (nnz_blocks) *nnz_blocks = (int64_t)D->colIdx.size();
    if (block_size) *block_size = D->dim + 1;
    if (n_colors) *n_colors = D->nColors;
    return NSFV1_OK;
}

int nsfv1_mesh_pattern(int elem_type, int64_t n_nodes, int64_t n_elems, const int32_t* conn, int64_t* nnz_blocks,
                       int* n_colors, int32_t* row_ptr, int32_t* col_idx, int32_t* elem_color) {
    const int nsh = ref_nsh(elem_type);
    if (nsh == 0 || n_nodes <= 0 || n_elems <= 0 || !conn) return NSFV1_ERR_ARGUMENT;
    try {
        if (check_connectivity(nsh, n_nodes, n_elems, conn)) return NSFV1_ERR_ARGUMENT;
        std::vector<int32_t> rp, ci, eb, col;
        build_pattern(nsh, n_nodes, n_elems, conn, rp, ci, eb);
        const int nc = build_coloring(nsh, n_nodes, n_elems, conn, col);
        if (nc < 0) return NSFV1_ERR_ARGUMENT;
        if (nnz_blocks) *nnz_blocks = (int64_t)ci.size();
        if (n_colors) *n_colors = nc;
        if (row_ptr) std::copy(rp.begin(), rp.end(), row_ptr);
        if (col_idx) std::copy(ci.begin(), ci.end(), col_idx);
        if (elem_color) std::copy(col.begin(), col.end(), elem_color);
        return NSFV1_OK;
    } catch (...) { return NSFV1_ERR_ARGUMENT; }
}

int nsfv1_get_pattern(const nsfv1_disc* h, int32_t* row_ptr, int32_t* col_idx) {
    const Disc* D = reinterpret_cast<const Disc*>(h);
    if (!D || !D->hasMesh) return NSFV1_ERR_STATE;
    if (row_ptr) std::copy(D->rowPtr.begin(), D->rowPtr.end(), row_ptr);
    if (col_idx) std::copy(D->colIdx.begin(), D->colIdx.end(), col_idx);
    return NSFV1_OK;
}

int nsfv1_get_coloring(const nsfv1_disc* h, int32_t* elem_color) {
    const Disc* D = reinterpret_cast<const Disc*>(h);
    if (!D || !D->hasMesh) return NSFV1_ERR_STATE;
    std::copy(D->color.begin(), D->color.end(), elem_color);
    return NSFV1_OK;
}

int nsfv1_device_pattern(const nsfv1_disc* h, const int32_t** row_ptr, const int32_t** col_idx) {
    const Disc* D = reinterpret_cast<const Disc*>(h);
    if (!D || !D->hasMesh) return NSFV1_ERR_STATE;
    if (row_ptr) *row_ptr = D->d_rowPtr;
    if (col_idx) *col_idx = D->d_colIdx;
    return NSFV1_OK;
}

int nsfv1_set_dirichlet(nsfv1_disc* h, int64_t n, const int32_t* dofs, const double* values) {
    NSFV1_H;
    if (!D->hasMesh) { D->fail(NSFV1_ERR_STATE, "set_dirichlet: no mesh"); return D->status; }
    const int b = D->dim + 1;
    for (int64_t k = 0; k < n; ++k)
        if (dofs[k] < 0 || dofs[k] >= D->nNodes * b) { D->fail(NSFV1_ERR_ARGUMENT, "Dirichlet dof out of range"); return D->status; }
    if (!D->cuda_ok(dupload(D->d_dirRow, dofs, (size_t)n), "upload dirichlet") ||
        !D->cuda_ok(dupload(D->d_dirVal, values, (size_t)n), "upload dirichlet values"))
        return D->status;
    D->nDir = n;
    D->dirRowHost.assign(dofs, dofs + n);
    D->dirValHost.assign(values, values + n);
    return NSFV1_OK;
}

}  // extern "C"

namespace {

// merges Dirichlet rows into the handle's (a later value of the same dof wins), rows sorted by dof
int merge_dirichlet(nsfv1_disc* h, Disc* D, const std::vector<int32_t>& dofs, const std::vector<double>& vals) {
    std::vector<std::pair<int32_t, double>> all;
    for (size_t k = 0; k < D->dirRowHost.size(); ++k) all.emplace_back(D->dirRowHost[k], D->dirValHost[k]);
    for (size_t k = 0; k < dofs.size(); ++k) all.emplace_back(dofs[k], vals[k]);
    std::stable_sort(all.begin(), all.end(), [](const auto& a, const auto& c) { return a.first < c.first; });
    std::vector<int32_t> rows;
    std::vector<double> v;
    for (size_t k = 0; k < all.size(); ++k) {
        if (!rows.empty() && rows.back() == all[k].first) v.back() = all[k].second;
        else { rows.push_back(all[k].first); v.push_back(all[k].second); }
    }
    return nsfv1_set_dirichlet(h, (int64_t)rows.size(), rows.data(), v.data());
}

// FV1 boundary faces of one element side (ugcore's boundary faces of the box
// dual mesh, restated): side corner a owns the part {a, mid(a, next), side centre,
// mid(prev, a)} (2D: {a, mid(a, other)}); its normal is area-weighted and points
// out of the element. nrm[j][d] receives the normal of side corner j.
bool side_bf_normals(int dim, int nco, const double (*x)[3], const double* elemCentre, double (*nrm)[3]) {
    double sc[3] = {0, 0, 0};
    for (int j = 0; j < nco; ++j)
        for (int d = 0; d < 3; ++d) sc[d] += x[j][d] / nco;
    for (int j = 0; j < nco; ++j) {
        for (int d = 0; d < 3; ++d) nrm[j][d] = 0.0;
        if (dim == 2) {
            const double* a = x[j];
            const double* o = x[1 - j];
            const double m[2] = {0.5 * (a[0] + o[0]), 0.5 * (a[1] + o[1])};
            nrm[j][0] = m[1] - a[1];
            nrm[j][1] = -(m[0] - a[0]);
        } else {
            const double* a = x[j];
            const double* nx = x[(j + 1) % nco];
            const double* pv = x[(j + nco - 1) % nco];
            double mn[3], mp[3], d1[3], d2[3];
            for (int d = 0; d < 3; ++d) {
                mn[d] = 0.5 * (a[d] + nx[d]); mp[d] = 0.5 * (pv[d] + a[d]);
                d1[d] = sc[d] - a[d]; d2[d] = mp[d] - mn[d];
            }
            nrm[j][0] = 0.5 * (d1[1] * d2[2] - d1[2] * d2[1]);
            nrm[j][1] = 0.5 * (d1[2] * d2[0] - d1[0] * d2[2]);
            nrm[j][2] = 0.5 * (d1[0] * d2[1] - d1[1] * d2[0]);
        }
        double dot = 0;
        for (int d = 0; d < dim; ++d) dot += nrm[j][d] * (sc[d] - elemCentre[d]);
        if (dot < 0) for (int d = 0; d < 3; ++d) nrm[j][d] = -nrm[j][d];
        if (!(dot != 0.0)) return false;   // degenerate side (or NaN)
    }
    return true;
}

// The element of every boundary side (the one element that has all of its nodes);
// false (with the disc's error set) for a bad side.
bool side_owners(Disc* D, int64_t n_sides, int side_nco, const int32_t* side_nodes, const std::string& who, std::vector<int64_t>& owner) {
    const int dim = D->dim, nsh = D->nsh;
    if (n_sides < 0 || (n_sides > 0 && !side_nodes) || (dim == 2 && side_nco != 2) || (dim == 3 && side_nco != 3 && side_nco != 4))
        return D->fail(NSFV1_ERR_ARGUMENT, who + ": sides of 2 (2D) or 3 / 4 (3D) nodes");
    for (int64_t k = 0; k < n_sides * side_nco; ++k)
        if (side_nodes[k] < 0 || side_nodes[k] >= D->nNodes) return D->fail(NSFV1_ERR_ARGUMENT, who + ": node out of range");
    std::vector<int64_t> nptr(D->nNodes + 1, 0);
    for (int64_t k = 0; k < D->nElems * nsh; ++k) nptr[D->connHost[k] + 1]++;
    for (int64_t r = 0; r < D->nNodes; ++r) nptr[r + 1] += nptr[r];
    std::vector<int32_t> nel(nptr[D->nNodes]);
    {
        std::vector<int64_t> fill(nptr.begin(), nptr.end() - 1);
        for (int64_t e = 0; e < D->nElems; ++e)
            for (int i = 0; i < nsh; ++i) nel[fill[D->connHost[e * nsh + i]]++] = (int32_t)e;
    }
    owner.assign(n_sides, -1);
    for (int64_t sIdx = 0; sIdx < n_sides; ++sIdx) {
        const int32_t* sn = side_nodes + sIdx * side_nco;
        int owners = 0;
        for (int64_t q = nptr[sn[0]]; q < nptr[sn[0] + 1]; ++q) {
            const int64_t e = nel[q];
            bool all = true;
            for (int j = 1; j < side_nco && all; ++j) {
                bool has = false;
                for (int i = 0; i < nsh; ++i) has |= D->connHost[e * nsh + i] == sn[j];
                all = has;
            }
            if (all) { owner[sIdx] = e; ++owners; }
        }
        if (owners != 1)
            return D->fail(NSFV1_ERR_ARGUMENT, who + ": side " + std::to_string(sIdx) + " is not a boundary side of exactly one element");
    }
    return true;
}

double ref_co(int roid, int c, int d) {
    switch (roid) {
        case ROID_TRIANGLE: return Ref<ROID_TRIANGLE>::co(c, d);
        case ROID_QUADRILATERAL: return Ref<ROID_QUADRILATERAL>::co(c, d);
        case ROID_TETRAHEDRON: return Ref<ROID_TETRAHEDRON>::co(c, d);
        case ROID_PRISM: return Ref<ROID_PRISM>::co(c, d);
        case ROID_HEXAHEDRON: return Ref<ROID_HEXAHEDRON>::co(c, d);
    }
    return 0.0;
}

}  // namespace

extern "C" {

int nsfv1_add_outflow(nsfv1_disc* h, int64_t n_sides, int side_nco, const int32_t* side_nodes) {
    NSFV1_H;
    const int dim = D->dim, nsh = D->nsh;
    const std::string who = "NavierStokesNoNormalStressOutflow::add";
    if (!D->hasMesh) { D->fail(NSFV1_ERR_STATE, who + ": no mesh"); return D->status; }
    std::vector<int64_t> owner;
    if (!side_owners(D, n_sides, side_nco, side_nodes, who, owner)) return D->status;
    for (int64_t sIdx = 0; sIdx < n_sides; ++sIdx) {
        const int32_t* sn = side_nodes + sIdx * side_nco;
        const int64_t e = owner[sIdx];
        double x[4][3] = {{0}}, cen[3] = {0, 0, 0}, nrm[4][3], lx[4][3] = {{0}}, lsc[3] = {0, 0, 0};
        int loc[4] = {0, 0, 0, 0};
        for (int j = 0; j < side_nco; ++j) {
            for (int d = 0; d < dim; ++d) x[j][d] = D->coordsHost[(size_t)sn[j] * dim + d];
            for (int i = 0; i < nsh; ++i)
                if (D->connHost[e * nsh + i] == sn[j]) loc[j] = i;
            for (int d = 0; d < dim; ++d) {
                lx[j][d] = ref_co(D->roid, loc[j], d);
                lsc[d] += lx[j][d] / side_nco;
            }
        }
        for (int i = 0; i < nsh; ++i)
            for (int d = 0; d < dim; ++d) cen[d] += D->coordsHost[(size_t)D->connHost[e * nsh + i] * dim + d] / nsh;
        if (!side_bf_normals(dim, side_nco, x, cen, nrm)) {
            D->fail(NSFV1_ERR_GEOMETRY, who + ": degenerate side " + std::to_string(sIdx));
            return D->status;
        }
        for (int j = 0; j < side_nco; ++j) {
            // the face {corner, side-edge midpoints, side centre}: its integration point is the
            // mean of those points in local coordinates (2D: {corner, side midpoint})
            Disc::OutflowFace f;
            f.node = sn[j];
            f.elem = (int32_t)e;
            f.local = loc[j];
            for (int d = 0; d < 3; ++d) { f.n[d] = nrm[j][d]; f.xi[d] = 0.0; }
            if (dim == 2) {
                const int o = 1 - j;
                for (int d = 0; d < 2; ++d) f.xi[d] = 0.5 * (lx[j][d] + 0.5 * (lx[j][d] + lx[o][d]));
            } else {
                const int nx = (j + 1) % side_nco, pv = (j + side_nco - 1) % side_nco;
                for (int d = 0; d < 3; ++d)
                    f.xi[d] = 0.25 * (lx[j][d] + 0.5 * (lx[j][d] + lx[nx][d]) + lsc[d] + 0.5 * (lx[pv][d] + lx[j][d]));
            }
            D->outflowHost.push_back(f);
        }
    }
    // faces grouped by node (stable: a node's faces keep the order they were added in)
    std::vector<Disc::OutflowFace> fs = D->outflowHost;
    std::stable_sort(fs.begin(), fs.end(), [](const Disc::OutflowFace& a, const Disc::OutflowFace& c) { return a.node < c.node; });
    std::vector<int32_t> seg, el, lo;
    std::vector<double> xi, nr;
    for (size_t k = 0; k < fs.size(); ++k) {
        if (k == 0 || fs[k].node != fs[k - 1].node) seg.push_back((int32_t)k);
        el.push_back(fs[k].elem);
        lo.push_back(fs[k].local);
        for (int d = 0; d < 3; ++d) { xi.push_back(fs[k].xi[d]); nr.push_back(fs[k].n[d]); }
    }
    seg.push_back((int32_t)fs.size());
    D->free_outflow();
    if (!D->cuda_ok(dupload(D->d_ofSeg, seg.data(), seg.size()), "outflow") || !D->cuda_ok(dupload(D->d_ofElem, el.data(), el.size()), "outflow") ||
        !D->cuda_ok(dupload(D->d_ofLocal, lo.data(), lo.size()), "outflow") || !D->cuda_ok(dupload(D->d_ofXi, xi.data(), xi.size()), "outflow") ||
        !D->cuda_ok(dupload(D->d_ofN, nr.data(), nr.size()), "outflow"))
        return D->status;
    D->nOfSeg = (int32_t)seg.size() - 1;
    return NSFV1_OK;
}

int nsfv1_add_dirichlet(nsfv1_disc* h, int64_t n, const int32_t* dofs, const double* values) {
    NSFV1_H;
    if (!D->hasMesh) { D->fail(NSFV1_ERR_STATE, "add_dirichlet: no mesh"); return D->status; }
    if (n < 0 || (n > 0 && (!dofs || !values))) { D->fail(NSFV1_ERR_ARGUMENT, "add_dirichlet: bad arguments"); return D->status; }
    const int b = D->dim + 1;
    for (int64_t k = 0; k < n; ++k)
        if (dofs[k] < 0 || dofs[k] >= D->nNodes * b) { D->fail(NSFV1_ERR_ARGUMENT, "Dirichlet dof out of range"); return D->status; }
    return merge_dirichlet(h, D, std::vector<int32_t>(dofs, dofs + n), std::vector<double>(values, values + n));
}

int nsfv1_add_wall(nsfv1_disc* h, int64_t n, const int32_t* nodes) {
    NSFV1_H;
    if (!D->hasMesh) { D->fail(NSFV1_ERR_STATE, "NavierStokesWall::add: no mesh"); return D->status; }
    if (n < 0 || (n > 0 && !nodes)) { D->fail(NSFV1_ERR_ARGUMENT, "NavierStokesWall::add: bad arguments"); return D->status; }
    const int b = D->dim + 1;
    std::vector<int32_t> dofs;
    std::vector<double> vals;
    for (int64_t k = 0; k < n; ++k) {
        if (nodes[k] < 0 || nodes[k] >= D->nNodes) { D->fail(NSFV1_ERR_ARGUMENT, "NavierStokesWall::add: node out of range"); return D->status; }
        for (int d = 0; d < D->dim; ++d) { dofs.push_back(nodes[k] * b + d); vals.push_back(0.0); }
    }
    return merge_dirichlet(h, D, dofs, vals);
}

int nsfv1_add_inflow(nsfv1_disc* h, int64_t n_sides, int side_nco, const int32_t* side_nodes, const double* vel) {
    NSFV1_H;
    const int dim = D->dim, b = dim + 1, nsh = D->nsh;
    if (!D->hasMesh) { D->fail(NSFV1_ERR_STATE, "NavierStokesInflow::add: no mesh"); return D->status; }
    if (n_sides > 0 && !vel) { D->fail(NSFV1_ERR_ARGUMENT, "NavierStokesInflow::add: a velocity of dim components is needed"); return D->status; }
    std::vector<int64_t> owners;
    if (!side_owners(D, n_sides, side_nco, side_nodes, "NavierStokesInflow::add", owners)) return D->status;
    std::vector<double> flux = D->bndFluxHost;
    flux.resize(D->nNodes, 0.0);
    std::vector<int32_t> dofs;
    std::vector<double> vals;
    for (int64_t sIdx = 0; sIdx < n_sides; ++sIdx) {
        const int32_t* sn = side_nodes + sIdx * side_nco;
        const int64_t owner = owners[sIdx];
        double x[4][3] = {{0}}, cen[3] = {0, 0, 0}, nrm[4][3];
        for (int j = 0; j < side_nco; ++j)
            for (int d = 0; d < dim; ++d) x[j][d] = D->coordsHost[(size_t)sn[j] * dim + d];
        for (int i = 0; i < nsh; ++i)
            for (int d = 0; d < dim; ++d) cen[d] += D->coordsHost[(size_t)D->connHost[owner * nsh + i] * dim + d] / nsh;
        if (!side_bf_normals(dim, side_nco, x, cen, nrm)) {
            D->fail(NSFV1_ERR_GEOMETRY, "NavierStokesInflow::add: degenerate side " + std::to_string(sIdx));
            return D->status;
        }
        for (int j = 0; j < side_nco; ++j) {
            double vn = 0.0;
            for (int d = 0; d < dim; ++d) vn += vel[d] * nrm[j][d];
            flux[sn[j]] += vn;
            for (int d = 0; d < dim; ++d) { dofs.push_back(sn[j] * b + d); vals.push_back(vel[d]); }
        }
    }
    if (!D->cuda_ok(dupload(D->d_bndFlux, flux.data(), flux.size()), "upload inflow flux")) return D->status;
    D->bndFluxHost.swap(flux);
    return merge_dirichlet(h, D, dofs, vals);
}

int nsfv1_clear_boundary(nsfv1_disc* h) {
    NSFV1_H;
    D->free_outflow();
    D->outflowHost.clear();
    dfree(D->d_bndFlux);
    D->bndFluxHost.clear();
    dfree(D->d_dirRow);
    dfree(D->d_dirVal);
    D->dirRowHost.clear();
    D->dirValHost.clear();
    D->nDir = 0;
    return NSFV1_OK;
}

int nsfv1_assemble_defect(nsfv1_disc* h, const double* u, const double* u_old, double dt, double* d, void* stream) {
    NSFV1_H;
    return D->assemble_defect(u, u_old, dt, d, (cudaStream_t)stream) ? NSFV1_OK : D->status;
}

int nsfv1_assemble_jacobian(nsfv1_disc* h, const double* u, const double* u_old, double dt, void* vals, int prec, void* stream) {
    NSFV1_H;
    return D->assemble_jacobian(u, u_old, dt, vals, prec, (cudaStream_t)stream) ? NSFV1_OK : D->status;
}

int nsfv1_assemble_defect_jacobian(nsfv1_disc* h, const double* u, const double* u_old, double dt, double* d, void* vals, int prec,
                                   void* stream) {
    NSFV1_H;
    return D->assemble_defect_jacobian(u, u_old, dt, d, vals, prec, (cudaStream_t)stream) ? NSFV1_OK : D->status;
}

int nsfv1_elem_batch(nsfv1_disc* h, int elem_type, int64_t n, const double* corners, const double* u, const double* u_old,
                     double dt, double* defA, double* jacA, double* defM, double* jacM, double* rhs, void* stream) {
    NSFV1_H;
    if (ref_dim(elem_type) != D->dim) { D->fail(NSFV1_ERR_ARGUMENT, "element dimension does not match the disc"); return D->status; }
    if (n < 0 || (n > 0 && (!corners || !u))) { D->fail(NSFV1_ERR_ARGUMENT, "elem_batch: bad arguments"); return D->status; }
    DiscParams P;
    if (!D->params(P, u_old != nullptr, dt)) return D->status;
    if (!D->d_err) {
        if (!D->cuda_ok(cudaMalloc((void**)&D->d_err, sizeof(int)), "alloc err")) return D->status;
        cudaMemset(D->d_err, 0, sizeof(int));
    }
    if (n > 0 && !D->bind_ipws(P)) return D->status;
    ElemBatchArgs a{n, corners, u, u_old, defA, jacA, defM, jacM, rhs, D->d_err};
    cudaStream_t s = (cudaStream_t)stream;
    if (!D->cuda_ok(launch_elem_batch(elem_type, P, a, s), "elem_batch")) return D->status;
    return D->check_err_word(s) ? NSFV1_OK : D->status;
}

int nsfv1_export(nsfv1_disc* h, int which, int elem_type, int64_t n, const double* corners, const double* u, const double* u_old, double dt,
                 int ip_kind, int nip, const double* local_ips, double* values, double* derivs, void* stream) {
    NSFV1_H;
    const int dim = ref_dim(elem_type);
    if (dim != D->dim) { D->fail(NSFV1_ERR_ARGUMENT, "element dimension does not match the disc"); return D->status; }
    if (which < NSFV1_EX_VELOCITY || which > NSFV1_EX_PRESSURE_GRAD) { D->fail(NSFV1_ERR_ARGUMENT, "export: unknown export id"); return D->status; }
    if (ip_kind < NSFV1_IPS_SCVF || ip_kind > NSFV1_IPS_GIVEN) { D->fail(NSFV1_ERR_ARGUMENT, "export: unknown kind of points"); return D->status; }
    if (ip_kind == NSFV1_IPS_GIVEN && (nip < 1 || nip > kMaxExportPoints || !local_ips)) {
        D->fail(NSFV1_ERR_ARGUMENT, "export: 1 to " + std::to_string(kMaxExportPoints) + " given local points needed");
        return D->status;
    }
    if (n < 0 || (n > 0 && (!corners || !u || !values))) { D->fail(NSFV1_ERR_ARGUMENT, "export: bad arguments"); return D->status; }
    DiscParams P;
    if (!D->params(P, u_old != nullptr, dt)) return D->status;
    if (n == 0) return NSFV1_OK;
    if (!D->d_err) {
        if (!D->cuda_ok(cudaMalloc((void**)&D->d_err, sizeof(int)), "alloc err")) return D->status;
        cudaMemset(D->d_err, 0, sizeof(int));
    }
    // the per-SCVF state of the stabilised ip velocity lives in the element path's workspace
    if (!D->ensure_ipws(true)) return D->status;
    P.ipws = D->d_ipws;
    P.ipwsStride = D->ipwsThreads;
    ExportArgs a{};
    a.which = which; a.ipKind = ip_kind; a.nip = ip_kind == NSFV1_IPS_GIVEN ? nip : 0; a.n = n;
    a.corners = corners; a.u = u; a.uold = u_old; a.values = values; a.derivs = derivs; a.err = D->d_err;
    if (ip_kind == NSFV1_IPS_GIVEN)
        for (int i = 0; i < nip; ++i)
            for (int d = 0; d < 3; ++d) a.lips[i][d] = d < dim ? local_ips[i * dim + d] : 0.0;
    cudaStream_t s = (cudaStream_t)stream;
    if (!D->cuda_ok(launch_export(elem_type, P, a, s), "export")) return D->status;
    return D->check_err_word(s) ? NSFV1_OK : D->status;
}

int nsfv1_vorticity(nsfv1_disc* h, const double* u, double* vort, void* stream) {
    NSFV1_H;
    if (!D->hasMesh) { D->fail(NSFV1_ERR_STATE, "vorticity: no mesh set"); return D->status; }
    if (!u || !vort) { D->fail(NSFV1_ERR_ARGUMENT, "vorticity: null vector"); return D->status; }
    cudaStream_t s = (cudaStream_t)stream;
    if (!D->d_nodeVol && !D->cuda_ok(cudaMalloc((void**)&D->d_nodeVol, sizeof(double) * D->nNodes), "vorticity scratch")) return D->status;
    if (!D->cuda_ok(cudaMemsetAsync(vort, 0, sizeof(double) * D->nNodes, s), "memset") ||
        !D->cuda_ok(cudaMemsetAsync(D->d_nodeVol, 0, sizeof(double) * D->nNodes, s), "memset"))
        return D->status;
    for (int c = 0; c < D->nColors; ++c) {
        AsmArgs a{D->d_coords, D->d_conn, D->d_elemBlk, D->d_colorElems + D->colorPtr[c], D->colorPtr[c + 1] - D->colorPtr[c], D->d_err,
                  u, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, D->nNodes, (int64_t)D->colIdx.size()};
        if (!D->cuda_ok(launch_vorticity(D->roid, a, vort, D->d_nodeVol, s), "vorticity")) return D->status;
    }
    if (!D->cuda_ok(launch_divide(D->nNodes, vort, D->d_nodeVol, s), "vorticity")) return D->status;
    return D->check_err_word(s) ? NSFV1_OK : D->status;
}

int nsfv1_eval_points(nsfv1_disc* h, const double* u, int64_t n, const double* points, int fct, double* values, void* stream) {
    NSFV1_H;
    if (!D->hasMesh) { D->fail(NSFV1_ERR_STATE, "eval_points: no mesh set"); return D->status; }
    if (n < 0 || (n > 0 && (!u || !points || !values)) || fct < 0 || fct > D->dim) {
        D->fail(NSFV1_ERR_ARGUMENT, "eval_points: bad arguments");
        return D->status;
    }
    cudaStream_t s = (cudaStream_t)stream;
    if (!D->cuda_ok(launch_eval_points(D->roid, D->nElems, D->nNodes, D->d_coords, D->d_conn, u, n, points, fct, values, s), "eval_points"))
        return D->status;
    return D->cuda_ok(cudaStreamSynchronize(s), "eval_points") ? NSFV1_OK : D->status;
}

int nsfv1_elem_batch_host(nsfv1_disc* h, int elem_type, int64_t n, const double* corners, const double* u, const double* u_old,
                          double dt, double* defA, double* jacA, double* defM, double* jacM, double* rhs) {
    NSFV1_H;
    const int dim = ref_dim(elem_type), nsh = ref_nsh(elem_type);
    if (dim != D->dim) { D->fail(NSFV1_ERR_ARGUMENT, "element dimension does not match the disc"); return D->status; }
    if (n < 0 || (n > 0 && (!corners || !u))) { D->fail(NSFV1_ERR_ARGUMENT, "elem_batch_host: bad arguments"); return D->status; }
    {
        DiscParams P;   // the setup checks of prep_elem_loop, also for an empty batch
        if (!D->params(P, u_old != nullptr, dt)) return D->status;
    }
    if (n == 0) return NSFV1_OK;
    const size_t nloc = (size_t)(dim + 1) * nsh, nc = (size_t)n * nsh * dim, nv = (size_t)n * nloc, nm = (size_t)n * nloc * nloc;
    // device staging: corners, u, u_old, and every requested output
    const size_t total = nc + nv * (u_old ? 2 : 1) + (defA ? nv : 0) + (defM ? nv : 0) + (rhs ? nv : 0) + (jacA ? nm : 0) + (jacM ? nm : 0);
    double* buf = nullptr;
    if (!D->cuda_ok(cudaMalloc((void**)&buf, total * sizeof(double)), "elem_batch_host: staging")) return D->status;
    double* p = buf;
    auto take = [&](size_t cnt) { double* q = p; p += cnt; return q; };
    double* dC = take(nc);
    double* dU = take(nv);
    double* dUo = u_old ? take(nv) : nullptr;
    double* dDA = defA ? take(nv) : nullptr;
    double* dDM = defM ? take(nv) : nullptr;
    double* dR = rhs ? take(nv) : nullptr;
    double* dJA = jacA ? take(nm) : nullptr;
    double* dJM = jacM ? take(nm) : nullptr;
    bool ok = D->cuda_ok(cudaMemcpy(dC, corners, nc * 8, cudaMemcpyHostToDevice), "elem_batch_host: copy") &&
              D->cuda_ok(cudaMemcpy(dU, u, nv * 8, cudaMemcpyHostToDevice), "elem_batch_host: copy") &&
              (!u_old || D->cuda_ok(cudaMemcpy(dUo, u_old, nv * 8, cudaMemcpyHostToDevice), "elem_batch_host: copy"));
    if (ok) ok = nsfv1_elem_batch(h, elem_type, n, dC, dU, dUo, dt, dDA, dJA, dDM, dJM, dR, nullptr) == NSFV1_OK;
    auto back = [&](double* host, const double* dev, size_t cnt) {
        return !host || D->cuda_ok(cudaMemcpy(host, dev, cnt * 8, cudaMemcpyDeviceToHost), "elem_batch_host: copy back");
    };
    if (ok) ok = back(defA, dDA, nv) && back(defM, dDM, nv) && back(rhs, dR, nv) && back(jacA, dJA, nm) && back(jacM, dJM, nm);
    const int st = D->status;
    cudaFree(buf);
    return ok ? NSFV1_OK : (st ? st : NSFV1_ERR_CUDA);
}

int nsfv1_set_assembly_threads(nsfv1_disc* h, int threads) {
    Disc* D = reinterpret_cast<Disc*>(h);
    if (!D) return NSFV1_ERR_ARGUMENT;
    D->status = NSFV1_OK;
    if (threads < 32 || threads > 128 || threads % 32) {
        D->fail(NSFV1_ERR_ARGUMENT, "set_assembly_threads: 32, 64, 96 or 128");
        return D->status;
    }
    D->asmThreads = threads;
    return NSFV1_OK;
}

int nsfv1_get_assembly_threads(const nsfv1_disc* h) {
    const Disc* D = reinterpret_cast<const Disc*>(h);
    return D ? D->asmThreads : 0;
}

int nsfv1_assembly_autotune(nsfv1_disc* h, const double* u, int prec, const int* candidates, int n_candidates, double* ms, void* stream) {
    Disc* D = reinterpret_cast<Disc*>(h);
    if (!D) return NSFV1_ERR_ARGUMENT;
    D->status = NSFV1_OK;
    if (!D->hasMesh) { D->fail(NSFV1_ERR_STATE, "assembly_autotune: no mesh"); return D->status; }
    if (!u || !candidates || n_candidates <= 0 || (prec != NSFV1_F64 && prec != NSFV1_F32)) {
        D->fail(NSFV1_ERR_ARGUMENT, "assembly_autotune: bad arguments");
        return D->status;
    }
    for (int c = 0; c < n_candidates; ++c)
        if (candidates[c] < 32 || candidates[c] > 128 || candidates[c] % 32) {
            D->fail(NSFV1_ERR_ARGUMENT, "assembly_autotune: candidates must be 32, 64, 96 or 128");
            return D->status;
        }
    cudaStream_t s = (cudaStream_t)stream;
    const int b = D->dim + 1;
    const size_t vbytes = D->colIdx.size() * b * b * (prec == NSFV1_F64 ? 8 : 4);
    void* J = nullptr;
    double* d = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    bool ok = D->cuda_ok(cudaMalloc(&J, vbytes), "autotune scratch") && D->cuda_ok(cudaMalloc(&d, D->nNodes * b * 8), "autotune scratch") &&
              D->cuda_ok(cudaEventCreate(&e0), "autotune") && D->cuda_ok(cudaEventCreate(&e1), "autotune");
    const int keep = D->asmThreads;
    std::vector<double> t(n_candidates, 0.0);
    for (int pass = 0; ok && pass < 2; ++pass)
        for (int c = 0; ok && c < n_candidates; ++c) {
            D->asmThreads = candidates[c];
            cudaEventRecord(e0, s);
            ok = D->assemble_defect_jacobian(u, nullptr, 0.0, d, J, prec, s);
            cudaEventRecord(e1, s);
            float msec = 0.f;
            if (ok) ok = D->cuda_ok(cudaEventSynchronize(e1), "autotune") && D->cuda_ok(cudaEventElapsedTime(&msec, e0, e1), "autotune");
            t[c] = msec;
        }
    if (J) cudaFree(J);
    if (d) cudaFree(d);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    D->asmThreads = keep;
    if (!ok) return D->status;
    int best = 0;
    for (int c = 1; c < n_candidates; ++c) if (t[c] < t[best]) best = c;
    D->asmThreads = candidates[best];
    if (ms) for (int c = 0; c < n_candidates; ++c) ms[c] = t[c];
    return NSFV1_OK;
}

int nsfv1_ref_tables(int elem_type, int* nco, int* nedge, int* edges, int* nside, int* side_nco, int* sides, int* edge_face) {
    auto fill = [&](auto r) {
        using R = Ref<decltype(r)::value>;
        *nco = R::nsh; *nedge = R::nip; *nside = R::nside;
        for (int e = 0; e < R::nip; ++e) {
            edges[2 * e] = R::edge(e, 0); edges[2 * e + 1] = R::edge(e, 1);
            edge_face[2 * e] = R::dim == 3 ? R::edge_face(e, 0) : -1;
            edge_face[2 * e + 1] = R::dim == 3 ? R::edge_face(e, 1) : -1;
        }
        for (int s = 0; s < R::nside; ++s) {
            side_nco[s] = R::side_nco(s);
            for (int j = 0; j < 4; ++j) sides[4 * s + j] = j < R::side_nco(s) ? R::side(s, j) : -1;
        }
    };
    switch (elem_type) {
        case ROID_TRIANGLE: fill(std::integral_constant<int, ROID_TRIANGLE>{}); return NSFV1_OK;
        case ROID_QUADRILATERAL: fill(std::integral_constant<int, ROID_QUADRILATERAL>{}); return NSFV1_OK;
        case ROID_TETRAHEDRON: fill(std::integral_constant<int, ROID_TETRAHEDRON>{}); return NSFV1_OK;
        case ROID_PRISM: fill(std::integral_constant<int, ROID_PRISM>{}); return NSFV1_OK;
        case ROID_HEXAHEDRON: fill(std::integral_constant<int, ROID_HEXAHEDRON>{}); return NSFV1_OK;
    }
    return NSFV1_ERR_ARGUMENT;
}

}  // extern "C"

// ============================================================================
// assembly drivers
// ============================================================================
namespace nsfv1 {

bool Disc::assemble_defect(const double* u, const double* u_old, double dt, double* d, cudaStream_t s) {
    if (!hasMesh) return fail(NSFV1_ERR_STATE, "assemble_defect: no mesh set");
    if (!u || !d) return fail(NSFV1_ERR_ARGUMENT, "assemble_defect: null vector");
    DiscParams P;
    if (!params(P, u_old != nullptr, dt) || !bind_ipws(P)) return false;
    const int b = dim + 1;
    if (!cuda_ok(cudaMemsetAsync(d, 0, sizeof(double) * nNodes * b, s), "memset defect")) return false;
    for (int c = 0; c < nColors; ++c) {
        AsmArgs a{d_coords, d_conn, d_elemBlk, d_colorElems + colorPtr[c], colorPtr[c + 1] - colorPtr[c], d_err, u, u_old, d, nullptr,
                  d_nuElem, instSkip ? d_elemInst : nullptr, d_instActive, nNodes, (int64_t)colIdx.size()};
        if (!cuda_ok(launch_defect(roid, P, a, s, asmThreads), "defect kernel")) return false;
    }
    if (!outflow_terms(P, u, d, nullptr, 0, s)) return false;
    if (!cuda_ok(launch_bnd_flux(b, nNodes, u_old ? dt : 1.0, d_bndFlux, d, s), "inflow flux")) return false;
    if (!cuda_ok(launch_dirichlet(b, nDir, d_dirRow, d_dirVal, d_rowPtr, d_colIdx, u, d, nullptr, 0, s), "dirichlet")) return false;
    return check_err_word(s);
}

bool Disc::assemble_defect_jacobian(const double* u, const double* u_old, double dt, double* d, void* vals, int prec, cudaStream_t s) {
    if (!hasMesh) return fail(NSFV1_ERR_STATE, "assemble_defect_jacobian: no mesh set");
    if (!u || !d || !vals) return fail(NSFV1_ERR_ARGUMENT, "assemble_defect_jacobian: null pointer");
    if (prec != NSFV1_F64 && prec != NSFV1_F32) return fail(NSFV1_ERR_ARGUMENT, "assemble_defect_jacobian: precision must be NSFV1_F64 or NSFV1_F32");
    if (prec == NSFV1_F32 && dim == 3 && (reinterpret_cast<uintptr_t>(vals) & 15))
        return fail(NSFV1_ERR_ARGUMENT, "assemble_defect_jacobian: FP32 values of a 3D mesh must be 16-byte aligned");
    DiscParams P;
    if (!params(P, u_old != nullptr, dt) || !bind_ipws(P)) return false;
    const int b = dim + 1;
    if (!cuda_ok(cudaMemsetAsync(d, 0, sizeof(double) * nNodes * b, s), "memset defect")) return false;
    const size_t vsize = prec == NSFV1_F64 ? sizeof(double) : sizeof(float);
    if (!cuda_ok(cudaMemsetAsync(vals, 0, colIdx.size() * b * b * vsize, s), "memset jacobian")) return false;
    for (int c = 0; c < nColors; ++c) {
        AsmArgs a{d_coords, d_conn, d_elemBlk, d_colorElems + colorPtr[c], colorPtr[c + 1] - colorPtr[c], d_err, u, u_old, d, vals,
                  d_nuElem, instSkip ? d_elemInst : nullptr, d_instActive, nNodes, (int64_t)colIdx.size()};
        if (!cuda_ok(launch_defect_jacobian(roid, P, a, prec, s, asmThreads), "defect+jacobian kernel")) return false;
    }
    if (!outflow_terms(P, u, d, vals, prec, s)) return false;
    if (!cuda_ok(launch_bnd_flux(b, nNodes, u_old ? dt : 1.0, d_bndFlux, d, s), "inflow flux")) return false;
    if (!cuda_ok(launch_dirichlet(b, nDir, d_dirRow, d_dirVal, d_rowPtr, d_colIdx, u, d, vals, prec, s), "dirichlet")) return false;
    return check_err_word(s);
}

bool Disc::assemble_jacobian(const double* u, const double* u_old, double dt, void* vals, int prec, cudaStream_t s, bool sync) {
    if (!hasMesh) return fail(NSFV1_ERR_STATE, "assemble_jacobian: no mesh set");
    if (!u || !vals) return fail(NSFV1_ERR_ARGUMENT, "assemble_jacobian: null pointer");
    if (prec != NSFV1_F64 && prec != NSFV1_F32) return fail(NSFV1_ERR_ARGUMENT, "assemble_jacobian: precision must be NSFV1_F64 or NSFV1_F32");
    if (prec == NSFV1_F32 && dim == 3 && (reinterpret_cast<uintptr_t>(vals) & 15))
        return fail(NSFV1_ERR_ARGUMENT, "assemble_jacobian: FP32 values of a 3D mesh must be 16-byte aligned");
    DiscParams P;
    if (!params(P, u_old != nullptr, dt) || !bind_ipws(P)) return false;
    const int b = dim + 1;
    const size_t bytes = colIdx.size() * b * b * (prec == NSFV1_F64 ? sizeof(double) : sizeof(float));
    if (!cuda_ok(cudaMemsetAsync(vals, 0, bytes, s), "memset jacobian")) return false;
    for (int c = 0; c < nColors; ++c) {
        AsmArgs a{d_coords, d_conn, d_elemBlk, d_colorElems + colorPtr[c], colorPtr[c + 1] - colorPtr[c], d_err, u, u_old, nullptr, vals,
                  d_nuElem, instSkip ? d_elemInst : nullptr, d_instActive, nNodes, (int64_t)colIdx.size()};
        if (!cuda_ok(launch_jacobian(roid, P, a, prec, s, asmThreads), "jacobian kernel")) return false;
    }
    if (!outflow_terms(P, u, nullptr, vals, prec, s)) return false;
    if (!cuda_ok(launch_dirichlet(b, nDir, d_dirRow, d_dirVal, d_rowPtr, d_colIdx, u, nullptr, vals, prec, s), "dirichlet")) return false;
    return sync ? check_err_word(s) : true;
}

}  // namespace nsfv1
