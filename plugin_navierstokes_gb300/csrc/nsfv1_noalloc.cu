// nsfv1_block_jacobi_noalloc: the point-block Jacobi preconditioner of
// nsfv1_block_jacobi for callers that cannot allocate device memory.
//
// Who needs it: applications whose device memory is entirely handed out by
// their own pool allocator (a cudaMalloc from a library would fail or fragment
// that pool). nsfv1_block_jacobi allocates its scratch (the inverted diagonal
// blocks) on first use; this variant keeps that scratch in a fixed device
// array of this file instead and allocates nothing.
//
// Limits and behaviour:
//  - The scratch holds NSFV1_NOALLOC_MAX_NODES (32768) nodes of 4 x 4 FP64
//    blocks, 4 MiB; every GPU that loads the library keeps it until exit.
//    Meshes with more nodes are rejected with NSFV1_ERR_ARGUMENT.
//  - The first call on a device looks up the array's device address with
//    cudaGetSymbolAddress (with that device current) and caches it; make that
//    first call before any stream capture.
//  - Each call waits for its stream to finish, as nsfv1_block_jacobi does: the
//    singular-block flag is read back to the host (NSFV1_ERR_BREAKDOWN).
//  - All calls in the process share the one array and it keeps the contents
//    of the last call: calls that overlap on the GPU (two streams, two
//    threads, two handles) race and must be serialised by the caller. Every
//    call rewrites the blocks of all its nodes before reading them, so nothing
//    has to start at zero; the handle's error word is cleared by each call.
#include <cstring>
#include <mutex>
#include <string>
#include "nsfv1_internal.h"
#include "nsfv1_host.h"
#include "../../include/nsfv1_gb300.h"

using namespace nsfv1;

namespace {

static __device__ __align__(256) double g_noallocDinv[(size_t)NSFV1_NOALLOC_MAX_NODES * 16];

constexpr int kMaxDevices = 64;
static double* s_scratch[kMaxDevices] = {nullptr};
static std::mutex s_mutex;

// device address of g_noallocDinv on the current device (looked up once per device)
static cudaError_t scratch_address(double** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(s_mutex);
    if (!s_scratch[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noallocDinv);
        if (e != cudaSuccess) return e;
        s_scratch[dev] = static_cast<double*>(p);
    }
    *out = s_scratch[dev];
    return cudaSuccess;
}

}  // namespace

extern "C" int nsfv1_block_jacobi_noalloc(nsfv1_disc* h, const void* vals, int prec, const double* r, double* z, void* stream) {
    Disc* D = reinterpret_cast<Disc*>(h);
    if (!D) return NSFV1_ERR_ARGUMENT;
    D->status = NSFV1_OK;
    if (!D->hasMesh) { D->fail(NSFV1_ERR_STATE, "block_jacobi_noalloc: no mesh"); return D->status; }
    if (!vals || !r || !z || (prec != NSFV1_F64 && prec != NSFV1_F32)) {
        D->fail(NSFV1_ERR_ARGUMENT, "block_jacobi_noalloc: bad arguments");
        return D->status;
    }
    if (D->nNodes > NSFV1_NOALLOC_MAX_NODES) {
        D->fail(NSFV1_ERR_ARGUMENT, "block_jacobi_noalloc: the mesh has " + std::to_string(D->nNodes) +
                " nodes, the fixed scratch holds at most " + std::to_string(NSFV1_NOALLOC_MAX_NODES) +
                " (use nsfv1_block_jacobi)");
        return D->status;
    }
    double* scratch = nullptr;
    if (!D->cuda_ok(scratch_address(&scratch), "block_jacobi_noalloc: cudaGetSymbolAddress")) return D->status;
    return block_jacobi_run(*D, vals, prec, r, z, scratch, (cudaStream_t)stream) ? NSFV1_OK : D->status;
}
