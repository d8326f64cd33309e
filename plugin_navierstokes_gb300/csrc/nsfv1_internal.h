// Internal declarations shared by the host C-ABI layer and the CUDA sources.
#pragma once
#include <cstdint>
#include <string>
#include <vector>
#include <cuda_runtime.h>
#include "nsfv1_params.h"

namespace nsfv1 {

// Device view of a mesh for one assembly launch (the elements of one colour).
struct AsmArgs {
    const double* coords;     // [nNodes][dim]
    const int32_t* conn;      // [nElems][nsh]
    const int32_t* elemBlk;   // [nElems][nsh][nsh] block index into the BSR values
    const int32_t* elems;     // element ids of this launch
    int32_t count;
    int* err;                 // error word (bit 0: upwind side not found)
    const double* U;          // [nNodes][b]
    const double* Uold;       // [nNodes][b] or null
    double* D;                // defect [nNodes][b]
    void* vals;               // BSR values (double or float)
    const double* nuElem;     // per-element kinematic viscosity, or null (the disc's constant)
    const int32_t* elemInst;  // per-element instance id, or null (no instance skipping)
    const int32_t* instActive;// per-instance flag: elements of inactive instances are skipped
    int64_t nNodes = 0;       // index bounds checked by a build with NSFV1_BOUNDS_CHECK
    int64_t nnzb = 0;
};

// Batched element-local callbacks (no global scatter).
struct ElemBatchArgs {
    int64_t n;
    const double* corners;    // [n][nsh][dim]
    const double* u;          // [n][b][nsh]
    const double* uold;       // [n][b][nsh] or null
    double* defA; double* jacA; double* defM; double* jacM; double* rhs;
    int* err;
};

// threads: CTA size of the colour launches (32..128, a multiple of 32)
cudaError_t launch_defect(int roid, const DiscParams& P, const AsmArgs& a, cudaStream_t s, int threads = 128);
cudaError_t launch_jacobian(int roid, const DiscParams& P, const AsmArgs& a, int prec, cudaStream_t s, int threads = 128);
// FP64 defect (a.D) and the Jacobian (a.vals; prec 0: FP64, 1: FP32 blocks from the FP64
// state) at the same state, one launch per colour
cudaError_t launch_defect_jacobian(int roid, const DiscParams& P, const AsmArgs& a, int prec, cudaStream_t s, int threads = 128);
cudaError_t launch_elem_batch(int roid, const DiscParams& P, const ElemBatchArgs& a, cudaStream_t s);
// D[node * b + b - 1] += scale * flux[node] (the inflow boundaries' continuity flux)
cudaError_t launch_bnd_flux(int b, int64_t nNodes, double scale, const double* flux, double* D, cudaStream_t s);
cudaError_t launch_dirichlet(int b, int64_t n, const int32_t* rows, const double* vals, const int32_t* rowPtr,
                             const int32_t* colIdx, const double* U, double* D, void* J, int prec, cudaStream_t s);

}  // namespace nsfv1
