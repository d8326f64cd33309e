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
// FP64 defect (a.D) and the Jacobian (a.vals) at the same state: prec 0 one FP64 launch
// per colour, prec 1 the FP64 defect and the lane-per-corner FP32 Jacobian of the colour
cudaError_t launch_defect_jacobian(int roid, const DiscParams& P, const AsmArgs& a, int prec, cudaStream_t s, int threads = 128);
cudaError_t launch_elem_batch(int roid, const DiscParams& P, const ElemBatchArgs& a, cudaStream_t s);
// FP32 Jacobian (values only, no defect) with one lane per element corner
cudaError_t launch_jacobian_lanes(int roid, const DiscParams& P, const AsmArgs& a, cudaStream_t s);
// The positive-upwind element path (uses_ipshape(P)): defect, Jacobian (prec 0: FP64,
// 1: FP32 values of FP64 arithmetic) and the stiffness part of the element batch;
// P.ipws must hold ipws_doubles_host(dim) doubles for each of P.ipwsStride threads.
constexpr int kIpwsCtaThreads = 64;
// The data exports (navier_stokes_fv1.cpp:894-1491) of n elements: values[e][ip][vs],
// derivs[e][ip][fct][sh][vs] (or null); ipKind 0: SCVF ips, 1: SCV ips (the
// corners), 2: the nip local points lips (at most kMaxExportPoints).
constexpr int kMaxExportPoints = 64;
struct ExportArgs {
    int which, ipKind, nip;
    int64_t n;
    const double* corners;    // [n][nsh][dim]
    const double* u;          // [n][b][nsh]
    const double* uold;       // [n][b][nsh] or null
    double* values;
    double* derivs;
    int* err;
    double lips[kMaxExportPoints][3];
};
cudaError_t launch_export(int roid, const DiscParams& P, const ExportArgs& a, cudaStream_t s);
// post-processing (navier_stokes_tools.h): vorticityFV1 of one colour's elements
// (a.U the state; vort and vol accumulate per node), a[i] /= d[i], point evaluation
cudaError_t launch_vorticity(int roid, const AsmArgs& a, double* vort, double* vol, cudaStream_t s);
cudaError_t launch_divide(int64_t n, double* a, const double* d, cudaStream_t s);
// Outflow boundary faces without normal stress (NavierStokesNoNormalStressOutflowFV1),
// sorted by the node they belong to: segment s = faces [segPtr[s], segPtr[s + 1]) of
// one node, so one thread owns each node's row.
struct OutflowArgs {
    int32_t nSeg;
    const int32_t* segPtr;
    const int32_t* elem;      // the element the face's side belongs to
    const int32_t* local;     // the face corner's index in that element
    const double* xi;         // [nFaces][3] local coordinates of the face's integration point
    const double* nrm;        // [nFaces][3] outward area-weighted normal
};
// adds the faces' terms to a.D (if set) and the a.vals Jacobian (if set; prec 0 FP64, 1 FP32),
// scaled by P.dt when P.transient
cudaError_t launch_outflow(int roid, const DiscParams& P, const AsmArgs& a, const OutflowArgs& o, int prec, cudaStream_t s);
cudaError_t launch_eval_points(int roid, int64_t nElems, int64_t nNodes, const double* coords, const int32_t* conn, const double* U,
                               int64_t np, const double* pts, int fct, double* out, cudaStream_t s);
int ipws_doubles_host(int dim);
cudaError_t launch_defect_ipshape(int roid, const DiscParams& P, const AsmArgs& a, cudaStream_t s);
cudaError_t launch_jacobian_ipshape(int roid, const DiscParams& P, const AsmArgs& a, int prec, cudaStream_t s);
cudaError_t launch_elem_batch_ipshape(int roid, const DiscParams& P, const ElemBatchArgs& a, cudaStream_t s);
// D[node * b + b - 1] += scale * flux[node] (the inflow boundaries' continuity flux)
cudaError_t launch_bnd_flux(int b, int64_t nNodes, double scale, const double* flux, double* D, cudaStream_t s);
cudaError_t launch_dirichlet(int b, int64_t n, const int32_t* rows, const double* vals, const int32_t* rowPtr,
                             const int32_t* colIdx, const double* U, double* D, void* J, int prec, cudaStream_t s);

}  // namespace nsfv1
