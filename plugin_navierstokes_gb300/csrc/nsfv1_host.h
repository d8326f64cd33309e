// The element-disc handle behind the opaque nsfv1_disc* of the C ABI.
#pragma once
#include <cstdint>
#include <string>
#include <vector>
#include <cuda_runtime.h>
#include "nsfv1_params.h"

namespace nsfv1 {

std::string lower_trim(const char* s);
int ref_dim(int roid);
int ref_nsh(int roid);

// Newton / Krylov device workspace (allocated on first solve, per precision)
struct Workspace {
    int prec = -1, gmresM = 0;
    int64_t n = 0;
    double *D = nullptr, *Dt = nullptr, *Ut = nullptr, *du = nullptr;   // FP64 Newton vectors
    void* J = nullptr;        // Jacobian values (VT)
    void* Dinv = nullptr;     // inverted diagonal blocks (VT)
    void* vec = nullptr;      // Krylov vectors (VT), nvec * n
    int nvec = 0;
    double* red = nullptr;    // reduction partials
    double* scal = nullptr;   // device scalars
    double* hscal = nullptr;  // pinned host mirror of the scalars
};

struct Disc {
    int dim = 2;
    // parameters (defaults of the reference constructors)
    double nu = 0.0, rho = 1.0, fullNewton = 0.0;
    double src[3] = {0, 0, 0};
    int hasSource = 0, stokes = 0, laplace = 0, peclet = 0;
    bool viscoSet = false, stabSet = false, convUpwindSet = false, stabSharesConv = false;
    bool pac = false;   // set_pac_upwind(true): the stabilisation is the convective upwind
    int convUpwindType = -1, stabUpwindType = -1, stabType = -1, diffLen = DL_RAW;

    // mesh
    bool hasMesh = false;
    int roid = 0, nsh = 0, nColors = 0;
    int64_t nNodes = 0, nElems = 0;
    std::vector<int32_t> rowPtr, colIdx, elemBlk, color, colorPtr, colorElems;
    double* d_coords = nullptr;
    int32_t *d_conn = nullptr, *d_elemBlk = nullptr, *d_colorElems = nullptr, *d_rowPtr = nullptr, *d_colIdx = nullptr;
    int32_t* d_diagPos = nullptr;   // block index of each row's diagonal block
    double* d_nuElem = nullptr;     // per-element viscosity (nsfv1_set_elem_viscosity), or null
    // independent instances (nsfv1_set_instances): node ranges, element -> instance
    int nInst = 0;
    std::vector<int32_t> instNode0;          // [nInst + 1] first node of each instance
    int32_t* d_instNode0 = nullptr;
    int32_t* d_elemInst = nullptr;
    int32_t* d_nodeInst = nullptr;
    int32_t* d_instActive = nullptr;         // per-instance active flag (assembly skips inactive ones)
    bool instSkip = false;                   // assembly honours d_instActive
    // host copies used to build coarse multigrid levels of structured instances
    std::vector<double> coordsHost, nuElemHost, dirValHost;
    std::vector<int32_t> connHost, dirRowHost;
    std::vector<int32_t> instCells;          // cells per side of each structured instance (nsfv1_set_instance_grids)
    // continuity-row flux of inflow boundaries (nsfv1_add_inflow), per node; added to the defect
    std::vector<double> bndFluxHost;
    double* d_bndFlux = nullptr;
    double* d_nodeVol = nullptr;    // nsfv1_vorticity scratch: SCV volume per node
    // outflow boundary faces without normal stress (nsfv1_add_outflow), grouped by node
    struct OutflowFace {
        int32_t node, elem, local;
        double xi[3], n[3];
    };
    std::vector<OutflowFace> outflowHost;
    int32_t *d_ofSeg = nullptr, *d_ofElem = nullptr, *d_ofLocal = nullptr;
    double *d_ofXi = nullptr, *d_ofN = nullptr;
    int32_t nOfSeg = 0;
    double* d_bjDinv = nullptr;     // nsfv1_block_jacobi scratch: inverted diagonal blocks
    int32_t* d_dirRow = nullptr;
    double* d_dirVal = nullptr;
    int64_t nDir = 0;
    int* d_err = nullptr;
    // workspace of the positive-upwind element path (allocated when such an upwind is set)
    double* d_ipws = nullptr;
    int64_t ipwsThreads = 0;
    int asmThreads = 32;            // CTA size of the assembly colour launches

    Workspace ws;
    void* batch = nullptr;   // workspace of the batched solver

    int status = 0;
    std::string lastError;

    ~Disc();
    void free_mesh();
    void free_outflow();
    bool outflow_terms(const DiscParams& P, const double* u, double* d, void* vals, int prec, cudaStream_t s);
    void free_workspace();
    bool fail(int code, const std::string& msg);
    bool cuda_ok(cudaError_t e, const char* where);
    bool check_err_word(cudaStream_t s);
    bool params(DiscParams& P, bool transient, double dt);
    bool ensure_ipws(bool force = false);   // allocates d_ipws if a positive upwind is configured (or force)
    bool bind_ipws(DiscParams& P);   // P.ipws for a launch that needs it
    bool assemble_defect(const double* u, const double* u_old, double dt, double* d, cudaStream_t s);
    bool assemble_jacobian(const double* u, const double* u_old, double dt, void* vals, int prec, cudaStream_t s, bool sync = true);
    bool assemble_defect_jacobian(const double* u, const double* u_old, double dt, double* d, void* vals, int prec, cudaStream_t s);
    bool ensure_workspace(int prec, int gmresM);
    bool set_dirichlet_values(double* u, cudaStream_t s);   // u[dof] = g for every Dirichlet row
};

void batch_free(void* p);

// point-block Jacobi on a caller's Jacobian with Dinv as scratch (nNodes*b*b
// doubles): shared by nsfv1_block_jacobi and its variant without allocation
bool block_jacobi_run(Disc& D, const void* vals, int prec, const double* r, double* z, double* Dinv, cudaStream_t s);

}  // namespace nsfv1
