// Parameter block and option ids shared by the host layer and the kernels.
#pragma once

namespace nsfv1 {

enum { ROID_TRIANGLE = 2, ROID_QUADRILATERAL = 3, ROID_TETRAHEDRON = 4, ROID_PRISM = 6, ROID_HEXAHEDRON = 8 };
enum { UPW_NO = 0, UPW_FULL = 1, UPW_SKEWED = 2, UPW_LPS = 3, UPW_POS = 4 };
enum { STAB_FIELDS = 0, STAB_FLOW = 1, STAB_WITHOUT = 2 };
enum { DL_RAW = 0, DL_FIVEPOINT = 1, DL_COR = 2 };

// Uniform (per launch) discretisation parameters.
struct DiscParams {
    double nu, rho, fullNewton, dt;
    double src[3];
    int convUpwind;   // upwind of the convective term (ignored when stokes)
    int stabUpwind;   // upwind object of the stabilisation
    int sameUpwind;   // 1: the stabilisation shares the convection upwind object
    int stab, diffLen;
    int stokes, laplace, peclet, hasSource, transient;
    int pac;          // the stabilisation is the convective upwind (set_pac_upwind)
    double* ipws;     // per-thread workspace of the positive-upwind element path (device), or null
    long long ipwsStride;   // its thread count: entry i of thread t at ipws[i * ipwsStride + t]
};

// the element terms couple all SCVFs of an element (an upwind with ip shapes is in use)
inline bool uses_ipshape(const DiscParams& P) { return !P.stokes && (P.convUpwind == UPW_POS || P.stabUpwind == UPW_POS); }

}  // namespace nsfv1
