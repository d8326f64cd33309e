/*
 * ref_driver.cpp -- runs the REFERENCE's own FV1 element callbacks on the host.
 *
 * TEST INFRASTRUCTURE (builds oracle/_ref/libnsfv1_ref.so; see oracle/Makefile,
 * target "ref"). The unmodified reference sources are compiled where they lie
 * (include path NSREF_ROOT = the reference checkout) against the ugcore stand-in
 * in oracle/ugshim/. Nothing is copied from the reference into this repository,
 * and nothing of the product links this library: tests use it to pin the
 * oracle (oracle/nsfv1_oracle.cpp) to the reference's own arithmetic.
 *
 * Entry points (C ABI, loaded with ctypes by oracle/__init__.py):
 *   ref_elem_batch  -- the reference's NavierStokesFV1<Domain{2,3}d>::prep_elem +
 *                      add_def_A_elem / add_jac_A_elem / add_def_M_elem /
 *                      add_jac_M_elem / add_rhs_elem (navier_stokes_fv1.cpp:
 *                      208-248, 250-869) on n independent elements, in the
 *                      element-local layouts u[fct * nsh + sh] and
 *                      J[((f1 * nsh + s1) * b + f2) * nsh + s2];
 *   ref_geometry    -- the shim's FV1 geometry of one element (SCVF from/to,
 *                      ip, normal, shapes, global gradients; SCV volumes), to
 *                      compare the shim's and the oracle's restatements of it.
 */
#include "ug_shim.h"

// the reference sources (include order as their own headers require)
#include "navier_stokes_base.cpp"
#include "incompressible/incompressible_navier_stokes_base.cpp"
#include "upwind_interface.cpp"
#include "upwind.cpp"
#include "incompressible/fv1/stabilization.cpp"
#include "incompressible/fv1/navier_stokes_fv1.cpp"
#include "incompressible/bnd/no_normal_stress_outflow_base.cpp"
#include "incompressible/fv1/bnd/no_normal_stress_outflow_fv1.cpp"

#include <cstdint>
#include <cstdio>

namespace ug {
namespace NavierStokes {
// The reference registers its element callbacks with the core assembler in
// register_all_funcs (navier_stokes_fv1.cpp:1497-1551, compiled only with
// UG_DIM_x); this driver calls the callbacks directly, so nothing is registered.
template <> void NavierStokesFV1<Domain2d>::register_all_funcs(bool) {}
template <> void NavierStokesFV1<Domain3d>::register_all_funcs(bool) {}
template <> void NavierStokesNoNormalStressOutflowFV1<Domain2d>::register_all_funcs(bool) {}
template <> void NavierStokesNoNormalStressOutflowFV1<Domain3d>::register_all_funcs(bool) {}
}  // namespace NavierStokes
}  // namespace ug

extern "C" {
typedef struct {
    double nu, rho, full_newton;
    double src[3];
    int has_source, stokes, laplace, peclet, pac;
    const char* upwind;        /* convection upwind id ("no", "full", "skewed", "lps", "pos", "reg") */
    const char* stab;          /* "fields", "flow" or "without" */
    const char* diff_length;   /* "raw", "fivepoint", "cor" (NULL = the default) */
    const char* stab_upwind;   /* NULL: the stabilisation shares the convection upwind */
} ref_config;
}

namespace {

using namespace ug;
using namespace ug::NavierStokes;

template <int dim> struct DomainOf;
template <> struct DomainOf<2> { typedef Domain2d type; };
template <> struct DomainOf<3> { typedef Domain3d type; };

template <int dim>
void configure(NavierStokesFV1<typename DomainOf<dim>::type>& disc, const ref_config& c) {
    typedef typename DomainOf<dim>::type TDomain;
    // the number / vector overloads live in the base classes (hidden by the
    // SmartPtr overloads of NavierStokesFV1), as in the reference's registry
    static_cast<NavierStokesBase<TDomain>&>(disc).set_kinematic_viscosity(c.nu);
    static_cast<IncompressibleNavierStokesBase<TDomain>&>(disc).set_density(c.rho);
    if (c.has_source) static_cast<NavierStokesBase<TDomain>&>(disc).set_source(std::vector<number>(c.src, c.src + dim));
    disc.set_exact_jacobian(c.full_newton);
    disc.set_stokes(c.stokes != 0);
    disc.set_laplace(c.laplace != 0);
    disc.set_peclet_blend(c.peclet != 0);
    const std::string stab = TrimString(c.stab ? c.stab : "");
    if (stab == "without") {
        // NavierStokesFV1WithoutStabilization with the convection upwind object, the way a
        // Lua setup builds it (register_fv1.cpp:285-293)
        SmartPtr<INavierStokesUpwind<dim> > up = CreateNavierStokesUpwind<dim>(c.upwind ? c.upwind : "");
        SmartPtr<INavierStokesFV1Stabilization<dim> > s(new NavierStokesFV1WithoutStabilization<dim>());
        s->set_upwind(up);
        disc.set_stabilization(s);
        disc.set_upwind(up);
    } else {
        disc.set_upwind(std::string(c.upwind ? c.upwind : ""));
        if (c.diff_length) disc.set_stabilization(stab, std::string(c.diff_length));
        else disc.set_stabilization(stab);
    }
    if (c.stab_upwind) disc.stabilization()->set_upwind(CreateNavierStokesUpwind<dim>(c.stab_upwind));
    if (c.pac) disc.set_pac_upwind(true);
}

template <int dim, class TElem>
void run_batch(const ref_config& c, int64_t n, const double* corners, const double* u, const double* uold, double dt, double* defA,
               double* jacA, double* defM, double* jacM, double* rhs) {
    typedef typename DomainOf<dim>::type TDomain;
    typedef FV1Geometry<TElem, dim> TGeom;
    static const int nsh = (int)TGeom::nsh, b = dim + 1, nloc = b * nsh;
    const ReferenceObjectID roid = TGeom::ROID;
    NavierStokesFV1<TDomain> disc(dim == 2 ? "u,v,p" : "u,v,w,p", "Inner");
    configure<dim>(disc, c);
    LocalVectorTimeSeries ts;
    LocalVector U(b, nsh), Uo(b, nsh), d(b, nsh);
    LocalMatrix J(b, nsh);
    if (uold) {
        ts.set(&U, dt, &Uo, 0.0);
        disc.set_time_series(&ts);
    }
    disc.template prep_elem_loop<TElem, TGeom>(roid, 0);
    MathVector<dim> co[nsh];
    for (int64_t e = 0; e < n; ++e) {
        for (int k = 0; k < nsh; ++k)
            for (int x = 0; x < dim; ++x) co[k][x] = corners[(e * nsh + k) * dim + x];
        for (int q = 0; q < nloc; ++q) {
            U.data()[q] = u[e * nloc + q];
            Uo.data()[q] = uold ? uold[e * nloc + q] : 0.0;
        }
        disc.template prep_elem<TElem, TGeom>(U, nullptr, roid, co);
        if (defA) {
            d.zero();
            disc.template add_def_A_elem<TElem, TGeom>(d, U, nullptr, co);
            std::copy(d.data(), d.data() + nloc, defA + e * nloc);
        }
        if (jacA) {
            J.zero();
            disc.template add_jac_A_elem<TElem, TGeom>(J, U, nullptr, co);
            std::copy(J.data(), J.data() + nloc * nloc, jacA + e * nloc * nloc);
        }
        if (defM) {
            d.zero();
            disc.template add_def_M_elem<TElem, TGeom>(d, U, nullptr, co);
            std::copy(d.data(), d.data() + nloc, defM + e * nloc);
        }
        if (jacM) {
            J.zero();
            disc.template add_jac_M_elem<TElem, TGeom>(J, U, nullptr, co);
            std::copy(J.data(), J.data() + nloc * nloc, jacM + e * nloc * nloc);
        }
        if (rhs) {
            d.zero();
            disc.template add_rhs_elem<TElem, TGeom>(d, nullptr, co);
            std::copy(d.data(), d.data() + nloc, rhs + e * nloc);
        }
    }
    disc.template fsh_elem_loop<TElem, TGeom>();
}

template <int dim, class TElem>
void geometry(const double* corners, double* out) {
    typedef FV1Geometry<TElem, dim> TGeom;
    TGeom geo;
    MathVector<dim> co[TGeom::nsh];
    for (size_t k = 0; k < TGeom::nsh; ++k)
        for (int x = 0; x < dim; ++x) co[k][x] = corners[k * dim + x];
    geo.update(nullptr, co);
    // per SCVF 40 numbers: from, to, ip[3], normal[3], shape[8], grad[8][3]
    for (size_t i = 0; i < geo.num_scvf(); ++i) {
        double* o = out + i * 40;
        std::fill(o, o + 40, 0.0);
        const typename TGeom::SCVF& f = geo.scvf(i);
        o[0] = (double)f.from();
        o[1] = (double)f.to();
        for (int x = 0; x < dim; ++x) { o[2 + x] = f.global_ip()[x]; o[5 + x] = f.normal()[x]; }
        for (size_t k = 0; k < TGeom::nsh; ++k) {
            o[8 + k] = f.shape(k);
            for (int x = 0; x < dim; ++x) o[16 + 3 * k + x] = f.global_grad(k)[x];
        }
    }
    for (size_t a = 0; a < geo.num_scv(); ++a) out[geo.num_scvf() * 40 + a] = geo.scv(a).volume();
}

// The reference's data exports (navier_stokes_fv1.cpp:894-1491) of n elements at the
// SCVF ips (ipKind 0), the SCV ips (1) or nip given local points (2); layouts as
// ora_export: values[e][ip][vs], derivs[e][ip][fct][sh][vs], zeroed before each call.
template <int dim> void put(double* o, const MathVector<dim>& v) { for (int d = 0; d < dim; ++d) o[d] = v[d]; }
template <int dim> void put(double* o, const MathMatrix<dim, dim>& m) {
    for (int r = 0; r < dim; ++r) for (int c = 0; c < dim; ++c) o[r * dim + c] = m(r, c);
}
template <int dim> void put(double* o, const number& v) { o[0] = v; }
template <class T> void zero(T& v) { v = 0.0; }

template <int dim, class TElem>
void run_export(const ref_config& c, int which, int64_t n, const double* corners, const double* u, const double* uold, double dt, int ipKind,
                int nipGiven, const double* lips, double* values, double* derivs) {
    typedef typename DomainOf<dim>::type TDomain;
    typedef FV1Geometry<TElem, dim> TGeom;
    typedef NavierStokesFV1<TDomain> TDisc;
    static const int nsh = (int)TGeom::nsh, b = dim + 1, nloc = b * nsh;
    const ReferenceObjectID roid = TGeom::ROID;
    TDisc disc(dim == 2 ? "u,v,p" : "u,v,w,p", "Inner");
    configure<dim>(disc, c);
    LocalVectorTimeSeries ts;
    LocalVector U(b, nsh), Uo(b, nsh);
    if (uold) {
        ts.set(&U, dt, &Uo, 0.0);
        disc.set_time_series(&ts);
    }
    disc.template prep_elem_loop<TElem, TGeom>(roid, 0);
    const TGeom& geo = GeomProvider<TGeom>::get();
    MathVector<dim> co[nsh];
    std::vector<MathVector<dim> > given(nipGiven > 0 ? nipGiven : 1);
    for (int i = 0; i < nipGiven; ++i) for (int d = 0; d < dim; ++d) given[i][d] = lips[i * dim + d];
    const int vs = (which == 1) ? dim * dim : (which == 3) ? 1 : dim;
    for (int64_t e = 0; e < n; ++e) {
        for (int k = 0; k < nsh; ++k)
            for (int x = 0; x < dim; ++x) co[k][x] = corners[(e * nsh + k) * dim + x];
        for (int q = 0; q < nloc; ++q) {
            U.data()[q] = u[e * nloc + q];
            Uo.data()[q] = uold ? uold[e * nloc + q] : 0.0;
        }
        disc.template prep_elem<TElem, TGeom>(U, nullptr, roid, co);
        const MathVector<dim>* lip = ipKind == 0 ? geo.scvf_local_ips() : ipKind == 1 ? geo.scv_local_ips() : &given[0];
        const size_t nip = ipKind == 0 ? geo.num_scvf() : ipKind == 1 ? geo.num_scv() : (size_t)nipGiven;
        std::vector<MathVector<dim> > gip(nip);
        double* val = values + e * (int64_t)nip * vs;
        double* der = derivs ? derivs + e * (int64_t)nip * b * nsh * vs : nullptr;
        auto run = [&](auto* proto, auto fn) {
            typedef typename std::remove_pointer<decltype(proto)>::type T;
            std::vector<T> v(nip);
            for (auto& x : v) zero(x);
            std::vector<std::vector<std::vector<T> > > dv(nip, std::vector<std::vector<T> >(b, std::vector<T>(nsh)));
            for (auto& a : dv) for (auto& bb : a) for (auto& x : bb) zero(x);
            fn(v.data(), gip.data(), lip, nip, der != nullptr, dv.data());
            for (size_t ip = 0; ip < nip; ++ip) {
                put<dim>(val + ip * vs, v[ip]);
                if (der)
                    for (int f = 0; f < b; ++f)
                        for (int sh = 0; sh < nsh; ++sh) put<dim>(der + ((ip * b + f) * nsh + sh) * vs, dv[ip][f][sh]);
            }
        };
        switch (which) {
            case 0:
                run((MathVector<dim>*)nullptr, [&](auto* v, auto* g, auto* l, size_t ni, bool bd, auto* dv) {
                    disc.template ex_nodal_velocity<TElem, TGeom>(v, g, 0.0, 0, U, nullptr, co, l, ni, bd, dv);
                });
                break;
            case 1:
                run((MathMatrix<dim, dim>*)nullptr, [&](auto* v, auto* g, auto* l, size_t ni, bool bd, auto* dv) {
                    disc.template ex_velocity_grad<TElem, TGeom>(v, g, 0.0, 0, U, nullptr, co, l, ni, bd, dv);
                });
                break;
            case 2:
                run((MathVector<dim>*)nullptr, [&](auto* v, auto* g, auto* l, size_t ni, bool bd, auto* dv) {
                    disc.template ex_velocity_ip<TElem, TGeom>(v, g, 0.0, 0, U, nullptr, co, l, ni, bd, dv);
                });
                break;
            case 3:
                run((number*)nullptr, [&](auto* v, auto* g, auto* l, size_t ni, bool bd, auto* dv) {
                    disc.template ex_nodal_pressure<TElem, TGeom>(v, g, 0.0, 0, U, nullptr, co, l, ni, bd, dv);
                });
                break;
            default:
                run((MathVector<dim>*)nullptr, [&](auto* v, auto* g, auto* l, size_t ni, bool bd, auto* dv) {
                    disc.template ex_pressure_grad<TElem, TGeom>(v, g, 0.0, 0, U, nullptr, co, l, ni, bd, dv);
                });
        }
    }
    disc.template fsh_elem_loop<TElem, TGeom>();
}

// The reference's NavierStokesNoNormalStressOutflowFV1 (no_normal_stress_outflow_fv1.cpp:
// 343-504) on n elements: sideMask[e] marks the element's sides on the outflow boundary
// (bit s = side s; the stand-in's boundary faces); the disc's add_def_A_elem /
// add_jac_A_elem in the element-local layouts.
template <int dim, class TElem>
void run_outflow(const ref_config& c, int64_t n, const double* corners, const double* u, const unsigned* sideMask, double* defA,
                 double* jacA) {
    typedef typename DomainOf<dim>::type TDomain;
    typedef FV1Geometry<TElem, dim> TGeom;
    static const int nsh = (int)TGeom::nsh, b = dim + 1, nloc = b * nsh;
    const ReferenceObjectID roid = TGeom::ROID;
    SmartPtr<NavierStokesFV1<TDomain> > master(new NavierStokesFV1<TDomain>(dim == 2 ? "u,v,p" : "u,v,w,p", "Inner"));
    configure<dim>(*master, c);
    NavierStokesNoNormalStressOutflowFV1<TDomain> outflow(master);
    outflow.add("Outflow");
    outflow.template prep_elem_loop<TElem, TGeom>(roid, 0);
    LocalVector U(b, nsh), d(b, nsh);
    LocalMatrix J(b, nsh);
    MathVector<dim> co[nsh];
    for (int64_t e = 0; e < n; ++e) {
        for (int k = 0; k < nsh; ++k)
            for (int x = 0; x < dim; ++x) co[k][x] = corners[(e * nsh + k) * dim + x];
        for (int q = 0; q < nloc; ++q) U.data()[q] = u[e * nloc + q];
        shim_boundary_sides() = sideMask[e];
        outflow.template prep_elem<TElem, TGeom>(U, nullptr, roid, co);
        if (defA) {
            d.zero();
            outflow.template add_def_A_elem<TElem, TGeom>(d, U, nullptr, co);
            std::copy(d.data(), d.data() + nloc, defA + e * nloc);
        }
        if (jacA) {
            J.zero();
            outflow.template add_jac_A_elem<TElem, TGeom>(J, U, nullptr, co);
            std::copy(J.data(), J.data() + nloc * nloc, jacA + e * nloc * nloc);
        }
    }
    shim_boundary_sides() = 0;
    outflow.template fsh_elem_loop<TElem, TGeom>();
}

thread_local std::string g_err;

}  // namespace

extern "C" {

const char* ref_last_error(void) { return g_err.c_str(); }

/* 0 on success, 1 on a reference exception (text in ref_last_error), 2 on a bad element type */
int ref_elem_batch(int roid, int64_t n, const ref_config* c, const double* corners, const double* u, const double* u_old, double dt,
                   double* defA, double* jacA, double* defM, double* jacM, double* rhs) {
    try {
        switch (roid) {
            case ROID_TRIANGLE: run_batch<2, Triangle>(*c, n, corners, u, u_old, dt, defA, jacA, defM, jacM, rhs); return 0;
            case ROID_QUADRILATERAL: run_batch<2, Quadrilateral>(*c, n, corners, u, u_old, dt, defA, jacA, defM, jacM, rhs); return 0;
            case ROID_TETRAHEDRON: run_batch<3, Tetrahedron>(*c, n, corners, u, u_old, dt, defA, jacA, defM, jacM, rhs); return 0;
            case ROID_PRISM: run_batch<3, Prism>(*c, n, corners, u, u_old, dt, defA, jacA, defM, jacM, rhs); return 0;
            case ROID_HEXAHEDRON: run_batch<3, Hexahedron>(*c, n, corners, u, u_old, dt, defA, jacA, defM, jacM, rhs); return 0;
        }
        return 2;
    } catch (std::exception& e) {
        g_err = e.what();
        return 1;
    }
}

int ref_export(int which, int roid, int64_t n, const ref_config* c, const double* corners, const double* u, const double* u_old, double dt,
               int ipKind, int nip, const double* lips, double* values, double* derivs) {
    try {
        switch (roid) {
            case ROID_TRIANGLE: run_export<2, Triangle>(*c, which, n, corners, u, u_old, dt, ipKind, nip, lips, values, derivs); return 0;
            case ROID_QUADRILATERAL: run_export<2, Quadrilateral>(*c, which, n, corners, u, u_old, dt, ipKind, nip, lips, values, derivs); return 0;
            case ROID_TETRAHEDRON: run_export<3, Tetrahedron>(*c, which, n, corners, u, u_old, dt, ipKind, nip, lips, values, derivs); return 0;
            case ROID_PRISM: run_export<3, Prism>(*c, which, n, corners, u, u_old, dt, ipKind, nip, lips, values, derivs); return 0;
            case ROID_HEXAHEDRON: run_export<3, Hexahedron>(*c, which, n, corners, u, u_old, dt, ipKind, nip, lips, values, derivs); return 0;
        }
        return 2;
    } catch (std::exception& e) {
        g_err = e.what();
        return 1;
    }
}

int ref_outflow_batch(int roid, int64_t n, const ref_config* c, const double* corners, const double* u, const unsigned* sideMask, double* defA,
                      double* jacA) {
    try {
        switch (roid) {
            case ROID_TRIANGLE: run_outflow<2, Triangle>(*c, n, corners, u, sideMask, defA, jacA); return 0;
            case ROID_QUADRILATERAL: run_outflow<2, Quadrilateral>(*c, n, corners, u, sideMask, defA, jacA); return 0;
            case ROID_TETRAHEDRON: run_outflow<3, Tetrahedron>(*c, n, corners, u, sideMask, defA, jacA); return 0;
            case ROID_PRISM: run_outflow<3, Prism>(*c, n, corners, u, sideMask, defA, jacA); return 0;
            case ROID_HEXAHEDRON: run_outflow<3, Hexahedron>(*c, n, corners, u, sideMask, defA, jacA); return 0;
        }
        return 2;
    } catch (std::exception& e) {
        g_err = e.what();
        return 1;
    }
}

int ref_geometry(int roid, const double* corners, double* out) {
    try {
        switch (roid) {
            case ROID_TRIANGLE: geometry<2, Triangle>(corners, out); return 0;
            case ROID_QUADRILATERAL: geometry<2, Quadrilateral>(corners, out); return 0;
            case ROID_TETRAHEDRON: geometry<3, Tetrahedron>(corners, out); return 0;
            case ROID_PRISM: geometry<3, Prism>(corners, out); return 0;
            case ROID_HEXAHEDRON: geometry<3, Hexahedron>(corners, out); return 0;
        }
        return 2;
    } catch (std::exception& e) {
        g_err = e.what();
        return 1;
    }
}

}  // extern "C"
