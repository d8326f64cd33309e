/*
 * nsfv1_gb300.hpp -- header-only C++ host class over the C ABI (nsfv1_gb300.h),
 * with the method names, string ids, overloads and exceptions of the
 * reference's element disc NavierStokesFV1 (incompressible/fv1/
 * navier_stokes_fv1.h:160-488, navier_stokes_base.h:163-196,
 * incompressible_navier_stokes_base.h:183-225), so that host code written
 * against the reference's class reads the same.
 *
 *  - Setters: set_kinematic_viscosity, set_density, set_source, set_exact_jacobian,
 *    set_stokes, set_laplace, set_peclet_blend, set_upwind(name),
 *    set_stabilization(name[, diffLength]), set_stabilization_upwind(name);
 *    ids trimmed and case-insensitive as in CreateNavierStokesUpwind /
 *    CreateNavierStokesStabilization. Errors raise nsfv1::Error (the reference
 *    raises UG_THROW) with the library's status code and text.
 *  - The per-element callbacks of the reference (prep_elem_loop, prep_elem,
 *    add_jac_A_elem, add_def_A_elem, add_jac_M_elem, add_def_M_elem,
 *    add_rhs_elem, fsh_elem_loop; navier_stokes_fv1.h:254-281) take the
 *    element-local LocalVector / LocalMatrix as flat arrays in the reference's
 *    function-major layouts
 *        u[fct * nsh + sh],  J[((f1 * nsh + s1) * b + f2) * nsh + s2],
 *    and ADD into them (d += ..., J += ...) as the reference does. Each call
 *    evaluates one element on the GPU; elem_batch() evaluates many elements
 *    per call and is the throughput path for host-side element loops.
 *  - Global assembly and the Newton solver stay on the C ABI (device pointers;
 *    handle() returns the underlying nsfv1_disc*).
 */
#ifndef NSFV1_GB300_HPP
#define NSFV1_GB300_HPP

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "nsfv1_gb300.h"

namespace nsfv1 {

/* the library's status and text (the reference throws UG_THROW on the same conditions) */
class Error : public std::runtime_error {
  public:
    Error(int status, const std::string& what) : std::runtime_error(what), m_status(status) {}
    int status() const { return m_status; }

  private:
    int m_status;
};

inline int num_corners(int roid) {
    switch (roid) {
        case NSFV1_TRIANGLE: return 3;
        case NSFV1_QUADRILATERAL: return 4;
        case NSFV1_TETRAHEDRON: return 4;
        case NSFV1_PRISM: return 6;
        case NSFV1_HEXAHEDRON: return 8;
    }
    return 0;
}

class NavierStokesFV1 {
  public:
    /* NavierStokesFV1(functions, subsets) (navier_stokes_fv1.cpp:45-87): dim + 1
     * comma-separated P1 functions, e.g. "u,v,p" or "u,v,w,p" */
    NavierStokesFV1(const char* functions, const char* subsets) : m_subsets(subsets ? subsets : "") {
        const int nf = count_functions(functions);
        if (nf != 3 && nf != 4)
            throw Error(NSFV1_ERR_ARGUMENT, "Wrong number of functions: The ElemDisc 'NavierStokes' needs exactly dim+1 symbolic function.");
        create(nf - 1);
    }
    explicit NavierStokesFV1(int dim) { create(dim); }
    ~NavierStokesFV1() { if (m_h) nsfv1_destroy(m_h); }
    NavierStokesFV1(const NavierStokesFV1&) = delete;
    NavierStokesFV1& operator=(const NavierStokesFV1&) = delete;

    nsfv1_disc* handle() const { return m_h; }
    int dim() const { return m_dim; }
    std::string disc_type() const { return nsfv1_disc_type(m_h); }

    /* ---- setters (navier_stokes_base.h, incompressible_navier_stokes_base.h, navier_stokes_fv1.h) */
    void set_kinematic_viscosity(double nu) { check(nsfv1_set_kinematic_viscosity(m_h, nu)); }
    void set_density(double rho) { check(nsfv1_set_density(m_h, rho)); }
    void set_source(const std::vector<double>& f) { check(nsfv1_set_source(m_h, f.data(), (int)f.size())); }
    void set_exact_jacobian(bool on) { check(nsfv1_set_exact_jacobian(m_h, on ? 1.0 : 0.0)); }
    void set_exact_jacobian(double factor) { check(nsfv1_set_exact_jacobian(m_h, factor)); }
    void set_stokes(bool on) { check(nsfv1_set_stokes(m_h, on ? 1 : 0)); }
    void set_laplace(bool on) { check(nsfv1_set_laplace(m_h, on ? 1 : 0)); }
    void set_peclet_blend(bool on) { check(nsfv1_set_peclet_blend(m_h, on ? 1 : 0)); }
    void set_upwind(const std::string& name) { check(nsfv1_set_upwind(m_h, name.c_str())); }
    void set_stabilization(const std::string& name) { check(nsfv1_set_stabilization(m_h, name.c_str(), nullptr)); }
    void set_stabilization(const std::string& name, const std::string& diffLength) {
        check(nsfv1_set_stabilization(m_h, name.c_str(), diffLength.c_str()));
    }
    void set_stabilization_upwind(const std::string& name) { check(nsfv1_set_stabilization_upwind(m_h, name.c_str())); }
    void set_pac_upwind(bool on) { check(nsfv1_set_pac_upwind(m_h, on ? 1 : 0)); }

    /* ---- per-element callbacks (navier_stokes_fv1.h:254-281) --------------- */
    /* checks of prep_elem_loop (navier_stokes_fv1.cpp:136-199) for element type roid */
    void prep_elem_loop(int roid, int /*si*/) {
        if (num_corners(roid) == 0) throw Error(NSFV1_ERR_ARGUMENT, "unsupported element type");
        m_roid = roid;
        m_nsh = num_corners(roid);
        // a zero-size batch runs the disc's setup checks (stabilisation, upwind, viscosity)
        check(nsfv1_elem_batch_host(m_h, roid, 0, nullptr, nullptr, nullptr, 0.0, nullptr, nullptr, nullptr, nullptr, nullptr));
    }
    /* the element state of the following add_* calls: u[(dim+1) * nsh] (LocalVector),
     * corners[nsh * dim]; roid as given to prep_elem_loop */
    void prep_elem(const double* u, int roid, const double* corners) {
        if (roid != m_roid) prep_elem_loop(roid, 0);
        m_u.assign(u, u + (size_t)(m_dim + 1) * m_nsh);
        m_co.assign(corners, corners + (size_t)m_nsh * m_dim);
    }
    /* time-dependent elements: the old-time local solution and the step (the
     * reference takes them from its LocalVectorTimeSeries); nullptr = stationary */
    void set_time_series(const double* u_old, double dt) {
        if (u_old) m_uold.assign(u_old, u_old + (size_t)(m_dim + 1) * m_nsh);
        else m_uold.clear();
        m_dt = dt;
    }
    void fsh_elem_loop() {}
    void add_def_A_elem(double* d) { add_one(d, nullptr, nullptr, nullptr, nullptr); }
    void add_jac_A_elem(double* J) { add_one(nullptr, J, nullptr, nullptr, nullptr); }
    void add_def_M_elem(double* d) { add_one(nullptr, nullptr, d, nullptr, nullptr); }
    void add_jac_M_elem(double* J) { add_one(nullptr, nullptr, nullptr, J, nullptr); }
    void add_rhs_elem(double* d) { add_one(nullptr, nullptr, nullptr, nullptr, d); }

    /* n elements at once: corners[n][nsh][dim], u / u_old [n][(dim+1) nsh]; outputs
     * (each may be nullptr) are OVERWRITTEN: defA, defM, rhs [n][(dim+1) nsh],
     * jacA, jacM [n][((dim+1) nsh)^2] */
    void elem_batch(int roid, int64_t n, const double* corners, const double* u, const double* u_old, double dt, double* defA,
                    double* jacA, double* defM, double* jacM, double* rhs) {
        check(nsfv1_elem_batch_host(m_h, roid, n, corners, u, u_old, dt, defA, jacA, defM, jacM, rhs));
    }

  private:
    static int count_functions(const char* f) {
        if (!f) return 0;
        int n = 0;
        bool tok = false;
        for (const char* p = f;; ++p) {
            const bool sep = (*p == ',' || *p == '\0');
            if (!sep && *p != ' ' && *p != '\t') tok = true;
            if (sep) { if (tok) ++n; tok = false; }
            if (*p == '\0') break;
        }
        return n;
    }
    void create(int dim) {
        m_dim = dim;
        const int st = nsfv1_create(dim, &m_h);
        if (st != NSFV1_OK) throw Error(st, "nsfv1_create failed (dim must be 2 or 3)");
    }
    void check(int st) const {
        if (st != NSFV1_OK) throw Error(st, nsfv1_last_error(m_h));
    }
    void add_one(double* dA, double* jA, double* dM, double* jM, double* r) {
        if (m_u.empty()) throw Error(NSFV1_ERR_STATE, "prep_elem has not been called");
        const size_t nloc = (size_t)(m_dim + 1) * m_nsh;
        std::vector<double> tmp(jA || jM ? nloc * nloc : nloc);
        check(nsfv1_elem_batch_host(m_h, m_roid, 1, m_co.data(), m_u.data(), m_uold.empty() ? nullptr : m_uold.data(), m_dt,
                                    dA ? tmp.data() : nullptr, jA ? tmp.data() : nullptr, dM ? tmp.data() : nullptr,
                                    jM ? tmp.data() : nullptr, r ? tmp.data() : nullptr));
        double* out = dA ? dA : jA ? jA : dM ? dM : jM ? jM : r;
        for (size_t i = 0; i < tmp.size(); ++i) out[i] += tmp[i];
    }

    nsfv1_disc* m_h = nullptr;
    int m_dim = 0, m_roid = -1, m_nsh = 0;
    std::string m_subsets;
    std::vector<double> m_u, m_uold, m_co;
    double m_dt = 0.0;
};

}  // namespace nsfv1

#endif  // NSFV1_GB300_HPP
