// A C++ client compiled against include/nsfv1_gb300.hpp / nsfv1_gb300.h and
// linked with libnsfv1_gb300.so, as an application built on the reference's
// element-disc interface would be. Without arguments it runs host-only checks
// (setters, string ids, error texts, the host pattern build). With "gpu" it
// also evaluates the element callbacks of two hexahedra on the GPU, per
// element and batched, and prints them (one number per line) for the test to
// compare with the oracle.
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "nsfv1_gb300.hpp"

static int fails = 0;
#define EXPECT(c)                                                   \
    do {                                                            \
        if (!(c)) { std::printf("FAIL %s:%d %s\n", __FILE__, __LINE__, #c); ++fails; } \
    } while (0)

int main(int argc, char** argv) {
    const bool gpu = argc > 1 && std::strcmp(argv[1], "gpu") == 0;
    nsfv1::NavierStokesFV1 disc("u, v, w, p", "Inner");
    EXPECT(disc.dim() == 3 && disc.disc_type() == "fv1");
    // string ids, as CreateNavierStokesUpwind / CreateNavierStokesStabilization
    disc.set_upwind(" LinearProfileSkewed ");
    disc.set_stabilization("FLOW");
    disc.set_stabilization("flow", "raw");
    bool threw = false;
    try { disc.set_upwind("weighted"); } catch (const nsfv1::Error& e) {
        threw = e.status() == NSFV1_ERR_ARGUMENT && std::string(e.what()).find("not found") != std::string::npos;
    }
    EXPECT(threw);
    threw = false;
    try { disc.set_stabilization("fields", "bogus"); } catch (const nsfv1::Error& e) {
        threw = std::string(e.what()).find("Diffusion Length") != std::string::npos;
    }
    EXPECT(threw);
    threw = false;
    try { nsfv1::NavierStokesFV1 bad("u,v", "Inner"); } catch (const nsfv1::Error&) { threw = true; }
    EXPECT(threw);
    // prep_elem_loop without a viscosity: the reference's text
    threw = false;
    try { disc.prep_elem_loop(NSFV1_HEXAHEDRON, 0); } catch (const nsfv1::Error& e) {
        threw = std::string(e.what()).find("Kinematic Viscosity has not been set") != std::string::npos;
    }
    EXPECT(threw);
    disc.set_kinematic_viscosity(0.0025);
    disc.set_density(1.0);
    disc.set_exact_jacobian(false);
    // host-only block-CSR pattern of a 2 x 1 x 1 hexahedral strip: 12 nodes, every pair of an element
    const int32_t conn[16] = {0, 1, 4, 3, 6, 7, 10, 9, 1, 2, 5, 4, 7, 8, 11, 10};
    int64_t nnz = 0;
    int ncol = 0;
    EXPECT(nsfv1_mesh_pattern(NSFV1_HEXAHEDRON, 12, 2, conn, &nnz, &ncol, nullptr, nullptr, nullptr) == NSFV1_OK);
    EXPECT(nnz == 8 * 8 + 4 * 12 && ncol == 2);
    if (gpu) {
        disc.prep_elem_loop(NSFV1_HEXAHEDRON, 0);
        const int nsh = 8, nloc = 32;
        std::vector<double> co(2 * nsh * 3), u(2 * nloc);
        const double ref[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0}, {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
        for (int e = 0; e < 2; ++e)
            for (int k = 0; k < nsh; ++k)
                for (int d = 0; d < 3; ++d) co[(e * nsh + k) * 3 + d] = 0.1 * (ref[k][d] + 0.07 * ((k * 3 + d + e) % 5 - 2)) + e;
        for (int i = 0; i < 2 * nloc; ++i) u[i] = 0.5 * ((i * 37 % 23) / 11.0 - 1.0);
        std::vector<double> dA(2 * nloc, 0.0), jA(2 * nloc * nloc, 0.0), dB(2 * nloc), jB(2 * nloc * nloc);
        for (int e = 0; e < 2; ++e) {
            disc.prep_elem(&u[e * nloc], NSFV1_HEXAHEDRON, &co[e * nsh * 3]);
            disc.add_def_A_elem(&dA[e * nloc]);
            disc.add_jac_A_elem(&jA[e * nloc * nloc]);
        }
        disc.fsh_elem_loop();
        disc.elem_batch(NSFV1_HEXAHEDRON, 2, co.data(), u.data(), nullptr, 0.0, dB.data(), jB.data(), nullptr, nullptr, nullptr);
        for (size_t i = 0; i < dA.size(); ++i) EXPECT(dA[i] == dB[i]);
        for (size_t i = 0; i < jA.size(); ++i) EXPECT(jA[i] == jB[i]);
        for (double x : co) std::printf("C %.17g\n", x);
        for (double x : u) std::printf("U %.17g\n", x);
        for (double x : dA) std::printf("D %.17g\n", x);
        for (double x : jA) std::printf("J %.17g\n", x);
    }
    std::printf(fails ? "FAILED %d\n" : "OK\n", fails);
    return fails ? 1 : 0;
}
