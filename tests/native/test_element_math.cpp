// Checks the product's closed-form element derivatives against the oracle's
// forward-mode dual numbers (the reference's differentiation scheme) on
// random element states.  Built and run by tests/test_element_math.py.
#include "khs_device_math.cuh"
#include "khs_oracle_math.hpp"

#include <cstdio>
#include <random>

using namespace khs_oracle;
namespace dm = khs::dm;

static M3 random_rotation(std::mt19937_64 &g)
{
    std::normal_distribution<double> n(0.0, 1.0);
    V3 a = normalized(v3(n(g), n(g), n(g)));
    V3 b = normalized(v3(n(g), n(g), n(g)));
    return frame_from_tangent(a, b);
}

int main()
{
    std::mt19937_64 g(1234);
    std::uniform_real_distribution<double> u(-1.0, 1.0);
    double worst_e = 0, worst_g = 0, worst_h = 0, worst_eps = 0;
    const double radius = 4e-5, young = 3e9, poisson = 0.25, kappa = 0.9;
    const dm::Weights w = dm::strain_weights(radius, young, poisson, kappa);
    for (int trial = 0; trial < 4000; ++trial) {
        const M3 refi = random_rotation(g), refj = random_rotation(g);
        const double L0 = 0.002 * (1.0 + 0.5 * u(g));
        // Rotation magnitudes from exactly zero (Taylor branch) up to ~pi.
        const double scale = trial % 4 == 0 ? 0.0 : (trial % 4 == 1 ? 1e-6 : (trial % 4 == 2 ? 1e-3 : 1.0));
        double q[12];
        for (int k = 0; k < 3; ++k) { q[k] = 0.1 * u(g); q[6 + k] = q[k] + 0.5 * L0 * u(g); }
        for (int k = 0; k < 3; ++k) { q[3 + k] = scale * u(g); q[9 + k] = scale * u(g); }
        const V3 g0 = v3(0.01 * u(g), 0.01 * u(g), 1.0 + 0.01 * u(g)), k0 = v3(10 * u(g), 10 * u(g), 10 * u(g));
        // Oracle: Dual<12> exactly as the reference differentiates.
        Dual<12> dq[12];
        for (int d = 0; d < 12; ++d) dq[d] = Dual<12>::var(q[d], d);
        DV3<12> xi{dq[0], dq[1], dq[2]}, ui{dq[3], dq[4], dq[5]}, xj{dq[6], dq[7], dq[8]}, uj{dq[9], dq[10], dq[11]};
        DM3<12> Ri, Rj;
        {
            DM3<12> a, b;
            for (int k = 0; k < 9; ++k) { a.m[k] = Dual<12>(refi.m[k]); b.m[k] = Dual<12>(refj.m[k]); }
            Ri = dm_mul(dexp_so3(ui), a);
            Rj = dm_mul(dexp_so3(uj), b);
        }
        const DV3<12> t = dvscale(dvsub(xj, xi), Dual<12>(1.0 / L0));
        const DV3<12> shear = dvscale(dm_vec(dm_add(dm_transpose(Ri), dm_transpose(Rj)), t), Dual<12>(0.5));
        const DV3<12> curv = dvscale(dcayley(dm_mul(dm_transpose(Ri), Rj)), Dual<12>(1.0 / L0));
        Dual<12> strain[6] = {shear.x - Dual<12>(g0.x), shear.y - Dual<12>(g0.y), shear.z - Dual<12>(g0.z),
                              curv.x - Dual<12>(k0.x), curv.y - Dual<12>(k0.y), curv.z - Dual<12>(k0.z)};
        Dual<12> re(0.0);
        for (int s = 0; s < 6; ++s) re = re + Dual<12>(0.5 * L0 * w.w[s]) * strain[s] * strain[s];
        // Product: closed form.
        dm::M Rpi, Rpj, Jli, Jlj;
        dm::rotation_and_jacobian(dm::v(q[3], q[4], q[5]), refi.m, Rpi, &Jli);
        dm::rotation_and_jacobian(dm::v(q[9], q[10], q[11]), refj.m, Rpj, &Jlj);
        double eps[6];
        dm::ElementJacobian J;
        dm::element_strain(Rpi, Rpj, dm::v(q[0], q[1], q[2]), dm::v(q[6], q[7], q[8]), L0, dm::v(g0.x, g0.y, g0.z),
                           dm::v(k0.x, k0.y, k0.z), eps, &J, &Jli, &Jlj);
        const double e = dm::element_energy(eps, w, L0);
        double gi[6], gj[6], Hii[36], Hjj[36], Hij[36];
        dm::element_gradient(J, eps, w, L0, gi, gj);
        dm::element_hessian(J, w, L0, Hii, Hjj, Hij);
        // Compare.
        double emax = 0, gmax = 0, hmax = 0;
        for (int s = 0; s < 6; ++s) worst_eps = std::max(worst_eps, std::fabs(eps[s] - strain[s].v) / (1e-3 + std::fabs(strain[s].v)));
        emax = std::fabs(e - re.v) / (1e-30 + std::fabs(re.v));
        double gscale = 0;
        for (int d = 0; d < 12; ++d) gscale = std::max(gscale, std::fabs(re.d[d]));
        for (int d = 0; d < 6; ++d) {
            gmax = std::max(gmax, std::fabs(gi[d] - re.d[d]) / gscale);
            gmax = std::max(gmax, std::fabs(gj[d] - re.d[6 + d]) / gscale);
        }
        double hscale = 0;
        double Hd[12][12];
        for (int a = 0; a < 12; ++a)
            for (int b = 0; b < 12; ++b) {
                double h = 0;
                for (int s = 0; s < 6; ++s) h += L0 * w.w[s] * strain[s].d[a] * strain[s].d[b];
                Hd[a][b] = h;
                hscale = std::max(hscale, std::fabs(h));
            }
        for (int a = 0; a < 6; ++a)
            for (int b = 0; b < 6; ++b) {
                hmax = std::max(hmax, std::fabs(Hii[6 * a + b] - Hd[a][b]) / hscale);
                hmax = std::max(hmax, std::fabs(Hjj[6 * a + b] - Hd[6 + a][6 + b]) / hscale);
                hmax = std::max(hmax, std::fabs(Hij[6 * a + b] - Hd[a][6 + b]) / hscale);
            }
        worst_e = std::max(worst_e, emax);
        worst_g = std::max(worst_g, gmax);
        worst_h = std::max(worst_h, hmax);
    }
    std::printf("strain %.3e energy %.3e gradient %.3e hessian %.3e\n", worst_eps, worst_e, worst_g, worst_h);
    const bool ok = worst_eps < 1e-9 && worst_e < 1e-9 && worst_g < 1e-9 && worst_h < 1e-9;
    std::printf(ok ? "PASS\n" : "FAIL\n");
    return ok ? 0 : 1;
}
