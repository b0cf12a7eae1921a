// Invariants of the operator surface (include/mbcg_operators.cuh), in FP64, for D3Q27 and D3Q19:
//   sum_i w_i = 1,  sum_i B_i = 1/3  (stencil_ct.cuh),
//   sum_i w_i cos2rule_i(F) = cs^2 = 1/3  (cos2rule omits 1/|c_i|^2, forces.cuh:92-94),
//   sum_i Omega2_i = 0 and sum_i Omega2_i c_i = 0 for |F| > 1e-4  (collisionOperators.cuh:16-25),
//   sum_i recolorDelta_i = 0  (collisionOperators.cuh:60-80: c_i and -c_i cancel).
// Prints one line per failure and exits 1 if any; prints "ok" and exits 0 otherwise.
#include <cmath>
#include <cstdio>
#include <random>

#include "mbcg_operators.cuh"

using namespace mbcg::ops;

static int failures = 0;

static void expect_near(const char* what, const char* lattice, double got, double want, double tol) {
    if (!(std::fabs(got - want) <= tol)) {
        std::printf("%s %s: %.17g, expected %.17g (tolerance %.3g)\n", lattice, what, got, want, tol);
        ++failures;
    }
}

template <typename L>
static void check(const char* name) {
    double sw = 0.0, sb = 0.0;
    constexpr_for<0, L::q>([&](auto Ic) {
        constexpr label_t i = decltype(Ic)::value;
        sw += L::template w<i, double>();
        sb += L::template B<i, double>();
    });
    expect_near("sum w", name, sw, 1.0, 1e-15);
    expect_near("sum B", name, sb, 1.0 / 3.0, 1e-15);

    OpParams<double> k{};
    k.beta_recolor = 0.7;
    std::mt19937_64 rng(12345);
    std::uniform_real_distribution<double> u(-1.0, 1.0);
    for (int t = 0; t < 200; ++t) {
        const double s = std::pow(10.0, -3.0 * (t % 4) / 3.0); // |F| from ~1 down to ~1e-3
        const double Fx = s * u(rng), Fy = s * u(rng), Fz = s * u(rng);
        const double absF = absforce_calcul(Fx, Fy, Fz);
        if (!(absF > 1e-4)) continue;
        const double A = 0.5 + 0.5 * u(rng);
        const double rr = 0.5 + 0.5 * u(rng), rb = 0.5 + 0.5 * u(rng);
        double c2 = 0.0, om = 0.0, omx = 0.0, omy = 0.0, omz = 0.0, dl = 0.0, scale = 0.0, dscale = 0.0;
        constexpr_for<0, L::q>([&](auto Ic) {
            constexpr label_t i = decltype(Ic)::value;
            const double wi = L::template w<i, double>();
            c2 += wi * cos2rule<i, L>(Fx, Fy, Fz, absF);
            const double o = Omega2<i, L>(Fx, Fy, Fz, absF, A);
            om += o;
            omx += o * L::template cx<i>();
            omy += o * L::template cy<i>();
            omz += o * L::template cz<i>();
            scale += std::fabs(o);
            const double d = recolorDelta<i, L>(rr, rb, Fx, Fy, Fz, absF, k);
            dl += d;
            dscale += std::fabs(d);
        });
        expect_near("sum w cos2rule", name, c2, 1.0 / 3.0, 1e-14);
        expect_near("sum Omega2", name, om, 0.0, 1e-14 * scale);
        expect_near("sum Omega2 cx", name, omx, 0.0, 1e-14 * scale);
        expect_near("sum Omega2 cy", name, omy, 0.0, 1e-14 * scale);
        expect_near("sum Omega2 cz", name, omz, 0.0, 1e-14 * scale);
        expect_near("sum recolorDelta", name, dl, 0.0, 1e-15 * dscale);
    }
}

int main() {
    check<D3Q27>("D3Q27");
    check<D3Q19>("D3Q19");
    if (failures) return 1;
    std::printf("ok\n");
    return 0;
}
