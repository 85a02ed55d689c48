// End-to-end cost of the C++ drop-in: the reference's own user code,
//     getV<1>(parts) = Lap(getV<0>(parts));   getV<2>(parts) = Grad(getV<0>(parts));
// (src/Operators/Vector/vector_dist_operators.hpp:1113-1135 evaluates such
// assignments on the host), on 128^3 jittered particles (h = 1/127, jitter
// U(+-0.15h) from std::mt19937_64 seed 2, rCut = 2.8h, order 2), through
// include/openfpm_dcpse with host-resident particle properties.  Times the
// default FP64 expression path (every output in the reference's order, one
// pass per Dcpse term) and the opt-in batched FP32 and budget-driven FP32
// paths; prints one JSON line.  Built and run by bench.py.
#include <array>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>
#include <vector>

#include "openfpm_dcpse/DCPSE_op.hpp"

using namespace openfpm_dcpse;

typedef vector_dist<3, double, double, double, std::array<double, 3>> Parts3;

static double now_s() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

template <typename F>
static double time_ms(F&& fn, int reps) {
    fn();  // warm-up: allocations, first-use layouts
    const double t0 = now_s();
    for (int r = 0; r < reps; ++r) fn();
    return (now_s() - t0) * 1e3 / reps;
}

int main(int argc, char** argv) {
    const int nside = argc > 1 ? std::atoi(argv[1]) : 128;
    const double h = 1.0 / 127.0, rCut = 2.8 * h;
    const std::size_t n = (std::size_t)nside * nside * nside;
    Parts3 parts(n);
    std::mt19937_64 rng(2);
    std::uniform_real_distribution<double> jit(-0.15 * h, 0.15 * h);
    for (int k = 0; k < nside; ++k)
        for (int j = 0; j < nside; ++j)
            for (int i = 0; i < nside; ++i) {
                const std::size_t p = ((std::size_t)k * nside + j) * nside + i;
                parts.getPos(p)[0] = i * h + jit(rng);
                parts.getPos(p)[1] = j * h + jit(rng);
                parts.getPos(p)[2] = k * h + jit(rng);
            }
    for (std::size_t p = 0; p < n; ++p) {
        const double* x = parts.getPos(p);
        const double r2 = (x[0] - 0.5) * (x[0] - 0.5) + (x[1] - 0.5) * (x[1] - 0.5) + (x[2] - 0.5) * (x[2] - 0.5);
        parts.getProp<0>(p) = std::exp(-10.0 * r2) * std::sin(3.0 * M_PI * x[0]);
    }
    double t0 = now_s();
    VerletList vl = getVerlet(parts, rCut);
    const double t_verlet = (now_s() - t0) * 1e3;
    t0 = now_s();
    Laplacian<VerletList> Lap(parts, vl, 2, rCut);
    Gradient<VerletList> Grad(parts, vl, 2, rCut);
    const double t_ops = (now_s() - t0) * 1e3;

    auto lap = [&] { getV<1>(parts) = Lap(getV<0>(parts)); };
    auto grad = [&] { getV<2>(parts) = Grad(getV<0>(parts)); };
    const double lap64 = time_ms(lap, 3), grad64 = time_ms(grad, 3);
    std::vector<double> l64(n);
    std::vector<std::array<double, 3>> g64(n);
    for (std::size_t p = 0; p < n; ++p) {
        l64[p] = parts.getProp<1>(p);
        g64[p] = parts.getProp<2>(p);
    }
    double res[3][3];
    double err[3][2];
    const int precs[3] = {DCPSE_F32, DCPSE_F32_BUDGET, DCPSE_F32_PAIR};
    for (int m = 0; m < 3; ++m) {
        t0 = now_s();
        Lap.set_apply_precision(precs[m]);
        Grad.set_apply_precision(precs[m]);
        res[m][2] = (now_s() - t0) * 1e3;
        res[m][0] = time_ms(lap, 10);
        res[m][1] = time_ms(grad, 10);
        double el = 0, ml = 0, eg = 0, mg = 0;
        for (std::size_t p = 0; p < n; ++p) {
            el = std::max(el, std::fabs(parts.getProp<1>(p) - l64[p]));
            ml = std::max(ml, std::fabs(l64[p]));
            for (int d = 0; d < 3; ++d) {
                eg = std::max(eg, std::fabs(parts.getProp<2>(p)[d] - g64[p][d]));
                mg = std::max(mg, std::fabs(g64[p][d]));
            }
        }
        err[m][0] = el / ml;
        err[m][1] = eg / mg;
    }
    const double nd = (double)n;
    std::printf("{\"particles\": %zu, \"verlet_ms\": %.3f, \"operators_ms\": %.3f, "
                "\"fp64_reference_order\": {\"laplacian_ms\": %.3f, \"gradient_ms\": %.3f, "
                "\"gparticle_ops_s\": %.5f}",
                n, t_verlet, t_ops, lap64, grad64, 4 * nd / ((lap64 + grad64) * 1e6));
    const char* names[3] = {"fp32_batched", "fp32_budget", "fp32_pair"};
    for (int m = 0; m < 3; ++m)
        std::printf(", \"%s\": {\"laplacian_ms\": %.3f, \"gradient_ms\": %.3f, \"gparticle_ops_s\": %.5f, "
                    "\"set_up_ms\": %.3f, \"laplacian_vs_fp64\": %.3e, \"gradient_vs_fp64\": %.3e}",
                    names[m], res[m][0], res[m][1], 4 * nd / ((res[m][0] + res[m][1]) * 1e6), res[m][2], err[m][0],
                    err[m][1]);
    std::printf("}\n");
    return 0;
}
