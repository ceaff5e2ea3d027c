// Host-side check of the hand-written reverse routines (phd_adjoint.cuh) against
// central finite differences of the forward routines (phd_physics.cuh), compiled for the
// host: the HLL / HLLC flux with and without boost (hll_family_adj), the exact solver
// (exact_flux_adj: Newton root by implicit differentiation, every sampled region), the wave-speed
// estimate (get_waves_adj), the GIZMO pair limiter (gizmo_pair_adj) and the
// MUSCL-Hancock half step (temporal_adj).
//
// For each seeded random case, inputs x, a direction v and output weights a: the
// adjoint gives (J^T a) . v, central differences give a . (F(x + h v) - F(x - h v)) / 2h.
// The forward routines are piecewise smooth (branch switches: wave-speed estimate,
// flux region, limiter clips, positivity reverts); a case whose difference quotients at
// h and 2h disagree crossed a switch and is counted as such, not compared.  Prints per
// routine: cases, cases compared, worst relative difference among them.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <functional>
#include <random>
#include <vector>

#include "phd_adjoint.cuh"

using namespace phd;

struct Stat {
    const char *name;
    long n = 0, compared = 0;
    double worst = 0.;
};

// dot(a, F(x)) for the routine under test
typedef std::function<double(const std::vector<double> &)> Scalar;

static void check(Stat &S, const std::vector<double> &x, const std::vector<double> &v, const Scalar &f,
                  double adj_dot_v) {
    S.n++;
    auto fd = [&](double h) {
        std::vector<double> xp(x), xm(x);
        for (size_t k = 0; k < x.size(); k++) { xp[k] += h * v[k]; xm[k] -= h * v[k]; }
        return (f(xp) - f(xm)) / (2. * h);
    };
    const double h = 1e-6;
    const double d1 = fd(h), d2 = fd(2. * h);
    const double scale = std::fabs(d1) + std::fabs(adj_dot_v) + 1e-300;
    if (std::fabs(d1 - d2) > 1e-6 * scale) return;     // crossed a branch switch
    S.compared++;
    S.worst = std::fmax(S.worst, std::fabs(d1 - adj_dot_v) / scale);
}

int main(int argc, char **argv) {
    const long cases = argc > 1 ? atol(argv[1]) : 4000;
    std::mt19937_64 rng(2024);
    std::uniform_real_distribution<double> U(0., 1.);
    auto u = [&](double a, double b) { return a + (b - a) * U(rng); };
    const double gamma = 1.4;
    Stat hllc{"hllc"}, hll{"hll"}, hllc_lab{"hllc_lab"}, exact{"exact"}, waves{"get_waves"}, gizmo{"gizmo_pair"},
        temp{"temporal"};

    for (long c = 0; c < cases; c++) {
        // ---- HLL / HLLC + deboost ------------------------------------------------
        {
            std::vector<double> x = {u(0.2, 2.), u(-1., 1.), u(-1., 1.), u(0.2, 2.),
                                     u(0.2, 2.), u(-1., 1.), u(-1., 1.), u(0.2, 2.)};
            const double th = u(0., 6.283185307179586);
            const double n[2] = {std::cos(th), std::sin(th)}, w[2] = {u(-.5, .5), u(-.5, .5)};
            std::vector<double> v(8), a(4);
            for (auto &e : v) e = u(-1., 1.);
            for (auto &e : a) e = u(-1., 1.);
            for (int variant = 0; variant < 3; variant++) {
                const bool is_hllc = variant != 1, boost = variant != 2;
                auto f = [&](const std::vector<double> &y) {
                    double F[4];
                    hll_family<double, 2>(is_hllc, y.data(), y.data() + 4, n, w, gamma, boost, F);
                    return a[0] * F[0] + a[1] * F[1] + a[2] * F[2] + a[3] * F[3];
                };
                double aL[4] = {0, 0, 0, 0}, aR[4] = {0, 0, 0, 0};
                hll_family_adj<double>(is_hllc, x.data(), x.data() + 4, n, w, gamma, boost, a.data(), aL, aR);
                double dot = 0.;
                for (int k = 0; k < 4; k++) dot += aL[k] * v[k] + aR[k] * v[4 + k];
                check(variant == 0 ? hllc : (variant == 1 ? hll : hllc_lab), x, v, f, dot);
            }
        }
        // ---- exact solver + deboost (states spanning shocks, rarefactions and fans) ----
        {
            std::vector<double> x = {u(0.2, 2.), u(-2., 2.), u(-2., 2.), u(0.1, 3.),
                                     u(0.2, 2.), u(-2., 2.), u(-2., 2.), u(0.1, 3.)};
            const double th = u(0., 6.283185307179586);
            const double n[2] = {std::cos(th), std::sin(th)}, w[2] = {u(-.5, .5), u(-.5, .5)};
            std::vector<double> v(8), a(4);
            for (auto &e : v) e = u(-1., 1.);
            for (auto &e : a) e = u(-1., 1.);
            auto f = [&](const std::vector<double> &y) {
                double F[4];
                bool failed = false;
                exact_flux<double, 2>(y.data(), y.data() + 4, n, w, gamma, 1000, F, &failed);
                return a[0] * F[0] + a[1] * F[1] + a[2] * F[2] + a[3] * F[3];
            };
            double aL[4] = {0, 0, 0, 0}, aR[4] = {0, 0, 0, 0};
            exact_flux_adj(x.data(), x.data() + 4, n, w, gamma, 1000, a.data(), aL, aR);
            double dot = 0.;
            for (int k = 0; k < 4; k++) dot += aL[k] * v[k] + aR[k] * v[4 + k];
            check(exact, x, v, f, dot);
        }
        // ---- wave speeds -------------------------------------------------------------
        {
            std::vector<double> x = {u(0.2, 2.), u(-2., 2.), u(0.05, 3.), u(0.2, 2.), u(-2., 2.), u(0.05, 3.)};
            std::vector<double> v(6), a(3);
            for (auto &e : v) e = u(-1., 1.);
            for (auto &e : a) e = u(-1., 1.);
            auto f = [&](const std::vector<double> &y) {
                double sl, sc, sr;
                get_waves<double>(y[0], y[1], y[2], y[3], y[4], y[5], gamma, sl, sc, sr);
                return a[0] * sl + a[1] * sc + a[2] * sr;
            };
            double g[6] = {0, 0, 0, 0, 0, 0};
            get_waves_adj<double>(x[0], x[1], x[2], x[3], x[4], x[5], gamma, a[0], a[1], a[2], g[0], g[1], g[2],
                                  g[3], g[4], g[5]);
            double dot = 0.;
            for (int k = 0; k < 6; k++) dot += g[k] * v[k];
            check(waves, x, v, f, dot);
        }
        // ---- GIZMO pair limiter: sl, sr, xl, xr (ci, cj and the geometry fixed) ------
        {
            std::vector<double> x = {u(-1., 1.), u(-1., 1.), u(-1.5, 1.5), u(-1.5, 1.5)};
            const double ci = x[0] + u(-.1, .1), cj = x[1] + u(-.1, .1);
            const double smi = u(.2, .8), smj = u(.2, .8), dm = u(.8, 1.2);
            std::vector<double> v(4), a(2);
            for (auto &e : v) e = u(-1., 1.);
            for (auto &e : a) e = u(-1., 1.);
            auto f = [&](const std::vector<double> &y) {
                double xl = y[2], xr = y[3];
                gizmo_pair<double>(y[0], y[1], ci, cj, smi, smj, dm, xl, xr);
                return a[0] * xl + a[1] * xr;
            };
            double asl = 0., asr = 0., axl = 0., axr = 0.;
            gizmo_pair_adj<double>(x[0], x[1], ci, cj, smi, smj, dm, x[2], x[3], a[0], a[1], asl, asr, axl, axr);
            check(gizmo, x, v, f, asl * v[0] + asr * v[1] + axl * v[2] + axr * v[3]);
        }
        // ---- MUSCL-Hancock half step: L, R, cell values, gradients --------------------
        {
            std::vector<double> x(4 + 4 + 4 + 4 + 8 + 8);
            double *Lin = x.data(), *Rin = Lin + 4, *pi = Rin + 4, *pj = pi + 4, *gi = pj + 4, *gj = gi + 8;
            for (double *s : {Lin, Rin, pi, pj}) {
                s[0] = u(0.5, 2.);
                s[1] = u(-1., 1.);
                s[2] = u(-1., 1.);
                s[3] = u(0.5, 2.);
            }
            for (int k = 0; k < 8; k++) { gi[k] = u(-2., 2.); gj[k] = u(-2., 2.); }
            const double w[2] = {u(-.3, .3), u(-.3, .3)}, dt = u(0.005, 0.05);
            const bool boost = (c % 2) == 0;
            std::vector<double> v(x.size()), a(8);
            for (auto &e : v) e = u(-1., 1.);
            for (auto &e : a) e = u(-1., 1.);
            auto f = [&](const std::vector<double> &y) {
                double L[4], R[4];
                for (int k = 0; k < 4; k++) { L[k] = y[k]; R[k] = y[4 + k]; }
                temporal<double, 2>(L, R, y.data() + 8, y.data() + 12, y.data() + 16, y.data() + 24, w, gamma, dt,
                                    boost);
                double s = 0.;
                for (int k = 0; k < 4; k++) s += a[k] * L[k] + a[4 + k] * R[k];
                return s;
            };
            std::vector<double> g(x.size(), 0.);
            temporal_adj<double>(Lin, Rin, pi, pj, gi, gj, w, gamma, dt, boost, a.data(), a.data() + 4, g.data(),
                                 g.data() + 4, g.data() + 8, g.data() + 12, g.data() + 16, g.data() + 24);
            double dot = 0.;
            for (size_t k = 0; k < x.size(); k++) dot += g[k] * v[k];
            check(temp, x, v, f, dot);
        }
    }
    for (const Stat &S : {hllc, hll, hllc_lab, exact, waves, gizmo, temp})
        printf("%s %ld %ld %.6e\n", S.name, S.n, S.compared, S.worst);
    return 0;
}
