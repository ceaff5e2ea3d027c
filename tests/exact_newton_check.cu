// Host-side check of the FP32 path's FP64 Newton iteration for the exact solver
// (ex_get_pstar_lean: host gamma constants, binomial-series powers, reused powers,
// shared reciprocals) against the reference's iteration restated verbatim
// (ex_get_pstar, riemann.pyx:974-1090), on seeded random Riemann problems: nearly
// uniform states, arbitrary jumps, strong two-rarefaction problems, gammas 1.1-2.1.
// Prints one line: problems, non-converged, disagreements of the convergence flag,
// max relative p* difference (p* above 1e-10 of the larger side pressure), max u*
// difference relative to |u_l| + |u_r| + c_l + c_r, and the integer exponents 2g/(g-1)
// found for g = 1.4 and 5/3 (the two-rarefaction guess's squaring path).
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>

#include "phd_physics.cuh"

using namespace phd;

int main(int argc, char **argv) {
    const long n_prob = argc > 1 ? atol(argv[1]) : 200000;
    std::mt19937_64 rng(12345);
    std::uniform_real_distribution<double> U(0., 1.);
    long n = 0, n_fail = 0, n_flag = 0;
    double worst_p = 0., worst_u = 0.;
    for (long t = 0; t < n_prob; t++) {
        const double gamma = (t % 3 == 0) ? 1.4 : (t % 3 == 1 ? 5. / 3. : 1.1 + U(rng));
        const int kind = int(t % 4);
        const double dl = std::exp(4. * U(rng) - 2.), dr = std::exp(4. * U(rng) - 2.);
        double pl, pr, ul, ur;
        if (kind == 0) {                       // nearly uniform (smooth flow)
            pl = 2.5 * (1. + 1e-3 * (U(rng) - .5));
            pr = 2.5 * (1. + 1e-3 * (U(rng) - .5));
            ul = 0.01 * (U(rng) - .5);
            ur = 0.01 * (U(rng) - .5);
        } else {
            pl = std::exp(12. * U(rng) - 6.);
            pr = std::exp(12. * U(rng) - 6.);
            ul = 4. * (U(rng) - .5);
            ur = 4. * (U(rng) - .5);
        }
        if (kind == 3) { ul = -2. - 2. * U(rng); ur = 2. + 2. * U(rng); }
        const double cl = std::sqrt(gamma * pl / dl), cr = std::sqrt(gamma * pr / dr);
        if (2. * (cl + cr) / (gamma - 1.) <= ur - ul) continue;      // vacuum generated
        bool fa = false, fb = false;
        const double a = ex_get_pstar(dl, ul, pl, cl, dr, ur, pr, cr, gamma, 1000, &fa);
        const ExGas64 X = ex_gas64(gamma);
        double fl, fr;
        const double b = ex_get_pstar_lean(dl, ul, pl, cl, dr, ur, pr, cr, X, 1000, &fb, fl, fr);
        if (fa != fb) n_flag++;
        if (fa || fb) { n_fail++; continue; }
        n++;
        if (a > 1e-10 * std::fmax(pl, pr)) worst_p = std::fmax(worst_p, std::fabs(a - b) / a);
        const double ua = 0.5 * (((ul + ur) + ex_p_func(dr, pr, cr, gamma, a)) - ex_p_func(dl, pl, cl, gamma, a));
        const double ub = 0.5 * (((ul + ur) + fr) - fl);
        worst_u = std::fmax(worst_u, std::fabs(ua - ub) / (std::fabs(ul) + std::fabs(ur) + cl + cr));
    }
    printf("%ld %ld %ld %.6e %.6e %d %d\n", n, n_fail, n_flag, worst_p, worst_u, ex_gas64(1.4).n_inv_z,
           ex_gas64(5. / 3.).n_inv_z);
    return 0;
}
