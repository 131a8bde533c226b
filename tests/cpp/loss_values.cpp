// Prints rho = (rho, rho', rho'') of the Huber, Cauchy and Tukey losses at a
// fixed set of squared errors, from whichever factor_graph.hpp is first on
// the include path: the drop-in or zeroslam's own, so the two can be diffed.
#include "factor_graph.hpp"

#include <cstdio>

int main() {
    const double e2s[] = {0.0, 0.25, 1.0, 3.99, 4.0, 4.01, 9.0, 100.0, 1e6};
    factor_graph::loss_huber h(2.0);
    factor_graph::loss_cauchy c(2.0);
    factor_graph::loss_tukey t(2.0);
    const factor_graph::loss_function_base* losses[] = {&h, &c, &t};
    for (const auto* l : losses) {
        for (double e2 : e2s) {
            matrix::matrix<double, 3, 1> rho = matrix::matrix<double, 3, 1>::zero();
            l->compute(e2, rho);
            std::printf("%.17g %.17g %.17g\n", rho[0], rho[1], rho[2]);
        }
    }
    return 0;
}
