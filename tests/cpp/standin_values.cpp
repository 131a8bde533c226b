// Prints values of the matrix / lie / camera operations the drop-in factor
// graph uses, one per line, so that the stand-in headers (tests/cpp/standin)
// can be compared with zeroslam's own (compiled once against each).
#include <cstdio>

#include "camera.hpp"
#include "lie.hpp"
#include "matrix.hpp"

static void put(const char* what, double v) {
    std::printf("%s %.17g\n", what, v);
}

int main() {
    const double quats[3][4] = {{1, 0, 0, 0}, {0.9238795325112867, 0.3826834323650898, 0, 0}, {0.5, 0.5, -0.5, 0.5}};
    for (const auto& q : quats) {
        const matrix::matrix<double, 3, 3> R = lie::so3<double>(q[0], q[1], q[2], q[3]).get_matrix();
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) put("R", R[i][j]);
    }
    const double twists[4][6] = {{0, 0, 0, 0.1, -0.2, 0.3},
                                 {1e-9, -2e-9, 3e-9, 0.5, 0.25, -1},
                                 {0.3, -0.1, 0.2, 0.4, 0.5, -0.6},
                                 {2.0, 1.0, -0.5, -1, 2, 0.5}};
    const lie::se3<double> base(lie::so3<double>(0.5, 0.5, -0.5, 0.5), matrix::matrix<double, 3, 1>{{0.1, 0.2, 0.3}});
    for (const auto& t : twists) {
        const matrix::matrix<double, 6, 1> d{{t[0], t[1], t[2], t[3], t[4], t[5]}};
        const lie::se3<double> e = lie::se3<double>::exp(d);
        const matrix::matrix<double, 4, 1> q = e.rotation().get_quaternion();
        for (int i = 0; i < 4; ++i) put("q", q[i]);
        for (int i = 0; i < 3; ++i) put("t", e.translation()[i]);
        const lie::se3<double> c = e * base;
        const matrix::matrix<double, 3, 1> p = c * matrix::matrix<double, 3, 1>{{1.0, -2.0, 5.0}};
        for (int i = 0; i < 3; ++i) put("Tp", p[i]);
    }
    const double intr[4] = {500.0, 510.0, 320.0, 240.0};
    camera::pinhole cam(intr, 4);
    double got[4];
    cam.get_parameters(got, 4);
    for (double v : got) put("intr", v);
    const double pts[3][3] = {{0.1, -0.2, 2.0}, {0.0, 0.0, 1e-13}, {0.3, 0.1, -1.0}};
    for (const auto& X : pts) {
        double uv[2] = {0, 0}, J[6] = {0, 0, 0, 0, 0, 0};
        const bool ok = cam.project(X, uv, J);
        put("ok", ok ? 1.0 : 0.0);
        if (!ok) continue;
        put("u", uv[0]);
        put("v", uv[1]);
        for (double j : J) put("J", j);
    }
    return 0;
}
