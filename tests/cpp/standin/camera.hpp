// Stand-in for zeroslam's source/camera.hpp (see matrix.hpp beside it for
// why): the pinhole model the drop-in factor graph uses, with zeroslam's
// behaviour (source/camera.hpp:26-130): parameters (fx, fy, cx, cy); a point
// projects to (fx x / z + cx, fy y / z + cy) unless its depth z is below
// 1e-12 (then project() returns false); the optional 2 x 3 Jacobian is
// row-major.
#pragma once

#include <cstddef>

namespace camera {

class pinhole {
    double f[2] = {1.0, 1.0};
    double c[2] = {0.5, 0.5};

public:
    pinhole() = default;
    pinhole(const double* p, std::size_t n) {
        if (n >= 4) {
            f[0] = p[0];
            f[1] = p[1];
            c[0] = p[2];
            c[1] = p[3];
        }
    }
    void get_parameters(double* p, std::size_t n) const {
        if (n >= 4) {
            p[0] = f[0];
            p[1] = f[1];
            p[2] = c[0];
            p[3] = c[1];
        }
    }
    bool project(const double* xyz, double* uv, double* jacobian = nullptr, double* jacobian_parameters = nullptr) const {
        (void)jacobian_parameters;
        if (xyz[2] < 1.0e-12) return false;
        const double iz = 1.0 / xyz[2];
        uv[0] = f[0] * (xyz[0] * iz) + c[0];
        uv[1] = f[1] * (xyz[1] * iz) + c[1];
        if (jacobian) {
            const double iz2 = iz * iz;
            jacobian[0] = f[0] * iz;
            jacobian[1] = 0.0;
            jacobian[2] = -f[0] * xyz[0] * iz2;
            jacobian[3] = 0.0;
            jacobian[4] = f[1] * iz;
            jacobian[5] = -f[1] * xyz[1] * iz2;
        }
        return true;
    }
};

}  // namespace camera
