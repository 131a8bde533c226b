// Stand-in for zeroslam's source/lie.hpp (see matrix.hpp beside it for why):
// the rotations and rigid transforms the drop-in factor graph uses, with
// zeroslam's conventions:
//   * so3(w, x, y, z) keeps the quaternion as given (no normalisation),
//     get_quaternion() returns it as (w, x, y, z), get_matrix() is the
//     rotation matrix of a unit quaternion (source/lie.hpp:133-145, 183-201);
//   * se3(rotation, translation) maps x to R x + t; products compose
//     (a * b)(x) = a(b(x)); exp((omega, upsilon)) is the exponential of the
//     twist with the rotation part first (source/lie.hpp:64-88).
// Small angles use the series of the same functions.
#pragma once

#include <cmath>

#include "matrix.hpp"

namespace lie {

template <typename T>
class so3 {
    T q[4] = {T(1), T(0), T(0), T(0)};  // w, x, y, z

public:
    so3() = default;
    so3(T w, T x, T y, T z) : q{w, x, y, z} {
    }
    matrix::matrix<T, 4, 1> get_quaternion() const {
        return matrix::matrix<T, 4, 1>({q[0], q[1], q[2], q[3]});
    }
    matrix::matrix<T, 3, 3> get_matrix() const {
        const T w = q[0], x = q[1], y = q[2], z = q[3];
        matrix::matrix<T, 3, 3> m;
        T* r = m.data();
        r[0] = T(1) - T(2) * (y * y + z * z);
        r[1] = T(2) * (x * y - w * z);
        r[2] = T(2) * (x * z + w * y);
        r[3] = T(2) * (x * y + w * z);
        r[4] = T(1) - T(2) * (x * x + z * z);
        r[5] = T(2) * (y * z - w * x);
        r[6] = T(2) * (x * z - w * y);
        r[7] = T(2) * (y * z + w * x);
        r[8] = T(1) - T(2) * (x * x + y * y);
        return m;
    }
    // exp of the rotation vector omega (angle |omega| about omega / |omega|)
    static so3 exp(const matrix::matrix<T, 3, 1>& omega) {
        const T t2 = omega[0] * omega[0] + omega[1] * omega[1] + omega[2] * omega[2];
        const T t = std::sqrt(t2);
        T c, s;  // cos(t / 2), sin(t / 2) / t
        if (t < T(1e-8)) {
            c = T(1) - t2 / T(8);
            s = T(0.5) - t2 / T(48);
        } else {
            c = std::cos(t / T(2));
            s = std::sin(t / T(2)) / t;
        }
        return so3(c, s * omega[0], s * omega[1], s * omega[2]);
    }
    so3 operator*(const so3& b) const {
        const T* a = q;
        return so3(a[0] * b.q[0] - a[1] * b.q[1] - a[2] * b.q[2] - a[3] * b.q[3],
                   a[0] * b.q[1] + a[1] * b.q[0] + a[2] * b.q[3] - a[3] * b.q[2],
                   a[0] * b.q[2] - a[1] * b.q[3] + a[2] * b.q[0] + a[3] * b.q[1],
                   a[0] * b.q[3] + a[1] * b.q[2] - a[2] * b.q[1] + a[3] * b.q[0]);
    }
    matrix::matrix<T, 3, 1> operator*(const matrix::matrix<T, 3, 1>& p) const {
        const matrix::matrix<T, 3, 3> m = get_matrix();
        matrix::matrix<T, 3, 1> out;
        for (int i = 0; i < 3; ++i) out[i] = m[i][0] * p[0] + m[i][1] * p[1] + m[i][2] * p[2];
        return out;
    }
};

template <typename T>
class se3 {
    so3<T> rot;
    matrix::matrix<T, 3, 1> trans;

public:
    se3() = default;
    se3(const so3<T>& r, const matrix::matrix<T, 3, 1>& t) : rot(r), trans(t) {
    }
    const so3<T>& rotation() const {
        return rot;
    }
    const matrix::matrix<T, 3, 1>& translation() const {
        return trans;
    }
    // twist (omega, upsilon): rotation exp(omega), translation V(omega) upsilon
    static se3 exp(const matrix::matrix<T, 6, 1>& d) {
        const T w[3] = {d[0], d[1], d[2]}, u[3] = {d[3], d[4], d[5]};
        const T t2 = w[0] * w[0] + w[1] * w[1] + w[2] * w[2];
        const T t = std::sqrt(t2);
        T a, b;  // V = I + a [w]x + b [w]x^2
        if (t < T(1e-8)) {
            a = T(0.5) - t2 / T(24);
            b = T(1) / T(6) - t2 / T(120);
        } else {
            a = (T(1) - std::cos(t)) / t2;
            b = (t - std::sin(t)) / (t2 * t);
        }
        const T wu[3] = {w[1] * u[2] - w[2] * u[1], w[2] * u[0] - w[0] * u[2], w[0] * u[1] - w[1] * u[0]};
        const T wwu[3] = {w[1] * wu[2] - w[2] * wu[1], w[2] * wu[0] - w[0] * wu[2], w[0] * wu[1] - w[1] * wu[0]};
        matrix::matrix<T, 3, 1> tr;
        for (int i = 0; i < 3; ++i) tr[i] = u[i] + a * wu[i] + b * wwu[i];
        return se3(so3<T>::exp(matrix::matrix<T, 3, 1>({w[0], w[1], w[2]})), tr);
    }
    se3 operator*(const se3& b) const {
        const matrix::matrix<T, 3, 1> rt = rot * b.trans;
        matrix::matrix<T, 3, 1> t;
        for (int i = 0; i < 3; ++i) t[i] = rt[i] + trans[i];
        return se3(rot * b.rot, t);
    }
    matrix::matrix<T, 3, 1> operator*(const matrix::matrix<T, 3, 1>& p) const {
        matrix::matrix<T, 3, 1> out = rot * p;
        for (int i = 0; i < 3; ++i) out[i] += trans[i];
        return out;
    }
};

}  // namespace lie
