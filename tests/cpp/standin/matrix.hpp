// Stand-in for zeroslam's source/matrix.hpp, for building the drop-in
// factor graph (include/zeroslam_gb300/factor_graph.hpp) where zeroslam's
// source tree is not available (the GPU test machines). It provides only
// what the drop-in and its tests use, with zeroslam's semantics:
//   * matrix<T, R, C> (fixed size, row-major): zero-initialised; built from
//     a flat array ({{a, b, c}}) or an array of rows; zero(), identity(),
//     data(), rows(), cols(); operator[] gives the element of a row or column
//     vector and a row pointer otherwise (source/matrix.hpp:186-209);
//   * matrix<T, 0, 0> (sized at run time): (rows, cols), (rows, cols,
//     values), zero(rows, cols), identity(rows, cols), data(), rows(),
//     cols(), size(); operator[] gives a row pointer (source/matrix.hpp:370-378).
// The header name and namespace are zeroslam's so that the drop-in compiles
// unchanged against either.
#pragma once

#include <cstddef>
#include <type_traits>
#include <vector>

namespace matrix {

template <typename T, std::size_t R, std::size_t C>
class matrix {
    T v[R * C] = {};

public:
    constexpr matrix() = default;
    constexpr matrix(const T (&values)[R * C]) {
        for (std::size_t i = 0; i < R * C; ++i) v[i] = values[i];
    }
    template <std::size_t RR = R, std::size_t CC = C, typename = typename std::enable_if<(RR > 1 && CC > 1)>::type>
    constexpr matrix(const T (&rows_values)[R][C]) {
        for (std::size_t i = 0; i < R; ++i)
            for (std::size_t j = 0; j < C; ++j) v[i * C + j] = rows_values[i][j];
    }
    static constexpr matrix zero() {
        return matrix();
    }
    static constexpr matrix identity() {
        matrix m;
        for (std::size_t i = 0; i < R && i < C; ++i) m.v[i * C + i] = T(1);
        return m;
    }
    constexpr std::size_t rows() const {
        return R;
    }
    constexpr std::size_t cols() const {
        return C;
    }
    constexpr const T* data() const {
        return v;
    }
    constexpr T* data() {
        return v;
    }
    // vectors: the element; matrices: the row
    template <std::size_t RR = R, std::size_t CC = C>
    constexpr typename std::enable_if<(RR == 1 || CC == 1), const T&>::type operator[](std::size_t i) const {
        return v[i];
    }
    template <std::size_t RR = R, std::size_t CC = C>
    constexpr typename std::enable_if<(RR == 1 || CC == 1), T&>::type operator[](std::size_t i) {
        return v[i];
    }
    template <std::size_t RR = R, std::size_t CC = C>
    constexpr typename std::enable_if<!(RR == 1 || CC == 1), const T*>::type operator[](std::size_t i) const {
        return v + i * C;
    }
    template <std::size_t RR = R, std::size_t CC = C>
    constexpr typename std::enable_if<!(RR == 1 || CC == 1), T*>::type operator[](std::size_t i) {
        return v + i * C;
    }
};

template <typename T>
class matrix<T, 0, 0> {
    std::size_t r = 0, c = 0;
    std::vector<T> v;

public:
    matrix() = default;
    matrix(std::size_t rows, std::size_t cols) : r(rows), c(cols), v(rows * cols, T(0)) {
    }
    matrix(std::size_t rows, std::size_t cols, const T* values) : r(rows), c(cols), v(values, values + rows * cols) {
    }
    static matrix zero(std::size_t rows, std::size_t cols) {
        return matrix(rows, cols);
    }
    static matrix identity(std::size_t rows, std::size_t cols) {
        matrix m(rows, cols);
        for (std::size_t i = 0; i < rows && i < cols; ++i) m.v[i * cols + i] = T(1);
        return m;
    }
    std::size_t rows() const {
        return r;
    }
    std::size_t cols() const {
        return c;
    }
    std::size_t size() const {
        return v.size();
    }
    const T* data() const {
        return v.data();
    }
    T* data() {
        return v.data();
    }
    const T* operator[](std::size_t i) const {
        return v.data() + i * c;
    }
    T* operator[](std::size_t i) {
        return v.data() + i * c;
    }
};

}  // namespace matrix
