// Builds a factor graph with the drop-in's classes the way zeroslam's map
// code does (poses as vertex_pose, points as marginalised vertex_point_xyz,
// one edge_reprojection<camera::pinhole> per observation with the graph's
// loss and information), runs factor_graph::solve() on the device and writes
// the solved vertices back out.
//
//   dropin_solve <scene file> <result file>
//
// Scene file (little-endian): int32 K, L, M, iterations, use_relative,
// loss_kind, has_info, precision; float64 loss_delta, intrinsics[4],
// poses[K][7] (tx ty tz qx qy qz qw), landmarks[L][3]; uint8 pose_fixed[K],
// landmark_fixed[L]; int32 obs_pose[M], obs_landmark[M]; float64
// obs_uv[M][2], then obs_info[M][4] when has_info.
// Result file: int32 solve's return value; float64 chi before, chi after,
// poses[K][7], landmarks[L][3].
#include "factor_graph.hpp"

#include <cstdint>
#include <cstdio>
#include <memory>
#include <vector>

namespace {

template <typename T>
bool read(std::FILE* f, T* v, std::size_t n) {
    return std::fread(v, sizeof(T), n, f) == n;
}

matrix::matrix<double, 0, 0> column(const double* v, std::size_t n) {
    return matrix::matrix<double, 0, 0>(n, 1, v);
}

}  // namespace

int main(int argc, char** argv) {
    if (argc != 3) {
        std::fprintf(stderr, "usage: dropin_solve <scene> <result>\n");
        return 2;
    }
    std::FILE* f = std::fopen(argv[1], "rb");
    if (!f) return 2;
    int32_t hdr[8];
    double loss_delta, intr[4];
    if (!read(f, hdr, 8) || !read(f, &loss_delta, 1) || !read(f, intr, 4)) return 2;
    const int K = hdr[0], L = hdr[1], M = hdr[2], iterations = hdr[3], use_relative = hdr[4], loss_kind = hdr[5],
              has_info = hdr[6], precision = hdr[7];
    std::vector<double> poses(7 * (std::size_t)K), lms(3 * (std::size_t)L), uv(2 * (std::size_t)M),
        info(has_info ? 4 * (std::size_t)M : 0);
    std::vector<uint8_t> pfix(K), lfix(L);
    std::vector<int32_t> op(M), ol(M);
    if (!read(f, poses.data(), poses.size()) || !read(f, lms.data(), lms.size()) || !read(f, pfix.data(), pfix.size()) ||
        !read(f, lfix.data(), lfix.size()) || !read(f, op.data(), op.size()) || !read(f, ol.data(), ol.size()) ||
        !read(f, uv.data(), uv.size()) || (has_info && !read(f, info.data(), info.size())))
        return 2;
    std::fclose(f);

    camera::pinhole cam(intr, 4);
    std::unique_ptr<factor_graph::loss_function_base> loss;
    if (loss_kind == ZS_LOSS_HUBER) loss.reset(new factor_graph::loss_huber(loss_delta));
    else if (loss_kind == ZS_LOSS_CAUCHY) loss.reset(new factor_graph::loss_cauchy(loss_delta));
    else if (loss_kind == ZS_LOSS_TUKEY) loss.reset(new factor_graph::loss_tukey(loss_delta));

    factor_graph::factor_graph graph;
    graph.set_precision(precision);
    std::vector<std::unique_ptr<factor_graph::vertex_pose>> pv;
    std::vector<std::unique_ptr<factor_graph::vertex_point_xyz>> lv;
    std::vector<std::unique_ptr<factor_graph::edge_reprojection<camera::pinhole>>> ev;
    for (int k = 0; k < K; ++k) {
        pv.emplace_back(new factor_graph::vertex_pose());
        pv.back()->set_parameters(column(&poses[7 * (std::size_t)k], 7));
        pv.back()->set_fixed(pfix[k] != 0);
        if (!graph.add_vertex(pv.back().get())) return 3;
    }
    for (int l = 0; l < L; ++l) {
        lv.emplace_back(new factor_graph::vertex_point_xyz());
        lv.back()->set_parameters(column(&lms[3 * (std::size_t)l], 3));
        lv.back()->set_marginalised(true);
        lv.back()->set_fixed(lfix[l] != 0);
        if (!graph.add_vertex(lv.back().get())) return 3;
    }
    for (int o = 0; o < M; ++o) {
        ev.emplace_back(new factor_graph::edge_reprojection<camera::pinhole>(cam));
        ev.back()->set_observation(column(&uv[2 * (std::size_t)o], 2));
        ev.back()->add_vertex(pv[op[o]].get());
        ev.back()->add_vertex(lv[ol[o]].get());
        if (loss) ev.back()->set_loss_function(loss.get());
        if (has_info) ev.back()->set_information(matrix::matrix<double, 0, 0>(2, 2, &info[4 * (std::size_t)o]));
        if (!graph.add_edge(ev.back().get())) return 3;
    }
    const double chi_before = graph.get_current_chi();
    const int32_t ret = graph.solve(iterations, use_relative != 0);
    const double chi_after = graph.get_current_chi();

    std::FILE* g = std::fopen(argv[2], "wb");
    if (!g) return 2;
    std::fwrite(&ret, sizeof(ret), 1, g);
    std::fwrite(&chi_before, sizeof(double), 1, g);
    std::fwrite(&chi_after, sizeof(double), 1, g);
    for (int k = 0; k < K; ++k) std::fwrite(pv[k]->get_parameters().data(), sizeof(double), 7, g);
    for (int l = 0; l < L; ++l) std::fwrite(lv[l]->get_parameters().data(), sizeof(double), 3, g);
    std::fclose(g);
    return 0;
}
