// Host-side checks of the drop-in factor graph (include/zeroslam_gb300/factor_graph.hpp):
// single-edge residuals and Jacobians (the values of zeroslam's
// tests/factor_graph.test.cpp:229-276), structure-of-arrays export,
// write-back, unsupported graphs, and solve() failing loudly without a GPU.
// Prints "OK" and returns 0 when every check passes.
#include "factor_graph.hpp"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <memory>
#include <string>
#include <vector>

static int failures = 0;
#define CHECK(x)                                                               \
    do {                                                                       \
        if (!(x)) {                                                            \
            std::fprintf(stderr, "FAILED line %d: %s\n", __LINE__, #x);        \
            ++failures;                                                        \
        }                                                                      \
    } while (0)

static matrix::matrix<double, 0, 0> column(std::vector<double> v) {
    return matrix::matrix<double, 0, 0>(v.size(), 1, v.data());
}

int main(int argc, char** argv) {
    const bool expect_gpu = argc > 1 && std::string(argv[1]) == "--gpu";
    camera::pinhole cam(std::vector<double>{1.0, 1.0, 0.0, 0.0}.data(), 4);
    // 1. residual and Jacobians in front of the camera
    {
        factor_graph::vertex_pose pose;
        pose.set_parameters(column({0, 0, 0, 0, 0, 0, 1}));
        factor_graph::vertex_point_xyz point;
        point.set_parameters(column({0, 0, 1}));
        point.set_marginalised(true);
        factor_graph::edge_reprojection<camera::pinhole> e(cam);
        e.set_observation(column({0.1, -0.2}));
        e.add_vertex(&pose);
        e.add_vertex(&point);
        e.compute_residual();
        e.compute_jacobians();
        CHECK(e.get_residual()[0][0] == 0.1);
        CHECK(e.get_residual()[1][0] == -0.2);
        const double jp[2][6] = {{0, -1, 0, -1, 0, 0}, {1, 0, 0, 0, -1, 0}};
        const double jl[2][3] = {{-1, 0, 0}, {0, -1, 0}};
        for (int r = 0; r < 2; ++r) {
            for (int c = 0; c < 6; ++c) CHECK(e.get_jacobians()[0][r][c] == jp[r][c]);
            for (int c = 0; c < 3; ++c) CHECK(e.get_jacobians()[1][r][c] == jl[r][c]);
        }
        CHECK(std::fabs(e.chi2() - 0.05) < 1e-15);
    }
    // 2. behind the camera: finite, non-zero penalty residual and Jacobians
    {
        factor_graph::vertex_pose pose;
        pose.set_parameters(column({0, 0, 0, 0, 0, 0, 1}));
        factor_graph::vertex_point_xyz point;
        point.set_parameters(column({0.1, 0.2, -10.0}));
        factor_graph::edge_reprojection<camera::pinhole> e(cam);
        e.set_observation(column({0.1, -0.2}));
        e.add_vertex(&pose);
        e.add_vertex(&point);
        e.compute_residual();
        CHECK(e.get_residual()[0][0] == 3.0 && e.get_residual()[1][0] == 3.0);  // -0.3 * (-10)
        e.compute_jacobians();
        CHECK(e.get_jacobians()[1][0][2] < 0.0 && e.get_jacobians()[1][1][2] < 0.0);
        CHECK(e.chi2() > 1.0);
    }
    // 3. numeric Jacobians of the base class against the analytic ones
    {
        struct numeric_reprojection final : factor_graph::edge_base {
            factor_graph::edge_reprojection<camera::pinhole> inner;
            explicit numeric_reprojection(const camera::pinhole& c) : edge_base(2, 2), inner(c) {
            }
            void compute_residual() override {
                inner.set_vertices(this->vertices);
                inner.set_observation(this->observation);
                inner.compute_residual();
                this->residual = inner.get_residual();
            }
        };
        factor_graph::vertex_pose pose;
        pose.set_parameters(column({0.1, -0.05, 0.2, 0.01, -0.02, 0.03, 0.9993}));
        factor_graph::vertex_point_xyz point;
        point.set_parameters(column({0.3, -0.2, 2.5}));
        camera::pinhole c2(std::vector<double>{500.0, 510.0, 320.0, 240.0}.data(), 4);
        factor_graph::edge_reprojection<camera::pinhole> ea(c2);
        numeric_reprojection en(c2);
        for (factor_graph::edge_base* e : {static_cast<factor_graph::edge_base*>(&ea), static_cast<factor_graph::edge_base*>(&en)}) {
            e->set_observation(column({350.0, 200.0}));
            e->add_vertex(&pose);
            e->add_vertex(&point);
            e->compute_residual();
            e->compute_jacobians();
        }
        double worst = 0.0;
        for (int v = 0; v < 2; ++v)
            for (int r = 0; r < 2; ++r)
                for (int c = 0; c < (v ? 3 : 6); ++c)
                    worst = std::fmax(worst, std::fabs(ea.get_jacobians()[v][r][c] - en.get_jacobians()[v][r][c]) /
                                                 (1.0 + std::fabs(ea.get_jacobians()[v][r][c])));
        CHECK(worst < 1e-5);
    }
    // 4. export / import of a small graph, unsupported graphs, solve without a device
    {
        factor_graph::factor_graph graph;
        std::vector<std::unique_ptr<factor_graph::vertex_pose>> poses;
        std::vector<std::unique_ptr<factor_graph::vertex_point_xyz>> points;
        std::vector<std::unique_ptr<factor_graph::edge_reprojection<camera::pinhole>>> edges;
        factor_graph::loss_huber huber(2.0);
        for (int k = 0; k < 3; ++k) {
            poses.emplace_back(new factor_graph::vertex_pose());
            poses.back()->set_parameters(column({0.1 * k, 0, 0, 0, 0, 0, 1}));
            poses.back()->set_fixed(k == 0);
            CHECK(graph.add_vertex(poses.back().get()));
        }
        CHECK(!graph.add_vertex(poses[1].get()));
        for (int l = 0; l < 4; ++l) {
            points.emplace_back(new factor_graph::vertex_point_xyz());
            points.back()->set_parameters(column({0.1 * l - 0.1, 0.05 * l, 2.0 + 0.1 * l}));
            points.back()->set_marginalised(true);
            CHECK(graph.add_vertex(points.back().get()));
        }
        for (int k = 0; k < 3; ++k)
            for (int l = 0; l < 4; ++l) {
                edges.emplace_back(new factor_graph::edge_reprojection<camera::pinhole>(cam));
                edges.back()->set_observation(column({0.01 * k, 0.02 * l}));
                edges.back()->add_vertex(poses[k].get());
                edges.back()->add_vertex(points[l].get());
                edges.back()->set_loss_function(&huber);
                CHECK(graph.add_edge(edges.back().get()));
            }
        CHECK(graph.get_connected_edges(points[2].get()).size() == 3);
        factor_graph::factor_graph::problem_buffers buf;
        CHECK(graph.export_problem(buf) == ZS_OK);
        CHECK(buf.problem.num_poses == 3 && buf.problem.num_landmarks == 4 && buf.problem.num_obs == 12);
        CHECK(buf.problem.obs_info == nullptr);
        CHECK(buf.problem.loss_kind == ZS_LOSS_HUBER && buf.problem.loss_delta == 2.0);
        CHECK(buf.pose_fixed[0] == 1 && buf.pose_fixed[1] == 0);
        CHECK(buf.obs_pose[5] == 1 && buf.obs_landmark[5] == 1);
        CHECK(buf.problem.intrinsics[0] == 1.0 && buf.problem.intrinsics[2] == 0.0);
        buf.poses[7 * 2 + 0] = 0.5;
        buf.landmarks[3 * 3 + 2] = 7.0;
        factor_graph::factor_graph::import_state(buf);
        CHECK(poses[2]->get_parameters()[0][0] == 0.5 && points[3]->get_parameters()[2][0] == 7.0);
        // a custom edge type is not solved on the device
        struct other_edge final : factor_graph::edge_base {
            other_edge() : edge_base(1, 1) {
            }
            void compute_residual() override {
                this->residual[0][0] = 1.0;
            }
        } odd;
        odd.add_vertex(poses[1].get());
        graph.add_edge(&odd);
        factor_graph::factor_graph::problem_buffers buf2;
        CHECK(graph.export_problem(buf2) == ZS_ERR_UNSUPPORTED);
        const double before = poses[1]->get_parameters()[0][0];
        CHECK(graph.solve(5) == ZS_ERR_UNSUPPORTED);
        CHECK(poses[1]->get_parameters()[0][0] == before);
        CHECK(graph.remove_edge(&odd));
        CHECK(!graph.remove_edge(&odd));
        const double chi0 = graph.get_current_chi();
        CHECK(chi0 > 0.0);
        const int r = graph.solve(5);
        if (expect_gpu) {
            CHECK(r >= 1);
            CHECK(graph.get_current_chi() < chi0);
        } else {
            // no device: a negative status, no CPU fallback, vertices untouched
            CHECK(r == ZS_ERR_CUDA);
            CHECK(poses[1]->get_parameters()[0][0] == before);
        }
        CHECK(graph.remove_vertex(points[0].get()));
        CHECK(graph.get_connected_edges(points[0].get()).empty());
    }
    // 5. an empty graph solves to 0 accepted steps
    {
        factor_graph::factor_graph empty;
        CHECK(empty.solve(3) == 0);
    }
    if (failures) return 1;
    std::printf("OK\n");
    return 0;
}
