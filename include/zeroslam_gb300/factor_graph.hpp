// Drop-in replacement for zeroslam's source/factor_graph.hpp whose solve()
// runs on the GPU through the C ABI of include/zeroslam_ba.h.
//
// Same namespace, class names, members and method semantics as the
// reference's factor graph (source/factor_graph.hpp:42-1049): loss functions,
// vertex_base / vertex_pose / vertex_point_xyz, edge_base /
// edge_reprojection<camera>, and factor_graph with add/remove of vertices and
// edges, solve(iterations, use_relative_convergence) and get_current_chi().
// Put the directory of this file before zeroslam's source directory on the
// include path; matrix.hpp, lie.hpp and camera.hpp still come from zeroslam.
//
// What runs where:
//   * factor_graph::solve packs the graph into the structure-of-arrays
//     problem (poses first, marginalised landmarks after, as the reference
//     orders them, source/factor_graph.hpp:633-645), solves it on the device
//     (zs_ba_solve: the reference's Levenberg-Marquardt loop and Schur
//     complement) and writes the parameters back into the vertices;
//   * single-edge calls (compute_residual, compute_jacobians, chi2,
//     robust_info) and get_current_chi are evaluated here on the host, as
//     in the reference, since they are per-edge API calls, not the solve.
// The device solves graphs of vertex_pose (not marginalised), vertex_point_xyz
// (marginalised) and edge_reprojection<camera::pinhole> with one shared
// intrinsics and loss; other graphs make solve() return
// ZS_ERR_UNSUPPORTED (negative) and leave every vertex unchanged. There is
// no CPU solver behind it: without a usable GPU solve() returns ZS_ERR_CUDA.
//
// Extensions (not in the reference): set_precision(ZS_PRECISION_MIXED) for
// the mixed-precision form, set_device(ordinal), last_status() and
// last_report() after a solve, export_problem() for inspection.
#ifndef ZEROSLAM_GB300_FACTOR_GRAPH_HPP
#define ZEROSLAM_GB300_FACTOR_GRAPH_HPP

#include "camera.hpp"
#include "lie.hpp"
#include "matrix.hpp"

#include "../zeroslam_ba.h"

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <unordered_map>
#include <vector>

namespace factor_graph {

    // Robust loss: rho = (rho(e2), rho'(e2), rho''(e2)) of the squared error.
    class loss_function_base {
    public:
        virtual ~loss_function_base() = default;

    protected:
        loss_function_base() = default;

    public:
        virtual void compute(double err2, matrix::matrix<double, 3, 1>& rho) const = 0;
        // The device's description of this loss (ZS_LOSS_*), or -1 when the
        // device has no equivalent.
        virtual int device_kind() const {
            return -1;
        }
        virtual double device_delta() const {
            return 0.0;
        }
    };

    class loss_trivial final : public loss_function_base {
    public:
        void compute(double e2, matrix::matrix<double, 3, 1>& rho) const override {
            rho[0] = e2;
            rho[1] = 1.0;
            rho[2] = 0.0;
        }
        int device_kind() const override {
            return ZS_LOSS_NONE;
        }
    };

    class loss_huber final : public loss_function_base {
        double delta;

    public:
        explicit loss_huber(double delta_value) : delta(delta_value) {
        }
        void compute(double e2, matrix::matrix<double, 3, 1>& rho) const override {
            const double d2 = this->delta * this->delta;
            if (e2 <= d2) {
                rho[0] = e2;
                rho[1] = 1.0;
                rho[2] = 0.0;
                return;
            }
            const double e = std::sqrt(e2);
            rho[0] = 2.0 * this->delta * e - d2;
            rho[1] = this->delta / e;
            rho[2] = -0.5 * rho[1] / e2;
        }
        int device_kind() const override {
            return ZS_LOSS_HUBER;
        }
        double device_delta() const override {
            return this->delta;
        }
    };

    class loss_cauchy final : public loss_function_base {
        double delta;

    public:
        explicit loss_cauchy(double delta_value) : delta(delta_value) {
        }
        void compute(double e2, matrix::matrix<double, 3, 1>& rho) const override {
            const double d2 = this->delta * this->delta;
            const double inv = 1.0 / d2;
            const double s = inv * e2 + 1.0;
            rho[0] = d2 * std::log(s);
            rho[1] = 1.0 / s;
            rho[2] = -inv * (rho[1] * rho[1]);
        }
        int device_kind() const override {
            return ZS_LOSS_CAUCHY;
        }
        double device_delta() const override {
            return this->delta;
        }
    };

    class loss_tukey final : public loss_function_base {
        double delta;

    public:
        explicit loss_tukey(double delta_value) : delta(delta_value) {
        }
        void compute(double e2, matrix::matrix<double, 3, 1>& rho) const override {
            const double d2 = this->delta * this->delta;
            if (e2 > d2) {
                rho[0] = d2 / 3.0;
                rho[1] = 0.0;
                rho[2] = 0.0;
                return;
            }
            const double u = 1.0 - e2 / d2;
            rho[0] = d2 * (1.0 - u * u * u) / 3.0;
            rho[1] = u * u;
            rho[2] = -2.0 * u / d2;
        }
        int device_kind() const override {
            return ZS_LOSS_TUKEY;
        }
        double device_delta() const override {
            return this->delta;
        }
    };

    // A vertex: parameters as a column vector, a local (tangent) dimension,
    // fixed / marginalised flags and a backup for rollback.
    class vertex_base {
    protected:
        int ordering_id = 0;
        int local_dimension;
        bool fixed = false;
        bool marginalised = false;
        matrix::matrix<double, 0, 0> parameters;
        matrix::matrix<double, 0, 0> parameters_backup;

    public:
        virtual ~vertex_base() = default;
        vertex_base(const vertex_base&) = default;
        vertex_base(vertex_base&&) = default;
        vertex_base& operator=(const vertex_base&) = default;
        vertex_base& operator=(vertex_base&&) = default;

    protected:
        explicit vertex_base(int parameter_dimension) : vertex_base(parameter_dimension, parameter_dimension) {
        }
        vertex_base(int parameter_dimension, int local_dimension_value)
            : local_dimension(local_dimension_value),
              parameters(matrix::matrix<double, 0, 0>::zero(parameter_dimension, 1)) {
        }

    public:
        void set_ordering_id(int id) {
            this->ordering_id = id;
        }
        int get_ordering_id() const {
            return this->ordering_id;
        }
        int get_local_dimensions() const {
            return this->local_dimension;
        }
        void set_fixed(bool value = true) {
            this->fixed = value;
        }
        bool is_fixed() const {
            return this->fixed;
        }
        void set_marginalised(bool value = true) {
            this->marginalised = value;
        }
        bool is_marginalised() const {
            return this->marginalised;
        }
        const matrix::matrix<double, 0, 0>& get_parameters() const {
            return this->parameters;
        }
        void set_parameters(const matrix::matrix<double, 0, 0>& value) {
            this->parameters = value;
        }
        void backup() {
            this->parameters_backup = this->parameters;
        }
        void restore() {
            this->parameters = this->parameters_backup;
        }
        // Additive update (the default manifold).
        virtual void plus(const matrix::matrix<double, 0, 0>& delta) {
            for (size_t i = 0; i < this->parameters.rows(); ++i) this->parameters[i][0] += delta[i][0];
        }
    };

    // A factor: residual, one Jacobian per vertex, information, observation,
    // optional robust loss.
    class edge_base {
    protected:
        int ordering_id = 0;
        std::vector<vertex_base*> vertices;
        matrix::matrix<double, 0, 0> residual;
        std::vector<matrix::matrix<double, 0, 0>> jacobians;
        matrix::matrix<double, 0, 0> information;
        matrix::matrix<double, 0, 0> observation;
        loss_function_base* loss_function = nullptr;

    public:
        virtual ~edge_base() = default;
        edge_base(const edge_base&) = default;
        edge_base(edge_base&&) = default;
        edge_base& operator=(const edge_base&) = default;
        edge_base& operator=(edge_base&&) = default;

    protected:
        edge_base(int residual_dimension, int num_vertices)
            : residual(matrix::matrix<double, 0, 0>::zero(residual_dimension, 1)),
              jacobians(num_vertices),
              information(matrix::matrix<double, 0, 0>::identity(residual_dimension, residual_dimension)) {
            this->vertices.reserve(num_vertices);
        }

    public:
        int get_ordering_id() const {
            return this->ordering_id;
        }
        void set_ordering_id(int id) {
            this->ordering_id = id;
        }
        size_t num_vertices() const {
            return this->vertices.size();
        }
        bool add_vertex(vertex_base* vertex) {
            if (this->vertices.size() >= this->jacobians.size()) {
                std::fprintf(stderr, "Attempting to add too many vertices to an edge.\n");
                return false;
            }
            this->vertices.push_back(vertex);
            return true;
        }
        const std::vector<vertex_base*>& get_vertices() const {
            return this->vertices;
        }
        bool set_vertices(const std::vector<vertex_base*>& value) {
            this->vertices = value;
            return true;
        }
        vertex_base* get_vertex(int i) {
            return this->vertices[i];
        }
        // r^T Omega r
        double chi2() const {
            const size_t n = this->residual.rows();
            double s = 0.0;
            for (size_t i = 0; i < n; ++i) {
                double oi = 0.0;
                for (size_t j = 0; j < n; ++j) oi += this->residual[j][0] * this->information[j][i];
                s += oi * this->residual[i][0];
            }
            return s;
        }
        double robust_chi2() const {
            if (!this->loss_function) return this->chi2();
            matrix::matrix<double, 3, 1> rho = matrix::matrix<double, 3, 1>::zero();
            this->loss_function->compute(this->chi2(), rho);
            return rho[0];
        }
        const matrix::matrix<double, 0, 0>& get_residual() const {
            return this->residual;
        }
        const std::vector<matrix::matrix<double, 0, 0>>& get_jacobians() const {
            return this->jacobians;
        }
        const matrix::matrix<double, 0, 0>& get_information() const {
            return this->information;
        }
        void set_information(const matrix::matrix<double, 0, 0>& value) {
            this->information = value;
        }
        loss_function_base* get_loss_function() {
            return this->loss_function;
        }
        void set_loss_function(loss_function_base* value) {
            this->loss_function = value;
        }
        // Robust weight: rho' Omega, plus 2 rho'' (Omega r)(Omega r)^T when
        // rho' + 2 rho'' e2 > 0.
        void robust_info(double& rho_delta, matrix::matrix<double, 0, 0>& robust_information) const {
            robust_information = this->information;
            rho_delta = 1.0;
            if (!this->loss_function) return;
            const double e2 = this->chi2();
            matrix::matrix<double, 3, 1> rho = matrix::matrix<double, 3, 1>::zero();
            this->loss_function->compute(e2, rho);
            rho_delta = rho[1];
            const size_t n = this->residual.rows();
            std::vector<double> w(n, 0.0);
            for (size_t i = 0; i < n; ++i)
                for (size_t j = 0; j < n; ++j) w[i] += this->information[i][j] * this->residual[j][0];
            const bool second = (rho[1] + 2.0 * rho[2] * e2) > 0.0;
            for (size_t i = 0; i < n; ++i)
                for (size_t j = 0; j < n; ++j)
                    robust_information[i][j] =
                        rho[1] * this->information[i][j] + (second ? 2.0 * rho[2] * w[i] * w[j] : 0.0);
        }
        const matrix::matrix<double, 0, 0>& get_observation() const {
            return this->observation;
        }
        void set_observation(const matrix::matrix<double, 0, 0>& value) {
            this->observation = value;
        }

    public:
        virtual void compute_residual() = 0;
        // Central differences with step 1e-5 through each vertex's plus().
        virtual void compute_jacobians() {
            const double h = 1e-5;
            const matrix::matrix<double, 0, 0> r0 = this->residual;
            const size_t m = r0.rows();
            for (size_t v = 0; v < this->vertices.size(); ++v) {
                vertex_base* vx = this->vertices[v];
                const int dim = vx->get_local_dimensions();
                this->jacobians[v] = matrix::matrix<double, 0, 0>::zero(m, dim);
                if (vx->is_fixed()) continue;
                for (int d = 0; d < dim; ++d) {
                    const matrix::matrix<double, 0, 0> keep = vx->get_parameters();
                    matrix::matrix<double, 0, 0> step = matrix::matrix<double, 0, 0>::zero(dim, 1);
                    step[d][0] = h;
                    vx->plus(step);
                    this->compute_residual();
                    const matrix::matrix<double, 0, 0> up = this->residual;
                    vx->set_parameters(keep);
                    step[d][0] = -h;
                    vx->plus(step);
                    this->compute_residual();
                    vx->set_parameters(keep);
                    for (size_t r = 0; r < m; ++r)
                        this->jacobians[v][r][d] = (up[r][0] - this->residual[r][0]) * (1.0 / (2.0 * h));
                }
            }
            this->residual = r0;
        }
    };

    // SE(3) pose (tx ty tz qx qy qz qw), world -> camera, left update exp(d) T.
    class vertex_pose final : public vertex_base {
    public:
        vertex_pose() : vertex_base(7, 6) {
        }
        void plus(const matrix::matrix<double, 0, 0>& delta) override {
            const matrix::matrix<double, 0, 0>& p = this->parameters;
            const lie::se3<double> current(lie::so3<double>(p[6][0], p[3][0], p[4][0], p[5][0]),
                                           matrix::matrix<double, 3, 1>{{p[0][0], p[1][0], p[2][0]}});
            const matrix::matrix<double, 6, 1> d{{delta[0][0], delta[1][0], delta[2][0], delta[3][0], delta[4][0], delta[5][0]}};
            const lie::se3<double> next = lie::se3<double>::exp(d) * current;
            const matrix::matrix<double, 4, 1> q = next.rotation().get_quaternion();  // (w, x, y, z)
            for (int i = 0; i < 3; ++i) this->parameters[i][0] = next.translation()[i];
            this->parameters[3][0] = q[1];
            this->parameters[4][0] = q[2];
            this->parameters[5][0] = q[3];
            this->parameters[6][0] = q[0];
        }
    };

    class vertex_point_xyz final : public vertex_base {
    public:
        vertex_point_xyz() : vertex_base(3) {
        }
    };

    // Reprojection of a landmark (vertex 1) into a camera (vertex 0):
    // r = observation - project(T X); behind the camera (projection fails)
    // r = (-0.3 Z, -0.3 Z) with Z the camera-frame depth.
    template <typename camera_type>
    class edge_reprojection final : public edge_base {
        camera_type camera;
        static constexpr double penalty = 0.3;

        matrix::matrix<double, 3, 1> camera_point(lie::se3<double>* pose_out = nullptr) {
            const matrix::matrix<double, 0, 0>& p = this->get_vertex(0)->get_parameters();
            const matrix::matrix<double, 0, 0>& x = this->get_vertex(1)->get_parameters();
            const lie::se3<double> pose(lie::so3<double>(p[6][0], p[3][0], p[4][0], p[5][0]),
                                        matrix::matrix<double, 3, 1>{{p[0][0], p[1][0], p[2][0]}});
            if (pose_out) *pose_out = pose;
            return pose * matrix::matrix<double, 3, 1>{{x[0][0], x[1][0], x[2][0]}};
        }

    public:
        explicit edge_reprojection(const camera_type& camera_model) : edge_base(2, 2), camera(camera_model) {
        }
        const camera_type& get_camera() const {
            return this->camera;
        }

        void compute_residual() override {
            const matrix::matrix<double, 3, 1> pc = this->camera_point();
            double uv[2] = {0.0, 0.0};
            if (!this->camera.project(pc.data(), uv)) {
                this->residual[0][0] = -penalty * pc[2];
                this->residual[1][0] = -penalty * pc[2];
                return;
            }
            this->residual[0][0] = this->get_observation()[0][0] - uv[0];
            this->residual[1][0] = this->get_observation()[1][0] - uv[1];
        }

        // J_pose = -Jc [-[P]x | I] (omega first), J_point = -Jc R, with Jc the
        // projection's 2 x 3 Jacobian, or (0, 0, 0.3) rows behind the camera.
        void compute_jacobians() override {
            lie::se3<double> pose;
            const matrix::matrix<double, 3, 1> pc = this->camera_point(&pose);
            double uv[2];
            double jc[6];
            if (!this->camera.project(pc.data(), uv, jc)) {
                jc[0] = 0.0; jc[1] = 0.0; jc[2] = penalty;
                jc[3] = 0.0; jc[4] = 0.0; jc[5] = penalty;
            }
            const double X = pc[0], Y = pc[1], Z = pc[2];
            // rows of [-[P]x | I]
            const double a[3][6] = {{0.0, Z, -Y, 1.0, 0.0, 0.0}, {-Z, 0.0, X, 0.0, 1.0, 0.0}, {Y, -X, 0.0, 0.0, 0.0, 1.0}};
            const matrix::matrix<double, 3, 3> R = pose.rotation().get_matrix();
            this->jacobians[0] = matrix::matrix<double, 0, 0>::zero(2, 6);
            this->jacobians[1] = matrix::matrix<double, 0, 0>::zero(2, 3);
            for (int r = 0; r < 2; ++r) {
                for (int c = 0; c < 6; ++c)
                    this->jacobians[0][r][c] = -(jc[3 * r] * a[0][c] + jc[3 * r + 1] * a[1][c] + jc[3 * r + 2] * a[2][c]);
                for (int c = 0; c < 3; ++c)
                    this->jacobians[1][r][c] = -(jc[3 * r] * R[0][c] + jc[3 * r + 1] * R[1][c] + jc[3 * r + 2] * R[2][c]);
            }
        }
    };

    // The graph and its solver (source/factor_graph.hpp:341-847): the
    // Levenberg-Marquardt solve runs on the GPU.
    class factor_graph final {
        bool verbose;
        double chi_squared = 0.0;
        std::vector<vertex_base*> vertices_general;
        std::vector<vertex_base*> vertices_marginalised;
        std::vector<edge_base*> edges;
        std::unordered_multimap<vertex_base*, edge_base*> vertex_to_edge;
        // device
        zs_ba_options options{};
        zs_ba_handle* handle = nullptr;
        int status = ZS_OK;
        zs_ba_report report{};

    public:
        explicit factor_graph(bool verbose_in = false) : verbose(verbose_in) {
            zs_ba_default_options(&this->options);
            this->options.verbose = verbose_in ? 1 : 0;
        }
        ~factor_graph() {
            if (this->handle) zs_ba_destroy(this->handle);
        }
        factor_graph(const factor_graph&) = delete;
        factor_graph& operator=(const factor_graph&) = delete;

        // ---- extensions
        void set_precision(int precision) {
            this->options.precision = precision;
            this->reset_handle();
        }
        void set_device(int device) {
            this->options.device = device;
            this->reset_handle();
        }
        int last_status() const {
            return this->status;
        }
        const zs_ba_report& last_report() const {
            return this->report;
        }

        // ---- the reference's interface
        bool add_vertex(vertex_base* vertex) {
            if (this->contains(this->vertices_general, vertex) || this->contains(this->vertices_marginalised, vertex))
                return false;
            (vertex->is_marginalised() ? this->vertices_marginalised : this->vertices_general).push_back(vertex);
            return true;
        }

        bool remove_vertex(vertex_base* vertex) {
            std::vector<vertex_base*>& list = vertex->is_marginalised() ? this->vertices_marginalised : this->vertices_general;
            bool found = false;
            for (size_t i = 0; i < list.size(); ++i) {
                if (list[i] == vertex) {
                    list.erase(list.begin() + static_cast<long>(i));
                    found = true;
                    break;
                }
            }
            if (!found) return false;
            for (edge_base* e : this->get_connected_edges(vertex)) this->remove_edge(e);
            return true;
        }

        bool add_edge(edge_base* edge) {
            for (edge_base* e : this->edges)
                if (e == edge) return false;
            this->edges.push_back(edge);
            for (vertex_base* v : edge->get_vertices()) this->vertex_to_edge.emplace(v, edge);
            return true;
        }

        bool remove_edge(edge_base* edge) {
            bool found = false;
            for (size_t i = 0; i < this->edges.size(); ++i) {
                if (this->edges[i] == edge) {
                    this->edges.erase(this->edges.begin() + static_cast<long>(i));
                    found = true;
                    break;
                }
            }
            if (!found) return false;
            for (vertex_base* v : edge->get_vertices()) {
                auto range = this->vertex_to_edge.equal_range(v);
                for (auto it = range.first; it != range.second; ++it) {
                    if (it->second == edge) {
                        this->vertex_to_edge.erase(it);
                        break;
                    }
                }
            }
            return true;
        }

        std::vector<edge_base*> get_connected_edges(vertex_base* vertex) const {
            std::vector<edge_base*> out;
            auto range = this->vertex_to_edge.equal_range(vertex);
            for (auto it = range.first; it != range.second; ++it) out.push_back(it->second);
            return out;
        }

        // Levenberg-Marquardt on the device. Returns the accepted steps (the
        // reference's return value), 0 without edges or vertices, or a
        // negative ZS_ERR_* status (no vertex changed).
        int solve(int iterations = 10, bool use_relative_convergence = false) {
            this->status = ZS_OK;
            std::memset(&this->report, 0, sizeof(this->report));
            if (this->edges.empty() || (this->vertices_general.empty() && this->vertices_marginalised.empty())) {
                if (this->verbose) std::fprintf(stderr, "Cannot solve problem without edges or vertices\n");
                return 0;
            }
            problem_buffers buf;
            int st = this->export_problem(buf);
            if (st == ZS_OK && !this->handle) st = zs_ba_create(&this->handle, &this->options);
            if (st == ZS_OK) st = zs_ba_set_problem(this->handle, &buf.problem);
            int accepted = 0;
            if (st == ZS_OK) {
                accepted = zs_ba_solve(this->handle, iterations, use_relative_convergence ? 1 : 0, &this->report);
                if (accepted < 0) st = accepted;
            }
            if (st == ZS_OK) st = zs_ba_get_state(this->handle, buf.poses.data(), buf.landmarks.data());
            if (st != ZS_OK) {
                this->status = st;
                if (this->verbose) std::fprintf(stderr, "GPU solve failed: %s %s\n", zs_ba_status_string(st), zs_last_error());
                return st;
            }
            this->import_state(buf);
            this->chi_squared = this->report.chi2_final;
            return accepted;
        }

        // Sum of robust costs over the edges (recomputing residuals first).
        double get_current_chi(bool recompute_residuals = true) {
            double s = 0.0;
            for (edge_base* e : this->edges) {
                if (recompute_residuals) e->compute_residual();
                s += e->robust_chi2();
            }
            this->chi_squared = s;
            return s;
        }

        // ---- the structure-of-arrays problem of the graph
        struct problem_buffers {
            std::vector<double> poses, landmarks, uv, info;
            std::vector<uint8_t> pose_fixed, landmark_fixed;
            std::vector<int32_t> obs_pose, obs_landmark;
            std::vector<vertex_base*> pose_vertices, landmark_vertices;
            zs_ba_problem problem{};
        };

        // Fills buf for the device; ZS_ERR_UNSUPPORTED for graphs the device
        // does not solve.
        int export_problem(problem_buffers& buf) const {
            std::unordered_map<const vertex_base*, int32_t> pose_index, landmark_index;
            for (vertex_base* v : this->vertices_general) {
                if (!dynamic_cast<vertex_pose*>(v)) return this->unsupported("a non-marginalised vertex that is not vertex_pose");
                pose_index.emplace(v, static_cast<int32_t>(buf.pose_vertices.size()));
                buf.pose_vertices.push_back(v);
            }
            for (vertex_base* v : this->vertices_marginalised) {
                if (!dynamic_cast<vertex_point_xyz*>(v)) return this->unsupported("a marginalised vertex that is not vertex_point_xyz");
                landmark_index.emplace(v, static_cast<int32_t>(buf.landmark_vertices.size()));
                buf.landmark_vertices.push_back(v);
            }
            const size_t K = buf.pose_vertices.size(), L = buf.landmark_vertices.size(), M = this->edges.size();
            buf.poses.resize(7 * K);
            buf.pose_fixed.resize(K);
            for (size_t k = 0; k < K; ++k) {
                const matrix::matrix<double, 0, 0>& p = buf.pose_vertices[k]->get_parameters();
                for (int i = 0; i < 7; ++i) buf.poses[7 * k + i] = p[i][0];
                buf.pose_fixed[k] = buf.pose_vertices[k]->is_fixed() ? 1 : 0;
            }
            buf.landmarks.resize(3 * L);
            buf.landmark_fixed.resize(L);
            for (size_t l = 0; l < L; ++l) {
                const matrix::matrix<double, 0, 0>& x = buf.landmark_vertices[l]->get_parameters();
                for (int i = 0; i < 3; ++i) buf.landmarks[3 * l + i] = x[i][0];
                buf.landmark_fixed[l] = buf.landmark_vertices[l]->is_fixed() ? 1 : 0;
            }
            buf.obs_pose.resize(M);
            buf.obs_landmark.resize(M);
            buf.uv.resize(2 * M);
            buf.info.resize(4 * M);
            bool all_identity = true;
            double intr[4] = {0.0, 0.0, 0.0, 0.0};
            int loss_kind = ZS_LOSS_NONE;
            double loss_delta = 0.0;
            for (size_t o = 0; o < M; ++o) {
                edge_base* e = this->edges[o];
                const auto* re = dynamic_cast<const edge_reprojection<camera::pinhole>*>(e);
                if (!re) return this->unsupported("an edge that is not edge_reprojection<camera::pinhole>");
                if (e->num_vertices() != 2) return this->unsupported("a reprojection edge without its two vertices");
                const auto pi = pose_index.find(e->get_vertices()[0]);
                const auto li = landmark_index.find(e->get_vertices()[1]);
                if (pi == pose_index.end() || li == landmark_index.end())
                    return this->unsupported("an edge whose vertices are not (pose, marginalised point) of this graph");
                buf.obs_pose[o] = pi->second;
                buf.obs_landmark[o] = li->second;
                buf.uv[2 * o] = e->get_observation()[0][0];
                buf.uv[2 * o + 1] = e->get_observation()[1][0];
                const matrix::matrix<double, 0, 0>& om = e->get_information();
                for (int i = 0; i < 4; ++i) buf.info[4 * o + i] = om[i / 2][i % 2];
                all_identity = all_identity && om[0][0] == 1.0 && om[0][1] == 0.0 && om[1][0] == 0.0 && om[1][1] == 1.0;
                double c[4];
                re->get_camera().get_parameters(c, 4);
                loss_function_base* lf = e->get_loss_function();
                const int kind = lf ? lf->device_kind() : ZS_LOSS_NONE;
                const double delta = lf ? lf->device_delta() : 0.0;
                if (kind < 0) return this->unsupported("a loss function without a device equivalent");
                if (o == 0) {
                    for (int i = 0; i < 4; ++i) intr[i] = c[i];
                    loss_kind = kind;
                    loss_delta = delta;
                } else if (c[0] != intr[0] || c[1] != intr[1] || c[2] != intr[2] || c[3] != intr[3] ||
                           kind != loss_kind || delta != loss_delta) {
                    return this->unsupported("edges with different intrinsics or losses");
                }
            }
            zs_ba_problem& p = buf.problem;
            p.num_poses = static_cast<int32_t>(K);
            p.num_landmarks = static_cast<int32_t>(L);
            p.num_obs = static_cast<int64_t>(M);
            p.poses = buf.poses.data();
            p.pose_fixed = buf.pose_fixed.data();
            p.landmarks = buf.landmarks.data();
            p.landmark_fixed = buf.landmark_fixed.data();
            p.obs_pose = buf.obs_pose.data();
            p.obs_landmark = buf.obs_landmark.data();
            p.obs_uv = buf.uv.data();
            p.obs_info = all_identity ? nullptr : buf.info.data();
            for (int i = 0; i < 4; ++i) p.intrinsics[i] = intr[i];
            p.loss_kind = loss_kind;
            p.loss_delta = loss_delta;
            return ZS_OK;
        }

        // Writes the solved parameters (buf.poses / buf.landmarks) back.
        static void import_state(const problem_buffers& buf) {
            for (size_t k = 0; k < buf.pose_vertices.size(); ++k) {
                matrix::matrix<double, 0, 0> p = buf.pose_vertices[k]->get_parameters();
                for (int i = 0; i < 7; ++i) p[i][0] = buf.poses[7 * k + i];
                buf.pose_vertices[k]->set_parameters(p);
            }
            for (size_t l = 0; l < buf.landmark_vertices.size(); ++l) {
                matrix::matrix<double, 0, 0> x = buf.landmark_vertices[l]->get_parameters();
                for (int i = 0; i < 3; ++i) x[i][0] = buf.landmarks[3 * l + i];
                buf.landmark_vertices[l]->set_parameters(x);
            }
        }

    private:
        static bool contains(const std::vector<vertex_base*>& list, const vertex_base* v) {
            for (const vertex_base* u : list)
                if (u == v) return true;
            return false;
        }
        int unsupported(const char* what) const {
            if (this->verbose) std::fprintf(stderr, "GPU factor graph: unsupported graph (%s)\n", what);
            return ZS_ERR_UNSUPPORTED;
        }
        void reset_handle() {
            if (this->handle) zs_ba_destroy(this->handle);
            this->handle = nullptr;
        }
    };
}  // namespace factor_graph

#endif  // ZEROSLAM_GB300_FACTOR_GRAPH_HPP
