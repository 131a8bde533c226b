// C-callable driver around zeroslam's own factor-graph solver.
//
// TEST INFRASTRUCTURE ONLY: compiled by oracle/build_ref.py against the
// unmodified reference headers (source/factor_graph.hpp, camera.hpp, lie.hpp,
// matrix*.hpp) into oracle/_ref/. It is used to pin the C restatement
// (ba_oracle.c), to write the golden fixtures under tests/golden/, and as the
// timed CPU baseline. Only the reference's public API is used. zsref_map_cull
// runs map::map::cull (source/map.hpp:269-323) on a map assembled from arrays.
#include "factor_graph.hpp"
#include "camera.hpp"
#include "map.hpp"

#include <chrono>
#include <cstring>
#include <memory>
#include <vector>

namespace {

struct graph_build {
    std::vector<std::unique_ptr<factor_graph::vertex_base>> poses;
    std::vector<std::unique_ptr<factor_graph::vertex_base>> landmarks;
    std::vector<std::unique_ptr<factor_graph::edge_base>> edges;
    std::unique_ptr<factor_graph::loss_function_base> loss;
};

// Builds the graph the way source/map.hpp:129-179 does: one vertex_pose per
// pose, one marginalised vertex_point_xyz per landmark, one
// edge_reprojection<pinhole> per observation sharing one loss object.
void build(factor_graph::factor_graph& fg, graph_build& g, int K, int L, long long M, const double* poses,
           const unsigned char* pose_fixed, const double* lms, const unsigned char* lm_fixed, const int* obs_pose,
           const int* obs_lm, const double* obs_uv, const double* obs_info, const double* intr, int loss_kind,
           double loss_delta) {
    if (loss_kind == 1) g.loss = std::make_unique<factor_graph::loss_huber>(loss_delta);
    if (loss_kind == 2) g.loss = std::make_unique<factor_graph::loss_cauchy>(loss_delta);
    if (loss_kind == 3) g.loss = std::make_unique<factor_graph::loss_tukey>(loss_delta);
    for (int k = 0; k < K; ++k) {
        auto v = std::make_unique<factor_graph::vertex_pose>();
        v->set_parameters(matrix::matrix<double, 0, 0>(7, 1, poses + 7LL * k));
        v->set_fixed(pose_fixed[k] != 0);
        fg.add_vertex(v.get());
        g.poses.push_back(std::move(v));
    }
    for (int l = 0; l < L; ++l) {
        auto v = std::make_unique<factor_graph::vertex_point_xyz>();
        v->set_parameters(matrix::matrix<double, 0, 0>(3, 1, lms + 3LL * l));
        v->set_fixed(lm_fixed[l] != 0);
        v->set_marginalised(true);
        fg.add_vertex(v.get());
        g.landmarks.push_back(std::move(v));
    }
    camera::pinhole cam(intr, 4);
    g.edges.reserve(static_cast<size_t>(M));
    for (long long o = 0; o < M; ++o) {
        auto e = std::make_unique<factor_graph::edge_reprojection<camera::pinhole>>(cam);
        e->set_observation(matrix::matrix<double, 0, 0>(2, 1, obs_uv + 2 * o));
        e->add_vertex(g.poses[obs_pose[o]].get());
        e->add_vertex(g.landmarks[obs_lm[o]].get());
        if (obs_info) e->set_information(matrix::matrix<double, 0, 0>(2, 2, obs_info + 4 * o));
        if (g.loss) e->set_loss_function(g.loss.get());
        fg.add_edge(e.get());
        g.edges.push_back(std::move(e));
    }
}

void read_back(const graph_build& g, double* poses, double* lms) {
    for (size_t k = 0; k < g.poses.size(); ++k)
        for (int i = 0; i < 7; ++i) poses[7 * k + i] = g.poses[k]->get_parameters()[i][0];
    for (size_t l = 0; l < g.landmarks.size(); ++l)
        for (int i = 0; i < 3; ++i) lms[3 * l + i] = g.landmarks[l]->get_parameters()[i][0];
}

}  // namespace

extern "C" {

// Runs factor_graph::solve(iterations, use_relative) and writes the solved
// state back into poses / lms. out[0] = chi2 before, out[1] = chi2 after,
// out[2] = seconds spent building the graph, out[3] = seconds in solve().
// Returns solve()'s accepted-step count.
int zsref_solve(int K, int L, long long M, double* poses, const unsigned char* pose_fixed, double* lms,
                const unsigned char* lm_fixed, const int* obs_pose, const int* obs_lm, const double* obs_uv,
                const double* obs_info, const double* intr, int loss_kind, double loss_delta, int iterations,
                int use_relative, double* out) {
    using clk = std::chrono::steady_clock;
    const auto t0 = clk::now();
    factor_graph::factor_graph fg(false);
    graph_build g;
    build(fg, g, K, L, M, poses, pose_fixed, lms, lm_fixed, obs_pose, obs_lm, obs_uv, obs_info, intr, loss_kind,
          loss_delta);
    const auto t1 = clk::now();
    out[0] = fg.get_current_chi();
    const auto t2 = clk::now();
    const int accepted = fg.solve(iterations, use_relative != 0);
    const auto t3 = clk::now();
    out[1] = fg.get_current_chi();
    out[2] = std::chrono::duration<double>(t1 - t0).count();
    out[3] = std::chrono::duration<double>(t3 - t2).count();
    read_back(g, poses, lms);
    return accepted;
}

double zsref_chi2(int K, int L, long long M, const double* poses, const unsigned char* pose_fixed, const double* lms,
                  const unsigned char* lm_fixed, const int* obs_pose, const int* obs_lm, const double* obs_uv,
                  const double* obs_info, const double* intr, int loss_kind, double loss_delta) {
    factor_graph::factor_graph fg(false);
    graph_build g;
    build(fg, g, K, L, M, poses, pose_fixed, lms, lm_fixed, obs_pose, obs_lm, obs_uv, obs_info, intr, loss_kind,
          loss_delta);
    return fg.get_current_chi();
}

// Residual and analytic Jacobians of one edge_reprojection<pinhole>
// (J_p 2x6 and J_l 2x3, row-major).
void zsref_edge(const double* pose7, const double* X3, const double* uv2, const double* intr, double* r2,
                double* Jp12, double* Jl6) {
    factor_graph::vertex_pose vp;
    vp.set_parameters(matrix::matrix<double, 0, 0>(7, 1, pose7));
    factor_graph::vertex_point_xyz vl;
    vl.set_parameters(matrix::matrix<double, 0, 0>(3, 1, X3));
    vl.set_marginalised(true);
    camera::pinhole cam(intr, 4);
    factor_graph::edge_reprojection<camera::pinhole> e(cam);
    e.set_observation(matrix::matrix<double, 0, 0>(2, 1, uv2));
    e.add_vertex(&vp);
    e.add_vertex(&vl);
    e.compute_residual();
    e.compute_jacobians();
    for (int i = 0; i < 2; ++i) r2[i] = e.get_residual()[i][0];
    for (int i = 0; i < 2; ++i)
        for (int c = 0; c < 6; ++c) Jp12[i * 6 + c] = e.get_jacobians()[0][i][c];
    for (int i = 0; i < 2; ++i)
        for (int c = 0; c < 3; ++c) Jl6[i * 3 + c] = e.get_jacobians()[1][i][c];
}

int zsref_cholesky(const double* A, int n, double* L) { return matrix::decompose_cholesky(A, n, n, L) ? 1 : 0; }

int zsref_cholesky_solve(const double* L, const double* b, int n, double* x) {
    return matrix::solve_cholesky(L, b, n, n, x) ? 1 : 0;
}

int zsref_invert3(const double* A, double* out) {
    matrix::matrix<double, 3, 3> a(A), o;
    const bool ok = matrix::invert(a, o);
    std::memcpy(out, o.data(), 9 * sizeof(double));
    return ok ? 1 : 0;
}

void zsref_pose_plus(double* pose7, const double* d6) {
    factor_graph::vertex_pose vp;
    vp.set_parameters(matrix::matrix<double, 0, 0>(7, 1, pose7));
    vp.plus(matrix::matrix<double, 0, 0>(6, 1, d6));
    for (int i = 0; i < 7; ++i) pose7[i] = vp.get_parameters()[i][0];
}

void zsref_loss(int kind, double delta, double e2, double* rho3) {
    matrix::matrix<double, 3, 1> rho = matrix::matrix<double, 3, 1>::zero();
    if (kind == 1) factor_graph::loss_huber(delta).compute(e2, rho);
    else if (kind == 2) factor_graph::loss_cauchy(delta).compute(e2, rho);
    else if (kind == 3) factor_graph::loss_tukey(delta).compute(e2, rho);
    else factor_graph::loss_trivial().compute(e2, rho);
    for (int i = 0; i < 3; ++i) rho3[i] = rho[i];
}

// Assembles a map::map from arrays (frame f: id frame_id[f], rotation and
// translation frame_pose[12 f..], camera frame_intr[4 f..], one keypoint per
// observation it makes; observations whose obs_frame is -1 name a frame id
// that is not in the map), sets both id generators, runs cull() and reports
// which landmarks it erased (and, in cull_seconds, how long cull() took).
// Landmarks without observations get an empty
// observation list when their index is odd and none when it is even, so both
// of cull()'s branches for them run.
long long zsref_map_cull(int F, const double* frame_pose, const double* frame_intr, const int* frame_id, int L,
                         const int* landmark_id, const double* lms, const long long* lm_obs, const int* obs_frame,
                         const int* obs_frame_id, const float* obs_kp, int lm_gen, int frame_gen,
                         unsigned char* erase, double* cull_seconds) {
    map::map m;
    std::vector<frame::frame> frames(static_cast<size_t>(F));
    for (int f = 0; f < F; ++f) {
        frame::frame& fr = frames[static_cast<size_t>(f)];
        fr.id = frame_id[f];
        for (int i = 0; i < 3; ++i) {
            for (int k = 0; k < 3; ++k) fr.rotation[i][k] = frame_pose[12 * f + 3 * i + k];
            fr.translation[i] = frame_pose[12 * f + 9 + i];
        }
        fr.camera = camera::pinhole(frame_intr + 4 * f, 4);
        fr.keypoint_pyramid.resize(1);
    }
    std::vector<size_t> kp_index(static_cast<size_t>(lm_obs[L]), 0);
    for (long long o = 0; o < lm_obs[L]; ++o) {
        const int f = obs_frame[o];
        if (f < 0) continue;
        std::vector<feature::point>& kps = frames[static_cast<size_t>(f)].keypoint_pyramid[0];
        kp_index[static_cast<size_t>(o)] = kps.size();
        kps.push_back(feature::point{obs_kp[2 * o], obs_kp[2 * o + 1], 0.0f, 0.0f});
    }
    for (int f = 0; f < F; ++f) m.add_frame(frames[static_cast<size_t>(f)]);
    for (int l = 0; l < L; ++l) {
        landmark::point p;
        p.id = landmark_id[l];
        for (int i = 0; i < 3; ++i) p.location[i] = lms[3 * l + i];
        m.add_landmark(p);
        if (lm_obs[l + 1] == lm_obs[l] && (l & 1)) m.observations[p.id];
        for (long long o = lm_obs[l]; o < lm_obs[l + 1]; ++o)
            m.observations[p.id].push_back({obs_frame_id[o], kp_index[static_cast<size_t>(o)]});
    }
    landmark::point::id_generator = lm_gen;
    frame::frame::id_generator = frame_gen;
    const auto t0 = std::chrono::steady_clock::now();
    m.cull();
    const auto t1 = std::chrono::steady_clock::now();
    if (cull_seconds) *cull_seconds = std::chrono::duration<double>(t1 - t0).count();
    long long erased = 0;
    for (int l = 0; l < L; ++l) {
        erase[l] = m.landmarks.count(landmark_id[l]) == 0 ? 1 : 0;
        erased += erase[l];
    }
    return erased;
}

// The rotation and translation map::optimise writes back to a frame from a
// vertex_pose (source/map.hpp:247-251).
void zsref_pose_rt(const double* pose7, double* Rt) {
    const lie::se3<double> v(lie::so3<double>(pose7[6], pose7[3], pose7[4], pose7[5]),
                             matrix::matrix<double, 3, 1>{{pose7[0], pose7[1], pose7[2]}});
    const matrix::matrix<double, 3, 3> R = v.rotation().get_matrix();
    for (int i = 0; i < 3; ++i) {
        for (int k = 0; k < 3; ++k) Rt[3 * i + k] = R[i][k];
        Rt[9 + i] = v.translation()[i];
    }
}

// vertex_pose parameters of a frame, as map::optimise builds them
// (source/map.hpp:131-135).
void zsref_rt_pose(const double* Rt, double* pose7) {
    matrix::matrix<double, 3, 3> R;
    matrix::matrix<double, 3, 1> t;
    for (int i = 0; i < 3; ++i) {
        for (int k = 0; k < 3; ++k) R[i][k] = Rt[3 * i + k];
        t[i] = Rt[9 + i];
    }
    const lie::se3<double> v(R, t);
    pose7[0] = v.translation()[0];
    pose7[1] = v.translation()[1];
    pose7[2] = v.translation()[2];
    pose7[3] = v.rotation().get_quaternion()[1];
    pose7[4] = v.rotation().get_quaternion()[2];
    pose7[5] = v.rotation().get_quaternion()[3];
    pose7[6] = v.rotation().get_quaternion()[0];
}

// Assembles a map::map as zsref_map_cull does (every landmark gets an
// observation list, empty or not, and every observing frame must be in the
// map: map::optimise looks both up with at()), sets the frame id generator,
// runs optimise(local_window, fix_landmarks, rounds, use_relative) and
// copies the frames' rotations and translations and the landmarks back.
void zsref_map_optimise(int F, double* frame_pose, const double* frame_intr, const int* frame_id, int L,
                        const int* landmark_id, double* lms, const long long* lm_obs, const int* obs_frame,
                        const float* obs_kp, int frame_gen, int local_window, int fix_landmarks, int rounds,
                        int use_relative) {
    map::map m;
    std::vector<frame::frame> frames(static_cast<size_t>(F));
    for (int f = 0; f < F; ++f) {
        frame::frame& fr = frames[static_cast<size_t>(f)];
        fr.id = frame_id[f];
        for (int i = 0; i < 3; ++i) {
            for (int k = 0; k < 3; ++k) fr.rotation[i][k] = frame_pose[12 * f + 3 * i + k];
            fr.translation[i] = frame_pose[12 * f + 9 + i];
        }
        fr.camera = camera::pinhole(frame_intr + 4 * f, 4);
        fr.keypoint_pyramid.resize(1);
    }
    std::vector<size_t> kp_index(static_cast<size_t>(lm_obs[L]), 0);
    for (long long o = 0; o < lm_obs[L]; ++o) {
        std::vector<feature::point>& kps = frames[static_cast<size_t>(obs_frame[o])].keypoint_pyramid[0];
        kp_index[static_cast<size_t>(o)] = kps.size();
        kps.push_back(feature::point{obs_kp[2 * o], obs_kp[2 * o + 1], 0.0f, 0.0f});
    }
    for (int f = 0; f < F; ++f) m.add_frame(frames[static_cast<size_t>(f)]);
    for (int l = 0; l < L; ++l) {
        landmark::point p;
        p.id = landmark_id[l];
        for (int i = 0; i < 3; ++i) p.location[i] = lms[3 * l + i];
        m.add_landmark(p);
        std::vector<map::map::observation<int, size_t>>& ob = m.observations[p.id];
        for (long long o = lm_obs[l]; o < lm_obs[l + 1]; ++o)
            ob.push_back({frame_id[obs_frame[o]], kp_index[static_cast<size_t>(o)]});
    }
    frame::frame::id_generator = frame_gen;
    m.optimise(local_window, fix_landmarks != 0, rounds, use_relative != 0);
    for (int f = 0; f < F; ++f) {
        const frame::frame& fr = m.frames.at(frame_id[f]);
        for (int i = 0; i < 3; ++i) {
            for (int k = 0; k < 3; ++k) frame_pose[12 * f + 3 * i + k] = fr.rotation[i][k];
            frame_pose[12 * f + 9 + i] = fr.translation[i];
        }
    }
    for (int l = 0; l < L; ++l)
        for (int i = 0; i < 3; ++i) lms[3 * l + i] = m.landmarks.at(landmark_id[l]).location[i];
}

// feature::find_matches on descriptor arrays (32 bytes each); matches holds
// size entries of (lhs, rhs, score) laid out as feature::match.
long long zsref_find_matches(const unsigned char* lhs, long long n_lhs, const unsigned char* rhs, long long n_rhs,
                             float threshold, long long k, feature::match* matches, long long size) {
    std::vector<feature::descriptor> l(static_cast<size_t>(n_lhs)), r(static_cast<size_t>(n_rhs));
    for (long long i = 0; i < n_lhs; ++i) std::memcpy(l[static_cast<size_t>(i)].data, lhs + 32 * i, 32);
    for (long long j = 0; j < n_rhs; ++j) std::memcpy(r[static_cast<size_t>(j)].data, rhs + 32 * j, 32);
    return static_cast<long long>(feature::find_matches(l.data(), l.size(), r.data(), r.size(), threshold,
                                                        static_cast<size_t>(k), matches, static_cast<size_t>(size)));
}

}  // extern "C"
