// Windowed bundle adjustment of a map: zeroslam's map::map::optimise
// (source/map.hpp:65-267) over the map as arrays. Host code: the window
// selection and the problem assembly are linear passes over the observation
// arrays (the reference builds a heap object per vertex and edge in hash
// containers and looks up each vertex's edges with a scan over all edges,
// factor_graph.hpp:473-485 from map.hpp:181-192), then the problem goes
// through the device solver's own C ABI (zs_ba_set_problem, zs_ba_solve,
// zs_ba_get_state) and the results are written back into the arrays.
//
// The frames' rotations become quaternions with lie.hpp:159-180 and come
// back with lie.hpp:188-204, term for term; this file is compiled with
// floating-point contraction off, so both round as the reference does.
#include <chrono>
#include <cmath>
#include <cstring>
#include <vector>

#include "zeroslam_ba.h"

namespace {

// vertex_pose parameters (tx ty tz qx qy qz qw) of a frame, map.hpp:131-135
// with so3(rotation matrix), lie.hpp:159-180.
void rt_to_pose(const double* Rt, double* pose) {
    const double* R = Rt;
    double q[4];
    const double tr = R[0] + R[4] + R[8];
    if (tr > 0) {
        const double s = std::sqrt(tr + 1);
        const double inv = 0.5 / s;
        q[0] = 0.5 * s;
        q[1] = (R[7] - R[5]) * inv;
        q[2] = (R[2] - R[6]) * inv;
        q[3] = (R[3] - R[1]) * inv;
    } else {
        const int i = (R[0] < R[4]) ? (1 + (R[4] < R[8])) : (2 * (R[0] < R[8]));
        const int j = (i + 1) % 3, k = (j + 1) % 3;
        const double s = std::sqrt(R[3 * i + i] - R[3 * j + j] - R[3 * k + k] + 1.0);
        const double inv = 0.5 / s;
        q[0] = (R[3 * j + k] - R[3 * k + j]) * inv;
        q[1 + i] = 0.5 * s;
        q[1 + j] = (R[3 * i + j] + R[3 * j + i]) * inv;
        q[1 + k] = (R[3 * i + k] + R[3 * k + i]) * inv;
    }
    pose[0] = Rt[9];
    pose[1] = Rt[10];
    pose[2] = Rt[11];
    pose[3] = q[1];
    pose[4] = q[2];
    pose[5] = q[3];
    pose[6] = q[0];
}

// The frame written back from a pose, map.hpp:247-251 (so3::get_matrix).
void pose_to_rt(const double* p, double* Rt) {
    const double w = p[6], x = p[3], y = p[4], z = p[5];
    const double tx = 2.0 * x, ty = 2.0 * y, tz = 2.0 * z;
    const double txx = tx * x, txy = tx * y, txz = tx * z, txw = tx * w;
    const double tyy = ty * y, tyz = ty * z, tyw = ty * w;
    const double tzz = tz * z, tzw = tz * w;
    Rt[0] = 1.0 - (tyy + tzz);
    Rt[1] = txy - tzw;
    Rt[2] = txz + tyw;
    Rt[3] = txy + tzw;
    Rt[4] = 1.0 - (txx + tzz);
    Rt[5] = tyz - txw;
    Rt[6] = txz - tyw;
    Rt[7] = tyz + txw;
    Rt[8] = 1.0 - (txx + tyy);
    Rt[9] = p[0];
    Rt[10] = p[1];
    Rt[11] = p[2];
}

}  // namespace

extern "C" void zs_frame_to_pose(const double* frame_pose, double* pose) { rt_to_pose(frame_pose, pose); }
extern "C" void zs_pose_to_frame(const double* pose, double* frame_pose) { pose_to_rt(pose, frame_pose); }

// The window and graph map::optimise builds from a map (map.hpp:65-233):
// validation, window selection, the edges, removal of frames without edges
// and the two early outcomes. Host-only: no device involved.
struct MapPlan {
    std::vector<uint8_t> relevant, fixed;  // [F] selected frames (written back), fixed frames
    std::vector<int32_t> pose_of;          // problem pose -> frame index
    std::vector<int32_t> pose_index;       // frame index -> problem pose or -1
    std::vector<int32_t> lm_of;            // problem landmark -> map landmark index
    std::vector<int32_t> obs_pose;         // per edge: frame index
    std::vector<int32_t> obs_lm;           // per edge: problem landmark
    std::vector<int64_t> edge_obs;         // per edge: index into the map's observation arrays
    std::vector<double> obs_uv;            // per edge: keypoint as double
    zs_map_optimise_report r{};
    bool solve = false;                    // the problem is to be solved
};

static int plan_window(const zs_map_optimise_input* m, int local_window, bool fix_landmarks, MapPlan& pl) {
    zs_map_optimise_report& r = pl.r;
    std::memset(&r, 0, sizeof(r));
    r.outcome = ZS_MAP_NOTHING_TO_OPTIMISE;
    const int F = m->num_frames, L = m->num_landmarks;
    if (F < 0 || L < 0) return ZS_ERR_INVALID;
    if (F == 0) return ZS_OK;  // map.hpp:66-68
    if (!m->frame_id || !m->frame_pose || !m->frame_intrinsics) return ZS_ERR_INVALID;
    if (L > 0 && (!m->landmark_id || !m->landmarks || !m->landmark_obs)) return ZS_ERR_INVALID;
    const int64_t M = L > 0 ? m->landmark_obs[L] : 0;
    if (L > 0 && m->landmark_obs[0] != 0) return ZS_ERR_INVALID;
    for (int l = 0; l < L; ++l)
        if (m->landmark_obs[l + 1] < m->landmark_obs[l]) return ZS_ERR_INVALID;
    if (M > 0 && (!m->obs_frame || !m->obs_keypoint)) return ZS_ERR_INVALID;
    for (int64_t o = 0; o < M; ++o)
        if (m->obs_frame[o] < -1 || m->obs_frame[o] >= F) return ZS_ERR_INVALID;

    // window selection, map.hpp:77-127
    const bool windowed = local_window > 0;
    const int fixed_below = m->frame_id_generator - 1 - local_window + 1;
    auto is_fixed = [&](int id) { return id == 0 || (id == 1 && F > 2) || (windowed && id < fixed_below); };
    std::vector<uint8_t>& relevant = pl.relevant;
    std::vector<uint8_t>& fixed = pl.fixed;
    relevant.assign(F, windowed ? 0 : 1);
    fixed.assign(F, 0);
    std::vector<uint8_t> active_lm(L, windowed ? 0 : 1);
    for (int f = 0; f < F; ++f) fixed[f] = is_fixed(m->frame_id[f]);
    if (windowed) {
        const int horizon = m->frame_id_generator - 1 - 2 * local_window;
        for (int l = 0; l < L; ++l) {
            const int64_t o0 = m->landmark_obs[l], o1 = m->landmark_obs[l + 1];
            bool seen = false;
            for (int64_t o = o0; o < o1 && !seen; ++o) seen = m->obs_frame[o] >= 0 && !fixed[m->obs_frame[o]];
            if (!seen) continue;
            active_lm[l] = 1;
            for (int64_t o = o0; o < o1; ++o) {
                const int f = m->obs_frame[o];
                if (f >= 0 && m->frame_id[f] >= horizon) relevant[f] = 1;
            }
        }
        for (int f = 0; f < F; ++f)
            if (!fixed[f]) relevant[f] = 1;
    }

    // the graph, map.hpp:129-179: frames in array order, landmarks in array
    // order, each landmark's edges in its observation order
    std::vector<int32_t> lm_index(L, -1);
    std::vector<uint8_t> has_edge(F, 0);
    for (int l = 0; l < L; ++l) {
        if (!active_lm[l]) continue;
        for (int64_t o = m->landmark_obs[l]; o < m->landmark_obs[l + 1]; ++o) {
            const int f = m->obs_frame[o];
            if (f < 0 || !relevant[f]) continue;
            if (fixed[f] && fix_landmarks) continue;
            if (lm_index[l] < 0) {
                lm_index[l] = (int32_t)pl.lm_of.size();
                pl.lm_of.push_back(l);
            }
            has_edge[f] = 1;
            pl.obs_pose.push_back(f);
            pl.obs_lm.push_back(lm_index[l]);
            pl.edge_obs.push_back(o);
            pl.obs_uv.push_back((double)m->obs_keypoint[2 * o]);
            pl.obs_uv.push_back((double)m->obs_keypoint[2 * o + 1]);
        }
    }
    // vertices without edges leave the graph, map.hpp:181-192
    pl.pose_index.assign(F, -1);
    bool any_relevant = false;
    for (int f = 0; f < F; ++f) {
        any_relevant |= relevant[f] != 0;
        if (relevant[f] && has_edge[f]) {
            pl.pose_index[f] = (int32_t)pl.pose_of.size();
            pl.pose_of.push_back(f);
            r.frames += !fixed[f];
        }
    }
    r.landmarks = fix_landmarks ? 0 : (int32_t)pl.lm_of.size();
    r.edges = (int32_t)pl.obs_pose.size();
    r.problem_poses = (int32_t)pl.pose_of.size();
    r.problem_landmarks = (int32_t)pl.lm_of.size();
    if (r.frames == 0 && r.landmarks == 0) {  // map.hpp:195-214
        r.outcome = ZS_MAP_ALL_FIXED;
        return ZS_OK;
    }
    if (!any_relevant || pl.lm_of.empty()) return ZS_OK;  // map.hpp:215-233
    pl.solve = true;
    return ZS_OK;
}

extern "C" int zs_map_optimise_plan(const zs_map_optimise_input* m, int32_t local_window, int32_t fix_landmarks,
                                    int32_t* pose_frame, int32_t* landmark_index, int64_t* edge_obs,
                                    uint8_t* frame_written, zs_map_optimise_report* rep) {
    if (!m) return ZS_ERR_INVALID;
    MapPlan pl;
    const int st = plan_window(m, local_window, fix_landmarks != 0, pl);
    if (st != ZS_OK) return st;
    if (pose_frame) std::memcpy(pose_frame, pl.pose_of.data(), sizeof(int32_t) * pl.pose_of.size());
    if (landmark_index) std::memcpy(landmark_index, pl.lm_of.data(), sizeof(int32_t) * pl.lm_of.size());
    if (edge_obs) std::memcpy(edge_obs, pl.edge_obs.data(), sizeof(int64_t) * pl.edge_obs.size());
    if (frame_written)
        for (size_t f = 0; f < pl.relevant.size(); ++f) frame_written[f] = pl.solve && pl.relevant[f] ? 1 : 0;
    if (rep) {
        *rep = pl.r;
        if (pl.solve) rep->outcome = ZS_MAP_OPTIMISED;  // what zs_map_optimise would do
    }
    return ZS_OK;
}

extern "C" int zs_map_optimise(zs_ba_handle* h, zs_map_optimise_input* m, int32_t local_window,
                               int32_t fix_landmarks, int32_t rounds, int32_t use_relative,
                               zs_map_optimise_report* rep) {
    if (!h || !m) return ZS_ERR_INVALID;
    const auto t0 = std::chrono::steady_clock::now();
    MapPlan pl;
    int st = plan_window(m, local_window, fix_landmarks != 0, pl);
    if (st != ZS_OK) return st;
    zs_map_optimise_report& r = pl.r;
    if (!pl.solve) {
        r.ms_select = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        if (rep) *rep = r;
        return ZS_OK;
    }
    const int F = m->num_frames;
    const int K = (int)pl.pose_of.size(), NL = (int)pl.lm_of.size();
    const int64_t NM = (int64_t)pl.obs_pose.size();
    std::vector<double> pose7((size_t)F * 7), poses((size_t)K * 7), lms((size_t)NL * 3);
    std::vector<uint8_t> pose_fixed(K), lm_fixed(NL, fix_landmarks ? 1 : 0);
    for (int f = 0; f < F; ++f)
        if (pl.relevant[f]) rt_to_pose(m->frame_pose + 12 * (int64_t)f, &pose7[(size_t)f * 7]);
    for (int k = 0; k < K; ++k) {
        std::memcpy(&poses[(size_t)k * 7], &pose7[(size_t)pl.pose_of[k] * 7], 7 * sizeof(double));
        pose_fixed[k] = pl.fixed[pl.pose_of[k]];
    }
    for (int i = 0; i < NL; ++i)
        std::memcpy(&lms[(size_t)i * 3], m->landmarks + 3 * (int64_t)pl.lm_of[i], 3 * sizeof(double));
    std::vector<int32_t> obs_pose(NM);
    for (int64_t e = 0; e < NM; ++e) obs_pose[e] = pl.pose_index[pl.obs_pose[e]];

    zs_ba_problem p;
    std::memset(&p, 0, sizeof(p));
    p.num_poses = K;
    p.num_landmarks = NL;
    p.num_obs = NM;
    p.poses = poses.data();
    p.pose_fixed = pose_fixed.data();
    p.landmarks = lms.data();
    p.landmark_fixed = lm_fixed.data();
    p.obs_pose = obs_pose.data();
    p.obs_landmark = pl.obs_lm.data();
    p.obs_uv = pl.obs_uv.data();
    p.obs_info = nullptr;
    for (int i = 0; i < 4; ++i) p.intrinsics[i] = m->frame_intrinsics[i];
    p.loss_kind = ZS_LOSS_HUBER;
    p.loss_delta = std::sqrt(5.991);  // map.hpp:74
    r.ms_select = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();

    st = zs_ba_set_problem(h, &p);
    if (st != ZS_OK) return st;
    st = zs_ba_solve(h, rounds, use_relative, &r.solve);
    if (st < 0) return st;
    st = zs_ba_get_state(h, poses.data(), lms.data());
    if (st != ZS_OK) return st;

    // write back, map.hpp:239-252: every selected frame (those that left the
    // graph keep their converted pose) and every optimised landmark
    for (int f = 0; f < F; ++f) {
        if (!pl.relevant[f]) continue;
        const double* src = pl.pose_index[f] >= 0 ? &poses[(size_t)pl.pose_index[f] * 7] : &pose7[(size_t)f * 7];
        pose_to_rt(src, m->frame_pose + 12 * (int64_t)f);
    }
    for (int i = 0; i < NL; ++i)
        std::memcpy(m->landmarks + 3 * (int64_t)pl.lm_of[i], &lms[(size_t)i * 3], 3 * sizeof(double));
    r.outcome = ZS_MAP_OPTIMISED;
    if (rep) *rep = r;
    return ZS_OK;
}
