// Map-level drop-ins for zeroslam: bodies for map::map::optimise
// (source/map.hpp:65-267), map::map::cull (source/map.hpp:269-323) and the
// feature::find_matches calls of slam::process_frame (source/slam.hpp:116-140)
// that run through the C ABI of include/zeroslam_ba.h.
//
// Include after zeroslam's map.hpp. The functions are templates over the map
// type, so this header names none of zeroslam's types; they read the public
// members map::map uses (frames, landmarks, observations; frame::id,
// rotation, translation, camera, keypoint_pyramid; landmark::point::id,
// location; the id_generator statics) and write back what the reference
// writes back. Frames and landmarks are gathered in the maps' iteration
// order, each landmark's observations in their list order.
//
//   zeroslam_gb300::optimise(map, handle, local_window, fix_landmarks, rounds, use_relative)
//   zeroslam_gb300::cull(map, handle)
//   zeroslam_gb300::find_matches(handle, lhs, lhs_size, rhs, rhs_size, threshold, count, matches, size)
//
// Each returns the library's status (ZS_OK = 0, negative on error) and, on
// error, leaves the map unchanged.
#ifndef ZEROSLAM_GB300_MAP_GLUE_HPP
#define ZEROSLAM_GB300_MAP_GLUE_HPP

#include "../zeroslam_ba.h"

#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <type_traits>
#include <unordered_map>
#include <vector>

namespace zeroslam_gb300 {

// A map as the arrays of zs_map_optimise_input / zs_map_cull_input.
struct map_arrays {
    std::vector<int32_t> frame_id;
    std::vector<double> frame_pose;        // 12 per frame: rotation (row-major), translation
    std::vector<double> frame_intrinsics;  // 4 per frame
    std::vector<int32_t> landmark_id;
    std::vector<double> landmarks;         // 3 per landmark
    std::vector<int64_t> landmark_obs{0};  // ranges into the observation arrays
    std::vector<int32_t> obs_frame;        // frame index, -1 when the frame is not in the map
    std::vector<int32_t> obs_frame_id;
    std::vector<float> obs_keypoint;       // 2 per observation
};

template <typename Map>
map_arrays gather(const Map& m) {
    map_arrays a;
    std::unordered_map<int, int32_t> index;
    for (const auto& [id, f] : m.frames) {
        index[id] = static_cast<int32_t>(a.frame_id.size());
        a.frame_id.push_back(id);
        for (int i = 0; i < 3; ++i)
            for (int k = 0; k < 3; ++k) a.frame_pose.push_back(f.rotation[i][k]);
        for (int i = 0; i < 3; ++i) a.frame_pose.push_back(f.translation[i]);
        double p[4];
        f.camera.get_parameters(p, 4);
        a.frame_intrinsics.insert(a.frame_intrinsics.end(), p, p + 4);
    }
    for (const auto& [id, l] : m.landmarks) {
        a.landmark_id.push_back(id);
        for (int i = 0; i < 3; ++i) a.landmarks.push_back(l.location[i]);
        const auto it = m.observations.find(id);
        if (it != m.observations.end()) {
            for (const auto& ob : it->second) {
                const auto fi = index.find(ob.first);
                a.obs_frame.push_back(fi == index.end() ? -1 : fi->second);
                a.obs_frame_id.push_back(ob.first);
                float x = 0.0f, y = 0.0f;
                if (fi != index.end()) {
                    const auto& kp = m.frames.at(ob.first).keypoint_pyramid[0][static_cast<size_t>(ob.second)];
                    x = kp.x;
                    y = kp.y;
                }
                a.obs_keypoint.push_back(x);
                a.obs_keypoint.push_back(y);
            }
        }
        a.landmark_obs.push_back(static_cast<int64_t>(a.obs_frame.size()));
    }
    return a;
}

// map::map::optimise. The frames' id generator is the map's frame type's.
template <typename Map>
int optimise(Map& m, zs_ba_handle* h, int local_window, bool fix_landmarks, int rounds, bool use_relative = false,
             zs_map_optimise_report* report = nullptr) {
    using frame_type = typename std::decay<decltype(m.frames.begin()->second)>::type;
    map_arrays a = gather(m);
    zs_map_optimise_input in;
    in.num_frames = static_cast<int32_t>(a.frame_id.size());
    in.frame_id = a.frame_id.data();
    in.frame_pose = a.frame_pose.data();
    in.frame_intrinsics = a.frame_intrinsics.data();
    in.num_landmarks = static_cast<int32_t>(a.landmark_id.size());
    in.landmark_id = a.landmark_id.data();
    in.landmarks = a.landmarks.data();
    in.landmark_obs = a.landmark_obs.data();
    in.obs_frame = a.obs_frame.data();
    in.obs_keypoint = a.obs_keypoint.data();
    in.frame_id_generator = frame_type::id_generator;
    zs_map_optimise_report rep{};
    const int st = zs_map_optimise(h, &in, local_window, fix_landmarks ? 1 : 0, rounds, use_relative ? 1 : 0, &rep);
    if (report) *report = rep;
    if (st != ZS_OK || rep.outcome != ZS_MAP_OPTIMISED) return st;
    for (size_t f = 0; f < a.frame_id.size(); ++f) {  // unselected frames come back unchanged
        auto& fr = m.frames.at(a.frame_id[f]);
        for (int i = 0; i < 3; ++i) {
            for (int k = 0; k < 3; ++k) fr.rotation[i][k] = a.frame_pose[12 * f + 3 * i + k];
            fr.translation[i] = a.frame_pose[12 * f + 9 + i];
        }
    }
    for (size_t l = 0; l < a.landmark_id.size(); ++l) {
        auto& lm = m.landmarks.at(a.landmark_id[l]);
        for (int i = 0; i < 3; ++i) lm.location[i] = a.landmarks[3 * l + i];
    }
    std::printf("Optimised: %f to %f error [frames: %d landmarks: %d edges: %d] [%d/%d valid rounds]\n",
                rep.solve.chi2_initial, rep.solve.chi2_final, rep.frames, rep.landmarks, rep.edges,
                rep.solve.accepted, rounds);
    return ZS_OK;
}

// map::map::cull.
template <typename Map>
int cull(Map& m, zs_ba_handle* h, zs_cull_report* report = nullptr) {
    using frame_type = typename std::decay<decltype(m.frames.begin()->second)>::type;
    using landmark_type = typename std::decay<decltype(m.landmarks.begin()->second)>::type;
    map_arrays a = gather(m);
    zs_map_cull_input in;
    in.num_frames = static_cast<int32_t>(a.frame_id.size());
    in.frame_pose = a.frame_pose.data();
    in.frame_intrinsics = a.frame_intrinsics.data();
    in.num_landmarks = static_cast<int32_t>(a.landmark_id.size());
    in.landmark_id = a.landmark_id.data();
    in.landmarks = a.landmarks.data();
    in.landmark_obs = a.landmark_obs.data();
    in.obs_frame = a.obs_frame.data();
    in.obs_frame_id = a.obs_frame_id.data();
    in.obs_keypoint = a.obs_keypoint.data();
    in.landmark_id_generator = landmark_type::id_generator;
    in.frame_id_generator = frame_type::id_generator;
    std::vector<uint8_t> erase(a.landmark_id.size());
    zs_cull_report rep{};
    const int st = zs_map_cull(h, &in, erase.data(), nullptr, &rep);
    if (report) *report = rep;
    if (st != ZS_OK) return st;
    for (size_t l = 0; l < erase.size(); ++l) {
        if (!erase[l]) continue;
        m.observations.erase(a.landmark_id[l]);
        m.landmarks.erase(a.landmark_id[l]);
    }
    std::printf("Culled: %zu points\n", static_cast<size_t>(rep.erased));
    return ZS_OK;
}

// feature::find_matches on descriptors of 32 bytes (feature::descriptor) into
// matches laid out as zs_match (feature::match: size_t, size_t, float).
template <typename Descriptor, typename Match>
int find_matches(zs_ba_handle* h, const Descriptor* lhs, size_t lhs_size, const Descriptor* rhs, size_t rhs_size,
                 float threshold, size_t matches_count, Match* matches, size_t matches_size, size_t* found) {
    static_assert(sizeof(Descriptor) == 32, "256-bit descriptors");
    static_assert(sizeof(Match) == sizeof(zs_match), "a match must have zs_match's layout");
    int64_t n = 0;
    const int st = zs_find_matches(h, reinterpret_cast<const uint8_t*>(lhs), static_cast<int64_t>(lhs_size),
                                   reinterpret_cast<const uint8_t*>(rhs), static_cast<int64_t>(rhs_size), threshold,
                                   static_cast<int64_t>(matches_count), reinterpret_cast<zs_match*>(matches),
                                   static_cast<int64_t>(matches_size), &n, nullptr);
    if (found) *found = static_cast<size_t>(n);
    return st;
}

}  // namespace zeroslam_gb300

#endif
