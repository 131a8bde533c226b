// Host checks of include/zeroslam_gb300/map_glue.hpp against zeroslam's own
// map, frame, landmark and feature types: the glue compiles against them,
// feature::match has zs_match's layout, gather() lays a map out as the C ABI
// expects, and the entry points refuse a missing handle without touching the
// map. Prints OK on success.
#include "map.hpp"

#include "map_glue.hpp"

#include <cstdio>
#include <cstdlib>

#define CHECK(c)                                                   \
    do {                                                           \
        if (!(c)) {                                                \
            std::fprintf(stderr, "%s:%d: %s\n", __FILE__, __LINE__, #c); \
            std::exit(1);                                          \
        }                                                          \
    } while (0)

int main() {
    static_assert(sizeof(feature::match) == sizeof(zs_match), "feature::match layout");
    static_assert(sizeof(feature::descriptor) == 32, "256-bit descriptors");

    map::map m;
    const double intr[4] = {500.0, 510.0, 320.0, 240.0};
    for (int id = 0; id < 3; ++id) {
        frame::frame f;
        f.id = id;
        f.rotation = matrix::matrix<double, 3, 3>::identity();
        f.translation = matrix::matrix<double, 3, 1>{{0.1 * id, 0.0, 0.0}};
        f.camera = camera::pinhole(intr, 4);
        f.keypoint_pyramid = {{feature::point{10.0f + id, 20.0f, 0.0f, 0.0f}, feature::point{30.0f, 40.0f + id, 0.0f, 0.0f}}};
        m.add_frame(f);
    }
    for (int id = 0; id < 4; ++id) {
        landmark::point p;
        p.id = 100 + id;
        p.location = matrix::matrix<double, 3, 1>{{0.5 * id, 0.25, 4.0}};
        m.add_landmark(p);
    }
    m.observations[100] = {{0, 0}, {1, 1}, {2, 0}};
    m.observations[101] = {{7, 0}, {1, 0}};  // frame 7 is not in the map
    m.observations[102] = {};
    // landmark 103 has no observation list

    const zeroslam_gb300::map_arrays a = zeroslam_gb300::gather(m);
    CHECK(a.frame_id.size() == 3 && a.frame_pose.size() == 36 && a.frame_intrinsics.size() == 12);
    CHECK(a.landmark_id.size() == 4 && a.landmarks.size() == 12 && a.landmark_obs.size() == 5);
    CHECK(a.landmark_obs.back() == 5 && a.obs_frame.size() == 5 && a.obs_keypoint.size() == 10);
    for (size_t f = 0; f < a.frame_id.size(); ++f) {
        const frame::frame& fr = m.frames.at(a.frame_id[f]);
        CHECK(a.frame_pose[12 * f + 0] == 1.0 && a.frame_pose[12 * f + 9] == fr.translation[0]);
        CHECK(a.frame_intrinsics[4 * f + 1] == 510.0);
    }
    for (size_t l = 0; l < a.landmark_id.size(); ++l) {
        const int id = a.landmark_id[l];
        const auto it = m.observations.find(id);
        const size_t n = it == m.observations.end() ? 0 : it->second.size();
        CHECK(static_cast<size_t>(a.landmark_obs[l + 1] - a.landmark_obs[l]) == n);
        CHECK(a.landmarks[3 * l + 2] == 4.0);
        for (size_t k = 0; k < n; ++k) {
            const int64_t o = a.landmark_obs[l] + static_cast<int64_t>(k);
            const auto& ob = it->second[k];
            CHECK(a.obs_frame_id[o] == ob.first);
            if (ob.first == 7) {
                CHECK(a.obs_frame[o] == -1);
            } else {
                CHECK(a.frame_id[a.obs_frame[o]] == ob.first);
                const feature::point& kp = m.frames.at(ob.first).keypoint_pyramid[0][ob.second];
                CHECK(a.obs_keypoint[2 * o] == kp.x && a.obs_keypoint[2 * o + 1] == kp.y);
            }
        }
    }

    // no handle: refused, map untouched
    CHECK(zeroslam_gb300::cull(m, nullptr) == ZS_ERR_INVALID && m.landmarks.size() == 4);
    CHECK(zeroslam_gb300::optimise(m, nullptr, 0, false, 5) == ZS_ERR_INVALID);
    CHECK(m.frames.at(1).translation[0] == 0.1);
    feature::descriptor d[2] = {};
    feature::match out[4];
    size_t found = 7;
    CHECK(zeroslam_gb300::find_matches(static_cast<zs_ba_handle*>(nullptr), d, 2, d, 2, 32.0f, 2, out, 4, &found) ==
          ZS_ERR_INVALID);
    CHECK(found == 0);
    std::printf("OK\n");
    return 0;
}
