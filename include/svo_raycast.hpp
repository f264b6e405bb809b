// svo_raycast.hpp -- drop-in host interface mirroring the reference's frame
// driver and octree builder entry points, implemented over the C ABI of
// svo_gb300.h (link with libsvo_gb300.so).
//
//   reference                                   here
//   set_voxel(x,y,z,uchar4)  octree.h:32        svo::set_voxel(x,y,z,rgba)
//   convert_tree_blocks      octree.h:232       (inside svo::octree_init)
//   octree_init()            raycast.h:13       svo::octree_init()
//   raycast_init()           raycast.h:61       svo::raycast_init()
//   raycast_draw(res_x,res_y) raycast.h:93      svo::raycast_draw(res_x,res_y)
//   raycast_exit()           raycast.h:511      svo::raycast_exit()
//   octree_array_compact / octree_root_normal   svo::octree_array_compact / svo::octree_root_normal
//   MOUSE_X/MOUSE_Y/KEYTAB/fps camera inputs    svo::camera (pos, rot) set by the application
//   PBO mem_screenbuffer_tex                    svo::raycast_framebuffer() (host BGRX8 copy)
//
// Error behaviour follows the reference's error_stop (src/error.h:2-11): a
// failure prints a message and stops the program -- with exit status 1
// instead of the reference's 0 -- unless the application installs its own
// handler with svo::set_error_handler (which may throw instead).
#pragma once
#include <cstdio>
#include <cstdlib>
#include <functional>
#include <string>
#include <algorithm>
#include <vector>

#include "svo_gb300.h"

#ifndef OCTREE_DEPTH
#define OCTREE_DEPTH 11
#endif

namespace svo {

inline std::function<void(const std::string&)>& error_handler() {
    static std::function<void(const std::string&)> h = [](const std::string& msg) {
        std::fprintf(stderr, "svo error: %s\n", msg.c_str());
        std::exit(1);
    };
    return h;
}
inline void set_error_handler(std::function<void(const std::string&)> h) { error_handler() = std::move(h); }

struct State {
    svo_builder* builder = nullptr;
    svo_context* ctx = nullptr;
    svo_target* target = nullptr;
    int res_x = 0, res_y = 0;
    int frame = -1;  // the static frame counter of raycast_draw (raycast.h:104)
    std::vector<uint32_t> framebuffer;
    svo_view view{};  // the camera of the last frame
};
inline State& state() {
    static State s;
    return s;
}

inline std::vector<uint32_t> octree_array_compact;  // octree.h:29
inline uint32_t octree_root_normal = 0;             // octree.h:25

// Camera inputs of raycast_draw (raycast.h:113-133): position in world units
// and the Euler angles the reference derives from the mouse.
struct Camera {
    float pos[3] = {1.0f, 50.0f, 1.0f};  // raycast.h:113
    float rot[3] = {0.0001f, 0.0f, 0.0f};
};
inline Camera camera;

inline void check(svo_status st, const char* what) {
    if (st == SVO_OK) return;
    std::string msg = std::string(what) + " failed (status " + std::to_string((int)st) + ")";
    if (state().ctx) msg += ": " + std::string(svo_last_error(state().ctx));
    error_handler()(msg);
}

inline void set_voxel(uint32_t x, uint32_t y, uint32_t z, uint32_t rgba) {
    State& s = state();
    if (!s.builder) check(svo_builder_create(OCTREE_DEPTH, &s.builder), "svo_builder_create");
    check(svo_builder_set_voxel(s.builder, x, y, z, rgba), "set_voxel");
}

// octree_init (raycast.h:13-46): converts the voxels inserted so far. The
// reference loads data/Imrodh.rle4 here (absent from its tree); with no voxels
// inserted this builds the seeded synthetic terrain instead.
inline void octree_init(uint32_t seed = 2024) {
    State& s = state();
    if (!s.builder) {
        check(svo_builder_create(OCTREE_DEPTH, &s.builder), "svo_builder_create");
        svo_terrain_spec spec{seed, OCTREE_DEPTH, 1, 0};
        check(svo_terrain_build(s.builder, &spec), "svo_terrain_build");
    }
    size_t n = 0;
    check(svo_builder_finish(s.builder, 0, &octree_root_normal, &n), "convert_tree_blocks");
    octree_array_compact.resize(n);
    check(svo_builder_copy_words(s.builder, octree_array_compact.data()), "svo_builder_copy_words");
    svo_builder_destroy(s.builder);
    s.builder = nullptr;
}

inline void raycast_init(int device = 0) {
    State& s = state();
    octree_init();
    check(svo_context_create(device, &s.ctx), "ocl_init");
    check(svo_octree_upload(s.ctx, octree_array_compact.data(), octree_array_compact.size(), octree_root_normal,
                            OCTREE_DEPTH, 1),
          "octree upload");
}

// One frame (raycast.h:93-441): camera from svo::camera, warp pipeline, then
// the BGRX8 image is copied into raycast_framebuffer().
inline void raycast_draw(int res_x, int res_y) {
    State& s = state();
    if (!s.ctx) error_handler()("raycast_draw before raycast_init");
    if (!s.target || s.res_x != res_x || s.res_y != res_y) {
        if (s.target) svo_target_destroy(s.target);
        s.target = nullptr;
        check(svo_target_create(s.ctx, res_x, res_y, &s.target), "target allocation");
        s.res_x = res_x;
        s.res_y = res_y;
        s.framebuffer.assign((size_t)res_x * res_y, 0u);
    }
    ++s.frame;
    float p[3] = {camera.pos[0], camera.pos[1], camera.pos[2]};
    check(svo_wrap_position(p, OCTREE_DEPTH), "position wrap");  // raycast.h:136-145
    for (int i = 0; i < 3; ++i) camera.pos[i] = p[i];
    svo_view v;
    check(svo_view_from_euler(camera.rot[0], camera.rot[1], camera.rot[2], p, res_x, res_y, 1.0f, &v), "camera");
    s.view = v;
    check(svo_warp_frame(s.ctx, s.target, &v, s.frame), "raycast_draw");
    check(svo_read_bgrx(s.target, s.framebuffer.data()), "framebuffer readback");
}

inline const std::vector<uint32_t>& raycast_framebuffer() { return state().framebuffer; }
// The camera raycast_draw derived for the last frame (position wrapped into
// the volume, view matrix from svo::camera.rot).
inline const svo_view& raycast_last_view() { return state().view; }

inline void raycast_exit() {
    State& s = state();
    if (s.target) svo_target_destroy(s.target);
    if (s.ctx) svo_context_destroy(s.ctx);
    s.target = nullptr;
    s.ctx = nullptr;
    s.frame = -1;
}

}  // namespace svo
