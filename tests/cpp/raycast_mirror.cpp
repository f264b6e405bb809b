// Drives the reference-named host interface (include/svo_raycast.hpp) the way
// the reference's main loop does (main.cpp:201,209-272): raycast_init, a
// number of raycast_draw calls with a moving camera, raycast_exit. Prints the
// frame count and a checksum of the last BGRX8 image; with a second argument,
// writes every frame's camera (position float4, view matrix float16) and BGRX8
// image to that file, so a test can replay the same cameras on the oracle.
#define OCTREE_DEPTH 8
#include "svo_raycast.hpp"

int main(int argc, char** argv) {
    int frames = argc > 1 ? std::atoi(argv[1]) : 8;
    std::FILE* dump = argc > 2 ? std::fopen(argv[2], "wb") : nullptr;
    if (argc > 2 && !dump) return 2;
    svo::raycast_init();
    const float extent = float(1 << (OCTREE_DEPTH + 1)) / 16.0f;
    svo::camera.pos[0] = 0.2f * extent;
    svo::camera.pos[1] = 0.8f * extent;
    svo::camera.pos[2] = 0.1f * extent;
    svo::camera.rot[0] = 0.45f;
    uint64_t sum = 0;
    for (int f = 0; f < frames; ++f) {
        svo::camera.rot[1] = 0.6f + 0.01f * f;  // the mouse's yaw (raycast.h:116)
        svo::raycast_draw(256, 160);
        if (dump) {
            const svo_view& v = svo::raycast_last_view();
            const std::vector<uint32_t>& fb = svo::raycast_framebuffer();
            if (std::fwrite(v.pos, sizeof(float), 4, dump) != 4 || std::fwrite(v.m, sizeof(float), 16, dump) != 16 ||
                std::fwrite(fb.data(), sizeof(uint32_t), fb.size(), dump) != fb.size())
                return 3;
        }
    }
    for (uint32_t p : svo::raycast_framebuffer()) sum = sum * 1315423911u + p;
    std::printf("frames=%d checksum=%016llx nonblack=%zu\n", frames, (unsigned long long)sum,
                (size_t)std::count_if(svo::raycast_framebuffer().begin(), svo::raycast_framebuffer().end(),
                                      [](uint32_t p) { return (p & 0xffffff) != 0; }));
    svo::raycast_exit();
    if (dump) std::fclose(dump);
    return 0;
}
