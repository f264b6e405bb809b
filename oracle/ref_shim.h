// OpenCL-C builtin shim for compiling the reference's own device code
// (kernel/kernel.cl) and octree builder (src/octree/octree.h) as host C++.
//
// TEST INFRASTRUCTURE ONLY. This header is the prefix of the translation unit
// that oracle/build_ref.sh streams together from the read-only reference tree;
// the result (oracle/_ref/libsvo_ref.so) is the checker that pins the oracle
// restatement and generates the golden fixtures. Nothing in the product links it.
//
// Semantics chosen here (they define what "the reference" computes on a CPU):
//   * strict IEEE-754 binary32 arithmetic: the recipe compiles with
//     -ffp-contract=off and without -ffast-math (kernel.cl was built with
//     -cl-fast-relaxed-math, src/ocl.h:47, which is not reproducible);
//   * dot(a,b) = (a.x*b.x + a.y*b.y) + a.z*b.z, left to right, no FMA;
//   * length(v) = sqrtf(dot(v,v));
//   * convert_int* truncates toward zero (OpenCL's default _rtz for float->int);
//   * sign(x) = 1, -1 or x itself for +-0 (OpenCL 1.1 section 6.11.2);
//   * atom_min is the plain sequential read-min-write (the emulator runs
//     work-items one after another in global row-major order);
//   * __local arrays are per-host-thread statics, zero at first use.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

// src/core.h:20-30 defines uint/ushort/uchar as macros, which breaks the
// functional cast uint(...) at src/octree/octree.h:147; typedef them and
// define each to itself so core.h's #ifndef guards skip its own macros.
typedef unsigned int uint;
typedef unsigned short ushort;
typedef unsigned char uchar;
#define uint uint
#define ushort ushort
#define uchar uchar

#include "Rle4.h"  // -> core.h: uchar4, loop macros (src/core.h:3-8,37-56)
#undef min
#undef max

#define __kernel
#define __global
#define __local static thread_local

struct float3 {
    float x, y, z;
    float3 xyz_() const { return *this; }
};
struct float4 {
    float x, y, z, w;
    float3 xyz_() const { return float3{x, y, z}; }
};
struct int2 { int x, y; };
struct int3 { int x, y, z; };
#define xyz xyz_()

inline float3 operator+(float3 a, float3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline float3 operator-(float3 a, float3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline float3 operator*(float3 a, float3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
inline float3 operator*(float3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
inline float3 operator/(float3 a, float s) { return {a.x / s, a.y / s, a.z / s}; }
inline float3& operator+=(float3& a, float3 b) { a = a + b; return a; }

inline int3 operator+(int3 a, int s) { return {a.x + s, a.y + s, a.z + s}; }
inline int3 operator>>(int3 a, int s) { return {a.x >> s, a.y >> s, a.z >> s}; }
inline int3 operator<<(int3 a, int s) { return {a.x << s, a.y << s, a.z << s}; }
inline int3 operator&(int3 a, int s) { return {a.x & s, a.y & s, a.z & s}; }

inline int3 convert_int3(float3 a) { return {(int)a.x, (int)a.y, (int)a.z}; }
inline float3 convert_float3(int3 a) { return {(float)a.x, (float)a.y, (float)a.z}; }
inline float convert_float(double v) { return (float)v; }
inline float convert_float(float v) { return v; }
inline float convert_float(int v) { return (float)v; }
inline float convert_float(uint v) { return (float)v; }
inline int convert_int(float v) { return (int)v; }

inline float dot(float3 a, float3 b) {
    float s = a.x * b.x;
    s = s + a.y * b.y;
    s = s + a.z * b.z;
    return s;
}
inline float length(float3 a) { return std::sqrt(dot(a, a)); }
inline float sign(float x) { return x > 0.0f ? 1.0f : (x < 0.0f ? -1.0f : x); }
inline int min(int a, int b) { return a < b ? a : b; }
inline int max(int a, int b) { return a > b ? a : b; }
using std::fabs;
using std::log2;
using std::pow;
using std::abs;

inline uint atom_min(uint* p, uint v) {
    uint old = *p;
    if (v < old) *p = v;
    return old;
}

#define CLK_GLOBAL_MEM_FENCE 1
#define CLK_LOCAL_MEM_FENCE 2
inline void barrier(int) {}

// NDRange emulation state (one work-item at a time per host thread).
struct RefWorkItem {
    static inline thread_local int gid[2];
    static inline thread_local int lid[2];
    static inline thread_local int lsz[2];
};
inline size_t get_global_id(int d) { return (size_t)RefWorkItem::gid[d]; }
inline size_t get_local_id(int d) { return (size_t)RefWorkItem::lid[d]; }
inline size_t get_local_size(int d) { return (size_t)RefWorkItem::lsz[d]; }

// Runs f() once per work-item of a 2-D NDRange whose global size is rounded up
// to the local size exactly as ocl_begin does (src/ocl.h:188-198,229-237).
// Work-items run in global row-major order (x fastest), a legal serialisation.
template <class F>
inline void ref_ndrange(int gx, int gy, int lx, int ly, F&& f) {
    auto round_up = [](int g, int l) { int r = g % l; return r == 0 ? g : g + l - r; };
    int GX = round_up(gx, lx), GY = round_up(gy, ly);
    RefWorkItem::lsz[0] = lx;
    RefWorkItem::lsz[1] = ly;
    for (int y = 0; y < GY; ++y)
        for (int x = 0; x < GX; ++x) {
            RefWorkItem::gid[0] = x;
            RefWorkItem::gid[1] = y;
            RefWorkItem::lid[0] = x % lx;
            RefWorkItem::lid[1] = y % ly;
            f();
        }
}
