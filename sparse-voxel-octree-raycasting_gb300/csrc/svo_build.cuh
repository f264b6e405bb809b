// svo_build.cuh -- the octree builder on the GPU.
//
// Same words as the host builder (svo_host.cpp) and the reference's
// set_voxel + convert_tree_blocks (src/octree/octree.h:32-293): voxels in
// insertion order become 3-D Morton keys with the insertion index in the low
// bits, a radix sort orders them (keys are unique, so the order equals a
// stable sort by Morton key), and every tree level is one compaction of the
// level below (a node is a run of children sharing key >> 3). The compact
// layout's offsets, which the reference fixes by a recursive depth-first
// walk, follow from subtree sizes by prefix sums:
//   * normal nodes (heights depth..7) sit at 10 * (post-order index);
//   * the 6-level blocks, one per height-6 node in depth-first (= Morton)
//     order, start at the first 64-aligned word after the previous block, so
//     block k starts at round64(initial_words) + sum_{j<k} round64(size_j);
//   * inside a block a node's children come first (each child's subtree in
//     child order), then the node's record; the height-6 record is at the
//     block start (octree.h:268-276 moves it there).
#pragma once
#include <cstdint>

namespace svo {

__device__ __forceinline__ uint64_t bld_spread3(uint32_t v) {
    uint64_t x = v & 0x1fffffu;
    x = (x | x << 32) & 0x1f00000000ffffull;
    x = (x | x << 16) & 0x1f0000ff0000ffull;
    x = (x | x << 8) & 0x100f00f00f00f00full;
    x = (x | x << 4) & 0x10c30c30c30c30c3ull;
    x = (x | x << 2) & 0x1249249249249249ull;
    return x;
}

// Sort keys: Morton key (child index x | y<<1 | z<<2 per level, octree.h:58)
// shifted over the insertion index. bad[0] |= 1 for a coordinate outside
// the volume.
__global__ void k_bld_keys(const uint32_t* __restrict__ x, const uint32_t* __restrict__ y,
                           const uint32_t* __restrict__ z, size_t n, int depth, int ib, uint64_t* __restrict__ keys,
                           uint32_t* bad) {
    const uint32_t D = 1u << depth;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const uint32_t a = x[i], b = y[i], c = z[i];
        if (a >= D || b >= D || c >= D) atomicOr(bad, 1u);
        const uint64_t m = bld_spread3(a) | (bld_spread3(b) << 1) | (bld_spread3(c) << 2);
        keys[i] = (m << ib) | (uint64_t)i;
    }
}

// ------------------------------------------------------------ radix sort --
// LSD radix sort of unique 64-bit keys, 8-bit digits. Each block owns a tile
// of kSortTile keys; within a tile the keys keep their order (ranks from
// __match_any_sync per warp, then per-warp digit counts scanned across the
// block), so every pass is stable.
constexpr int kSortThreads = 256;
constexpr int kSortIters = 8;
constexpr int kSortTile = kSortThreads * kSortIters;

__global__ void __launch_bounds__(kSortThreads) k_sort_hist(const uint64_t* __restrict__ keys, size_t n, int shift,
                                                            uint32_t* __restrict__ counts, uint32_t nblocks) {
    __shared__ uint32_t h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    const size_t base = (size_t)blockIdx.x * kSortTile;
    for (int it = 0; it < kSortIters; ++it) {
        const size_t i = base + (size_t)it * kSortThreads + threadIdx.x;
        if (i < n) atomicAdd(&h[(keys[i] >> shift) & 255u], 1u);
    }
    __syncthreads();
    counts[(size_t)threadIdx.x * nblocks + blockIdx.x] = h[threadIdx.x];
}

__global__ void __launch_bounds__(kSortThreads) k_sort_scatter(const uint64_t* __restrict__ in,
                                                               uint64_t* __restrict__ out, size_t n, int shift,
                                                               const uint32_t* __restrict__ offsets,
                                                               uint32_t nblocks) {
    constexpr int kWarps = kSortThreads / 32;
    __shared__ uint32_t warp_cnt[kWarps][256];
    __shared__ uint32_t running[256];
    __shared__ uint32_t base_off[256];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    running[tid] = 0;
    base_off[tid] = offsets[(size_t)tid * nblocks + blockIdx.x];
    const size_t base = (size_t)blockIdx.x * kSortTile;
    for (int it = 0; it < kSortIters; ++it) {
        for (int w = 0; w < kWarps; ++w) warp_cnt[w][tid] = 0;
        __syncthreads();
        const size_t i = base + (size_t)it * kSortThreads + tid;
        const bool valid = i < n;
        const uint64_t key = valid ? in[i] : 0ull;
        const uint32_t d = valid ? (uint32_t)((key >> shift) & 255u) : 256u;
        const uint32_t peers = __match_any_sync(0xffffffffu, d);
        const uint32_t rank = (uint32_t)__popc(peers & ((1u << lane) - 1u));
        if (valid && rank == 0) warp_cnt[warp][d] = (uint32_t)__popc(peers);
        __syncthreads();
        {  // exclusive scan of digit tid's counts over the warps
            uint32_t acc = 0;
            for (int w = 0; w < kWarps; ++w) {
                const uint32_t c = warp_cnt[w][tid];
                warp_cnt[w][tid] = acc;
                acc += c;
            }
            __syncthreads();
            if (valid) out[base_off[d] + running[d] + warp_cnt[warp][d] + rank] = key;
            __syncthreads();
            running[tid] += acc;
        }
    }
}

// ------------------------------------------------------------------ scan --
// Exclusive prefix sum of uint32 (blocks of 1024 threads x 4 items, block
// sums scanned recursively by the host).
constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanThreads * kScanItems;

// in and out may be the same array (each thread reads its items before it
// writes them; threads own disjoint items).
__global__ void __launch_bounds__(kScanThreads) k_scan_tiles(const uint32_t* in, uint32_t* out, size_t n,
                                                             uint32_t* __restrict__ tile_sums) {
    __shared__ uint32_t warp_sums[32];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const size_t base = (size_t)blockIdx.x * kScanTile + (size_t)tid * kScanItems;
    uint32_t v[kScanItems], local = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        v[k] = base + k < n ? in[base + k] : 0u;
        local += v[k];
    }
    uint32_t incl = local;
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    if (lane == 31) warp_sums[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = warp_sums[lane];
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += t;
        }
        warp_sums[lane] = w;
    }
    __syncthreads();
    uint32_t acc = incl - local + (warp > 0 ? warp_sums[warp - 1] : 0u);
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        if (base + k < n) out[base + k] = acc;
        acc += v[k];
    }
    if (tid == kScanThreads - 1 && tile_sums) tile_sums[blockIdx.x] = warp_sums[31];
}

__global__ void k_scan_add(uint32_t* __restrict__ out, size_t n, const uint32_t* __restrict__ tile_offsets) {
    const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i < n) out[i] += tile_offsets[i / kScanTile];
}

// ---------------------------------------------------------------- levels --
// Run starts: flag[i] = 1 where key >> shift differs from the previous key.
__global__ void k_bld_flags(const uint64_t* __restrict__ key, size_t n, int shift, uint32_t* __restrict__ flags) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        flags[i] = (i == 0 || (key[i] >> shift) != (key[i - 1] >> shift)) ? 1u : 0u;
}

// Level 0 (unique voxels): Morton key, first insertion (the lowest index of
// the run, as keys sort by index within a Morton key), leaf colour = colour
// of the last insertion (octree.h:82-86 overwrites it), run start.
__global__ void k_bld_level0(const uint64_t* __restrict__ keys, size_t n, int ib, const uint32_t* __restrict__ flags,
                             const uint32_t* __restrict__ pos, const uint32_t* __restrict__ rgba,
                             uint64_t* __restrict__ key0, uint32_t* __restrict__ first0, uint32_t* __restrict__ begin0,
                             uint32_t* __restrict__ leaf) {
    const uint64_t imask = (1ull << ib) - 1ull;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const uint32_t r = pos[i] + flags[i] - 1u;
        if (flags[i]) {
            key0[r] = keys[i] >> ib;
            first0[r] = (uint32_t)(keys[i] & imask);
            begin0[r] = (uint32_t)i;
        }
        if (i + 1 == n || flags[i + 1]) leaf[r] = rgba[(uint32_t)(keys[i] & imask)];
    }
}

// Parents of a level: key >> 3 at each run start, the run start as `begin`.
__global__ void k_bld_parents(const uint64_t* __restrict__ ckey, size_t m, const uint32_t* __restrict__ flags,
                              const uint32_t* __restrict__ pos, uint64_t* __restrict__ key, uint32_t* __restrict__ begin) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < m; i += (size_t)gridDim.x * blockDim.x)
        if (flags[i]) {
            key[pos[i]] = ckey[i] >> 3;
            begin[pos[i]] = (uint32_t)i;
        }
}

// Child mask and first insertion of every parent (its children are
// begin[p] .. begin[p+1]-1, at most 8).
__global__ void k_bld_reduce(const uint64_t* __restrict__ ckey, const uint32_t* __restrict__ cfirst, size_t np,
                             const uint32_t* __restrict__ begin, uint8_t* __restrict__ mask,
                             uint32_t* __restrict__ first) {
    for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < np; p += (size_t)gridDim.x * blockDim.x) {
        uint32_t mk = 0, f = 0xffffffffu;
        for (uint32_t c = begin[p]; c < begin[p + 1]; ++c) {
            mk |= 1u << (uint32_t)(ckey[c] & 7u);
            f = min(f, cfirst[c]);
        }
        mask[p] = (uint8_t)mk;
        first[p] = f;
    }
}

// ------------------------------------------------------------------ sizes --
// Words each block-level node's subtree occupies (children first, then the
// node's record). Height 2: one byte-packed record (colour byte, the child
// masks, the non-zero leaf colour bytes, octree.h:126-140). Heights 3-6: the
// children's subtrees plus 1 + (child count) words.
__global__ void k_bld_size2(size_t n2, const uint32_t* __restrict__ begin2, const uint32_t* __restrict__ begin1,
                            const uint32_t* __restrict__ leaf, uint32_t* __restrict__ size2) {
    for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < n2; p += (size_t)gridDim.x * blockDim.x) {
        uint32_t bytes = 1;
        for (uint32_t c = begin2[p]; c < begin2[p + 1]; ++c) {
            ++bytes;
            for (uint32_t v = begin1[c]; v < begin1[c + 1]; ++v) bytes += leaf[v] != 0u;
        }
        size2[p] = (bytes + 3) / 4;
    }
}

__global__ void k_bld_size_up(size_t np, const uint32_t* __restrict__ begin, const uint32_t* __restrict__ csize,
                              uint32_t* __restrict__ size) {
    for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < np; p += (size_t)gridDim.x * blockDim.x) {
        uint32_t s = 1;
        for (uint32_t c = begin[p]; c < begin[p + 1]; ++c) s += 1 + csize[c];
        size[p] = s;
    }
}

__global__ void k_bld_round64(size_t n, const uint32_t* __restrict__ size, uint32_t* __restrict__ out) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        out[i] = (size[i] + 63u) & ~63u;
}

// ------------------------------------------------------------- emission --
// Every store of the emission kernels is checked against the array size; a
// store outside it sets bit 4 of `bad` instead (an internal error).
__device__ __forceinline__ void bld_store(uint32_t* words, size_t limit, size_t at, uint32_t v, uint32_t* bad) {
    if (at < limit) words[at] = v;
    else atomicOr(bad, 4u);
}

struct BlockLevel {
    const uint32_t* begin;  // children of each node
    const uint8_t* mask;
    const uint32_t* first;
    const uint32_t* size;   // subtree words (heights 2-6)
};

// Heights 6..3: each node writes its record and places its children.
// kTop (height 6): the record is at the block start lr = base + off[i] and
// the children follow it; otherwise the node's subtree starts at st[i] (its
// children first) and its record follows them.
template <bool kTop>
__global__ void k_bld_emit_block(size_t np, BlockLevel L, BlockLevel C, bool child_is_h2, const uint32_t* __restrict__ rgba,
                                 const uint32_t* __restrict__ st_in, const uint32_t* __restrict__ lr_in, uint32_t base,
                                 uint32_t* __restrict__ st_out, uint32_t* __restrict__ lr_out, uint32_t* __restrict__ words,
                                 size_t limit, uint32_t* __restrict__ bad) {
    for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < np; p += (size_t)gridDim.x * blockDim.x) {
        const uint32_t c0 = L.begin[p], c1 = L.begin[p + 1], nch = c1 - c0;
        uint32_t lr, rec, cs;
        if (kTop) {
            lr = base + st_in[p];
            rec = lr;
            cs = lr + 1 + nch;
        } else {
            lr = lr_in[p];
            cs = st_in[p];
            rec = cs + L.size[p] - (1 + nch);
        }
        if (kTop && (lr >> 6) >= (1u << 23)) atomicOr(bad, 2u);
        bld_store(words, limit, rec, rgba[L.first[p]], bad);
        uint32_t at = cs;
        for (uint32_t c = c0; c < c1; ++c) {
            const uint32_t csz = C.size[c];
            const uint32_t crec = child_is_h2 ? at : at + csz - (1 + (C.begin[c + 1] - C.begin[c]));
            const uint32_t rel = crec - lr;
            if (rel >= (1u << 23)) atomicOr(bad, 2u);
            bld_store(words, limit, (size_t)rec + 1 + (c - c0), (rel << 9) + 256u + C.mask[c], bad);
            st_out[c] = at;
            lr_out[c] = lr;
            at += csz;
        }
    }
}

// Height 2: the byte-packed record at st[i].
__global__ void k_bld_emit_h2(size_t n2, BlockLevel L2, const uint32_t* __restrict__ begin1,
                              const uint8_t* __restrict__ mask1, const uint32_t* __restrict__ leaf,
                              const uint32_t* __restrict__ rgba, const uint32_t* __restrict__ st,
                              uint32_t* __restrict__ words, size_t limit, uint32_t* __restrict__ bad) {
    for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < n2; p += (size_t)gridDim.x * blockDim.x) {
        uint32_t at = st[p], acc = 0, nb = 0;
        auto put = [&](uint32_t byte) {
            acc |= (byte & 0xffu) << (8 * (nb & 3));
            if ((++nb & 3) == 0) {
                bld_store(words, limit, at++, acc, bad);
                acc = 0;
            }
        };
        put(rgba[L2.first[p]]);
        const uint32_t c0 = L2.begin[p], c1 = L2.begin[p + 1];
        for (uint32_t c = c0; c < c1; ++c) put(mask1[c]);
        for (uint32_t c = c0; c < c1; ++c)
            for (uint32_t v = begin1[c]; v < begin1[c + 1]; ++v)
                if (leaf[v] != 0u) put(leaf[v]);
        if (nb & 3) bld_store(words, limit, at, acc, bad);
    }
}

// Normal levels: subtree node counts bottom-up, then post-order placement
// top-down: the node with post-order start ps and subtree count cnt sits at
// words 10*(ps+cnt-1) .. +9 (octree.h:232-293: children first).
__global__ void k_bld_count_up(size_t np, const uint32_t* __restrict__ begin, const uint32_t* __restrict__ ccnt,
                               uint32_t* __restrict__ cnt) {
    for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < np; p += (size_t)gridDim.x * blockDim.x) {
        uint32_t s = 1;
        if (ccnt)
            for (uint32_t c = begin[p]; c < begin[p + 1]; ++c) s += ccnt[c];
        cnt[p] = s;
    }
}

__global__ void k_bld_emit_normal(size_t np, int h, int depth, const uint32_t* __restrict__ begin,
                                  const uint8_t* __restrict__ mask, const uint32_t* __restrict__ first,
                                  const uint32_t* __restrict__ cnt, const uint32_t* __restrict__ ps,
                                  const uint64_t* __restrict__ ckey, const uint8_t* __restrict__ cmask,
                                  const uint32_t* __restrict__ ccnt, uint32_t* __restrict__ cps,
                                  const uint32_t* __restrict__ block_off, uint32_t base, const uint32_t* __restrict__ rgba,
                                  uint32_t* __restrict__ words, size_t limit, uint32_t* __restrict__ bad) {
    for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < np; p += (size_t)gridDim.x * blockDim.x) {
        const uint32_t at = 10u * (ps[p] + cnt[p] - 1u);
        if (at >= (1u << 23)) atomicOr(bad, 2u);
        uint32_t cw[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        uint32_t run = ps[p];
        for (uint32_t c = begin[p]; c < begin[p + 1]; ++c) {
            const uint32_t j = (uint32_t)(ckey[c] & 7u);
            if (h - 1 >= 7) {
                cps[c] = run;
                cw[j] = ((10u * (run + ccnt[c] - 1u)) << 9) | cmask[c];
                run += ccnt[c];
            } else {
                const uint32_t lr = base + block_off[c];
                cw[j] = ((lr >> 6) << 9) | 256u | cmask[c];
            }
        }
        for (int j = 0; j < 8; ++j) bld_store(words, limit, (size_t)at + j, cw[j], bad);
        const uint32_t col = h == depth ? 0u : rgba[first[p]];
        bld_store(words, limit, (size_t)at + 8, col, bad);
        bld_store(words, limit, (size_t)at + 9, col, bad);
    }
}

}  // namespace svo
