// Internal declarations shared by the host and device parts of the SWE step library.
#pragma once

#include <stdint.h>

#include <algorithm>
#include <memory>
#include <thread>
#include <type_traits>
#include <utility>
#include <vector>

#include "../../include/samoa_swe.h"

namespace swe {

constexpr int kMaxDepth = 60;  // bit_size(int64) - 4, src/SFC_data_types.f90:77

// One edge task of a segment: 16 bytes, loaded with one 128-bit load.
//   a, b: cells (b = -1 for a domain-boundary edge); on an inner edge a < b.
//   meta: bits 0-1 local edge index of a (0..2), bits 2-3 of b,
//         bits 4-8 plotter type of a + 8, bits 9-13 of b + 8, bit 14 boundary,
//         bits 15-16 normal direction: 0 diagonal, 1 along x, 2 along y (the
//         same for both cells: their normals are opposite), bit 17 halo.
//   pad: in a segment's list, a halo task (an edge whose other cell lies in
//        another segment) holds the edge's index in the cross-edge list, whose
//        pass computes both sides' updates once; in the cross-edge list, the
//        instance.
constexpr uint32_t kHaloBit = 1u << 17;
struct alignas(16) Task {
    int32_t a, b;
    uint32_t meta;
    uint32_t pad;
};

inline uint32_t pack_meta(int la, int lb, int pa, int pb, bool bnd, int axis = 0) {
    return (uint32_t)la | ((uint32_t)lb << 2) | ((uint32_t)(pa + 8) << 4) | ((uint32_t)(pb + 8) << 9) |
           ((uint32_t)(bnd ? 1 : 0) << 14) | ((uint32_t)axis << 15);
}

// Per-instance parameters on the device (the cfg fields the step reads,
// src/Config.f90:30-121, plus the depth range present in the instance's mesh).
// dt_by_max: the cell volumes are exactly RN(scaling^2) * 2^-(d+1) for every
// depth of the mesh (no underflow), so min over cells of RN(volume / ds) equals
// RN(RN(scaling^2) / max over cells of ds * 2^(d+1)) and the step divides once
// per instance instead of once per cell.
struct InstParams {
    double drytol, courant, scaling, thr_refine, thr_coarsen, max_time, tout;
    int32_t min_depth, max_depth, dmin, ndepth, bc, dt_by_max;
};

// Per-instance scalars on the device. The step kernel reads dt, reduces into
// dt_acc / refine_acc, and the last CTA to finish advances time and dt, so
// many steps run back to back without the host.
struct InstScalars {
    double time;                    // grid%r_time
    double dt;                      // grid%r_dt for the next step
    double dt_new;                  // min(volume / sum(len * speed)) of the last step
    unsigned long long dt_acc;      // bits of the running minimum (non-negative doubles order as integers)
    unsigned long long ds_acc;      // bits of the running maximum of ds * 2^(d+1) (dt_by_max)
    unsigned long long refine_acc;  // refinements issued in the running step
    unsigned long long n_refine;    // refinements issued in the last step
};

struct GlobalScalars {
    unsigned int done;       // CTAs finished in the running step
    unsigned int error;      // nonzero: a kernel saw a bad index or a wait ran out
    unsigned int next_seg;   // next segment to hand out in the running step
    unsigned int pad;
    long long step;          // steps since the mesh upload (parity = traversal direction)
    long long dt_seq_base;   // step at which the frozen dt sequence starts
};

// Mesh as ingested from the C ABI (validated, a < b on inner edges).
// std::vector storage whose resize leaves new elements default-initialised (no
// zeroing pass): large host arrays are first written, page by page, by the
// threads that fill them.
template <class T>
struct NoInit : std::allocator<T> {
    template <class U>
    struct rebind {
        using other = NoInit<U>;
    };
    NoInit() = default;
    template <class U>
    NoInit(const NoInit<U>&) noexcept {}
    template <class U>
    void construct(U* p) noexcept(std::is_nothrow_default_constructible<U>::value) {
        ::new ((void*)p) U;
    }
    template <class U, class... A>
    void construct(U* p, A&&... a) {
        ::new ((void*)p) U(std::forward<A>(a)...);
    }
};
template <class T>
using hvec = std::vector<T, NoInit<T>>;

struct HostMesh {
    int64_t n_cells = 0, n_edges = 0, n_bnd = 0;
    int min_depth = 0, max_depth = 0;
    std::vector<int8_t> depth, plotter;
    hvec<int64_t> ea, eb, bc;
    hvec<int8_t> la, lb, bl;
};

int set_error(int code, const char* fmt, ...);

// Host passes over large meshes run on several threads: [0, n) is split into
// `parts` contiguous ranges, fn(begin, end, part) runs each (part 0 on the
// calling thread). Meshes below 2^20 items stay on one thread.
#ifndef SWE_HOST_THREADS
#define SWE_HOST_THREADS 16
#endif
inline int host_parts(int64_t n) {
    if (n < ((int64_t)1 << 20)) return 1;
    const int hw = (int)std::max(1u, std::thread::hardware_concurrency());
    return (int)std::max<int64_t>(1, std::min<int64_t>({(int64_t)std::min(hw, SWE_HOST_THREADS), n >> 16}));
}
template <class F>
void parallel_parts(int64_t n, int parts, F&& fn) {
    auto range = [&](int p, int64_t& b, int64_t& e) {
        b = n * p / parts;
        e = n * (p + 1) / parts;
    };
    std::vector<std::thread> th;
    for (int p = 1; p < parts; ++p) {
        int64_t b, e;
        range(p, b, e);
        th.emplace_back([&fn, b, e, p] { fn(b, e, p); });
    }
    int64_t b, e;
    range(0, b, e);
    fn(b, e, 0);
    for (auto& t : th) t.join();
}

// A mesh built by the Sierpinski walk from its leaf depths (swe_mesh.cpp).
struct BuiltMesh {
    int64_t n = 0, ne = 0, nb = 0;
    std::vector<int8_t> depth, plotter, el, bl;
    std::vector<int64_t> ec, bc;
    std::vector<double> vert;     // 6 per cell (optional)
    std::vector<int8_t> leg;      // per cell (optional): the local edge index of the leg (x0, x1)
    std::vector<int64_t> parent;  // the bisected node a leaf came from (negative for the two roots)
};
// What build_mesh records besides the streams.
constexpr int kWantVertices = 1;  // BuiltMesh::vert
constexpr int kWantLegs = 2;      // BuiltMesh::leg
// Result of one remesh (swe_adapt.cpp): new leaf depths in traversal order, for
// each new cell its source cell(s) (second = -1 unless two siblings merged),
// and the transferred h, hu, hv, b (empty where no input was given).
struct AdaptResult {
    int64_t n = 0;
    std::vector<int8_t> depth;
    std::vector<std::pair<int64_t, int64_t>> source;
    std::vector<double> state[4];
    void reserve_hint(int64_t n0) {
        depth.reserve((size_t)n0 + (size_t)n0 / 4);
        source.reserve((size_t)n0 + (size_t)n0 / 4);
    }
};
int mesh_adapt(int64_t n, const int8_t* depth, const int8_t* flags, const double* const in[4], AdaptResult& out);
int build_mesh(int64_t n_leaves, const int8_t* leaf_depth, int uniform_depth, int want, BuiltMesh& m);
int export_mesh(const BuiltMesh& m, int8_t* depth_out, int8_t* plotter_out, int64_t* edge_cells, int8_t* edge_local,
                int64_t* bnd_cell, int8_t* bnd_local, double* centroids, double* vertices);
int mesh_uniform(int depth, int64_t* n_cells, int64_t* n_edges, int64_t* n_bnd, int8_t* depth_out,
                 int8_t* plotter_out, int64_t* edge_cells, int8_t* edge_local, int64_t* bnd_cell,
                 int8_t* bnd_local, double* centroids, double* vertices = nullptr);
int ingest_mesh(HostMesh& m, int64_t n_cells, const int8_t* depth, const int8_t* plotter, int64_t n_edges,
                const int64_t* edge_cells, const int8_t* edge_local, int64_t n_bnd, const int64_t* bnd_cell,
                const int8_t* bnd_local);
// Segment descriptor: cells [c0, c0 + cn) of instance `inst`; the last `halo`
// tasks of its list are halo tasks.
struct alignas(16) SegInfo {
    int32_t c0, cn, inst, halo;
};

// Edge tasks of one instance's segments (appended to seg_ptr / seg_info /
// tasks) and its cross-segment edges (appended to xtasks).
int build_tasks(const HostMesh& m, int64_t offset, int32_t inst, int32_t seg_cells, std::vector<int64_t>& seg_ptr,
                std::vector<SegInfo>& seg_info, hvec<Task>& tasks, hvec<Task>& xtasks);

// Geometry tables restating src/SFC_data_types.f90:509-700 (host side, exact).
void geometry_tables(double leg[kMaxDepth + 2], double vol[kMaxDepth + 1], double normal[17][3][2]);

}  // namespace swe
