// Host side of the mesh: the uniform Sierpinski mesh generator (a restatement of
// init_grid, src/SFC_node_traversal.f90:22-292) and the conversion of a mesh
// in the C-ABI layout into the per-segment edge task lists the step kernel
// reads. Both run once per remesh, not per step.
#include "swe_internal.h"

#include <algorithm>
#include <cstring>
#include <memory>
#include <vector>

namespace swe {

namespace {

// Sierpinski grammar state of one cell (src/SFC_data_types.f90:84-91).
struct GrammarCell {
    int8_t prev_bnd, next_bnd;  // previous / next crossed edge on the domain boundary
    int8_t color_type;          // OLD = 0, NEW = 1, OLD_BND = 2, NEW_BND = 3
    int8_t depth, plotter, turtle, color;
};

constexpr int kK = 1, kV = 2, kH = 3;
constexpr int kRed = -1, kGreen = 0;

// Children of a bisected cell, create_child_cells (src/SFC_node_traversal.f90:252-292).
void bisect(const GrammarCell& p, GrammarCell& c1, GrammarCell& c2) {
    static const int8_t first_turtle[4] = {0, kH, kH, kV};
    static const int8_t second_turtle[4] = {0, kV, kK, kK};
    // i_plotter_child_type(-8:8)
    static const int8_t child_plotter[17] = {3, 2, 1, 8, 7, 6, 5, 4, 0, -6, -7, -8, -1, -2, -3, -4, -5};
    c1.turtle = first_turtle[p.turtle];
    c2.turtle = second_turtle[p.turtle];
    c1.plotter = child_plotter[p.plotter + 8];
    c2.plotter = (int8_t)-child_plotter[-p.plotter + 8];
    c1.depth = c2.depth = (int8_t)(p.depth + 1);
    const int8_t flip = (int8_t)(kRed + kGreen - p.color);
    // first child: previous edge of the parent, new crossed edge to the sibling
    c1.prev_bnd = p.prev_bnd;
    c1.next_bnd = 0;
    // second child: old crossed edge from the sibling, next edge of the parent
    c2.prev_bnd = 0;
    c2.next_bnd = p.next_bnd;
    if (p.turtle == kK) {
        c1.color_type = (int8_t)(1 | (p.next_bnd << 1));  // the parent's next edge
        c2.color_type = p.color_type;
        c1.color = flip;
        c2.color = p.color;
    } else if (p.turtle == kV) {
        c1.color_type = p.color_type;
        c2.color_type = p.color_type;
        c1.color = c2.color = p.color;
    } else {
        c1.color_type = p.color_type;
        c2.color_type = (int8_t)(0 | (p.prev_bnd << 1));  // the parent's previous edge
        c1.color = p.color;
        c2.color = flip;
    }
}

// Local edge index (1..3) of the previous, colour and next edge per turtle type
// (cell_get_edge_indices, src/SFC_data_types.f90:370-384).
const int8_t kPrevIdx[4] = {0, 3, 3, 2};
const int8_t kColorIdx[4] = {0, 1, 2, 3};
const int8_t kNextIdx[4] = {0, 2, 1, 1};

}  // namespace

int64_t uniform_boundary_edges(int depth) { return (int64_t)4 << (depth / 2); }

// The Sierpinski walk of init_grid over a tree given by its leaf depths in
// traversal order (depth-first bisection with an explicit stack: a node is
// bisected while it is shallower than the next leaf's depth), numbering the
// edges the way the traversal's colour-edge stacks meet them. A uniform mesh
// is the sequence of 2^(d+1) leaves of depth d.
namespace {
// Outward unit normals of the local edges by plotter type (geometry_tables).
struct NormalTable {
    double n[17][3][2];
    NormalTable() {
        double leg[kMaxDepth + 2], vol[kMaxDepth + 1];
        geometry_tables(leg, vol, n);
    }
};
}  // namespace

int build_mesh(int64_t n_leaves, const int8_t* leaf_depth, int uniform_depth, int want, BuiltMesh& m) {
    const bool want_vertices = (want & kWantVertices) != 0, want_legs = (want & kWantLegs) != 0;
    static const NormalTable normals;
    const bool uniform = leaf_depth == nullptr;
    if (uniform) n_leaves = (int64_t)2 << uniform_depth;
    if (n_leaves < 2) return set_error(SWE_E_INVALID, "a mesh has at least the two root cells");
    m.n = n_leaves;
    m.depth.assign((size_t)n_leaves, 0);
    m.plotter.assign((size_t)n_leaves, 0);
    m.parent.assign((size_t)n_leaves, 0);
    m.ec.assign((size_t)(3 * n_leaves), -1);  // at most (3 n) / 2 edges, two cells each
    m.el.assign((size_t)(3 * n_leaves), 0);
    m.bc.clear();
    m.bl.clear();
    if (want_vertices) m.vert.assign((size_t)(6 * n_leaves), 0.0);
    else m.vert.clear();
    if (want_legs) m.leg.assign((size_t)n_leaves, 0);
    else m.leg.clear();

    struct Item {
        GrammarCell c;
        double x[3][2];
        int64_t parent;
    };
    std::vector<Item> stack;
    stack.reserve(2 * (size_t)kMaxDepth + 8);
    // the two root triangles of the unit square (init_section, src/SFC_node_traversal.f90:90-109);
    // pushed in reverse so the first one is expanded first
    Item r2{{0, 1, 3, 0, -6, kH, kRed}, {{1, 1}, {0, 1}, {0, 0}}, -2};
    Item r1{{1, 0, 2, 0, -2, kK, kRed}, {{0, 0}, {1, 0}, {1, 1}}, -1};
    stack.push_back(r2);
    stack.push_back(r1);

    std::vector<int64_t> color_stack[2];
    int64_t open_crossed = -1, next_edge = 0, k = 0, node = 0;
    while (!stack.empty()) {
        Item it = stack.back();
        stack.pop_back();
        if (k >= n_leaves) return set_error(SWE_E_INVALID, "depth sequence ends before the tree does");
        const int target = uniform ? uniform_depth : leaf_depth[k];
        if (target < 0 || target > kMaxDepth)
            return set_error(SWE_E_INVALID, "cell %lld: depth %d out of range", (long long)k, target);
        if (it.c.depth < target) {
            Item a, b;
            bisect(it.c, a.c, b.c);
            double mx = 0.5 * (it.x[0][0] + it.x[2][0]), my = 0.5 * (it.x[0][1] + it.x[2][1]);
            a.x[0][0] = it.x[0][0]; a.x[0][1] = it.x[0][1];
            a.x[1][0] = mx; a.x[1][1] = my;
            a.x[2][0] = it.x[1][0]; a.x[2][1] = it.x[1][1];
            b.x[0][0] = it.x[1][0]; b.x[0][1] = it.x[1][1];
            b.x[1][0] = mx; b.x[1][1] = my;
            b.x[2][0] = it.x[2][0]; b.x[2][1] = it.x[2][1];
            a.parent = b.parent = node++;
            stack.push_back(b);
            stack.push_back(a);
            continue;
        }
        if (it.c.depth > target)
            return set_error(SWE_E_INVALID, "cell %lld: depth %d is not a leaf of the tree (node depth %d)",
                             (long long)k, target, it.c.depth);
        // a leaf: cell number k in traversal order
        const GrammarCell& c = it.c;
        m.depth[(size_t)k] = c.depth;
        m.plotter[(size_t)k] = c.plotter;
        m.parent[(size_t)k] = it.parent;
        if (want_vertices)
            for (int v = 0; v < 3; ++v) {
                m.vert[(size_t)(6 * k + 2 * v)] = it.x[v][0];
                m.vert[(size_t)(6 * k + 2 * v + 1)] = it.x[v][1];
            }
        if (want_legs) {
            // which local edge is the leg (x0, x1), where x0 -> x2 is the hypotenuse and
            // x1 the right-angle vertex: the outward normal of (x0, x1) points along
            // x1 - x2, so its dot product with x2 - x0 is negative, the other leg's
            // positive (which end of the hypotenuse comes first is not a function of
            // the plotter type alone)
            const double* nv = normals.n[c.plotter + 8][0];
            const double dd = nv[0] * (it.x[2][0] - it.x[0][0]) + nv[1] * (it.x[2][1] - it.x[0][1]);
            m.leg[(size_t)k] = dd < 0.0 ? 0 : 2;
        }
        const int8_t ip = kPrevIdx[c.turtle], ic = kColorIdx[c.turtle], in = kNextIdx[c.turtle];
        // previous crossed edge: the open crossed edge of the previous cell, or the boundary
        if (!c.prev_bnd) {
            if (open_crossed < 0) return set_error(SWE_E_INVALID, "mesh walk: missing crossed edge");
            m.ec[(size_t)(2 * open_crossed + 1)] = k;
            m.el[(size_t)(2 * open_crossed + 1)] = ip;
        } else {
            m.bc.push_back(k);
            m.bl.push_back(ip);
        }
        open_crossed = -1;
        // colour edge: first touch pushes, second touch pops
        std::vector<int64_t>& cs = color_stack[c.color + 1];
        if (c.color_type == 0) {
            if (cs.empty()) return set_error(SWE_E_INVALID, "mesh walk: colour stack underflow (not conforming)");
            int64_t e = cs.back();
            cs.pop_back();
            m.ec[(size_t)(2 * e + 1)] = k;
            m.el[(size_t)(2 * e + 1)] = ic;
        } else if (c.color_type == 1) {
            int64_t e = next_edge++;
            cs.push_back(e);
            m.ec[(size_t)(2 * e)] = k;
            m.el[(size_t)(2 * e)] = ic;
        } else {
            m.bc.push_back(k);
            m.bl.push_back(ic);
        }
        // next crossed edge
        if (!c.next_bnd) {
            int64_t e = next_edge++;
            m.ec[(size_t)(2 * e)] = k;
            m.el[(size_t)(2 * e)] = in;
            open_crossed = e;
        } else {
            m.bc.push_back(k);
            m.bl.push_back(in);
        }
        ++k;
    }
    if (k != n_leaves) return set_error(SWE_E_INVALID, "depth sequence longer than the tree");
    if (open_crossed >= 0 || !color_stack[0].empty() || !color_stack[1].empty())
        return set_error(SWE_E_INVALID, "mesh walk inconsistent (not conforming)");
    m.ne = next_edge;
    m.nb = (int64_t)m.bc.size();
    if (2 * m.ne + m.nb != 3 * m.n) return set_error(SWE_E_INVALID, "mesh walk: edge count inconsistent");
    for (int64_t e = 0; e < m.ne; ++e)
        if (m.ec[(size_t)(2 * e + 1)] < 0) return set_error(SWE_E_INVALID, "mesh walk: edge %lld has one cell",
                                                            (long long)e);
    m.ec.resize((size_t)(2 * m.ne));
    m.el.resize((size_t)(2 * m.ne));
    return SWE_OK;
}

int mesh_uniform(int depth, int64_t* n_cells, int64_t* n_edges, int64_t* n_bnd, int8_t* depth_out,
                 int8_t* plotter_out, int64_t* edge_cells, int8_t* edge_local, int64_t* bnd_cell, int8_t* bnd_local,
                 double* centroids, double* vertices) {
    if (depth < 0 || depth > 29) return set_error(SWE_E_INVALID, "mesh depth %d out of range 0..29", depth);
    const int64_t n = (int64_t)2 << depth;
    const int64_t nb = uniform_boundary_edges(depth);
    const int64_t ne = (3 * n - nb) / 2;
    if (n_cells) *n_cells = n;
    if (n_edges) *n_edges = ne;
    if (n_bnd) *n_bnd = nb;
    if (!depth_out && !plotter_out && !edge_cells && !edge_local && !bnd_cell && !bnd_local && !centroids &&
        !vertices)
        return SWE_OK;
    if (!depth_out || !plotter_out || !edge_cells || !edge_local || !bnd_cell || !bnd_local)
        return set_error(SWE_E_INVALID, "mesh outputs must all be given (centroids optional)");
    BuiltMesh m;
    int rc = build_mesh(n, nullptr, depth, (centroids || vertices) ? kWantVertices : 0, m);
    if (rc) return rc;
    return export_mesh(m, depth_out, plotter_out, edge_cells, edge_local, bnd_cell, bnd_local, centroids, vertices);
}

int export_mesh(const BuiltMesh& m, int8_t* depth_out, int8_t* plotter_out, int64_t* edge_cells, int8_t* edge_local,
                int64_t* bnd_cell, int8_t* bnd_local, double* centroids, double* vertices) {
    if (depth_out) std::memcpy(depth_out, m.depth.data(), (size_t)m.n);
    if (plotter_out) std::memcpy(plotter_out, m.plotter.data(), (size_t)m.n);
    if (edge_cells) std::memcpy(edge_cells, m.ec.data(), sizeof(int64_t) * 2 * (size_t)m.ne);
    if (edge_local) std::memcpy(edge_local, m.el.data(), 2 * (size_t)m.ne);
    if (bnd_cell) std::memcpy(bnd_cell, m.bc.data(), sizeof(int64_t) * (size_t)m.nb);
    if (bnd_local) std::memcpy(bnd_local, m.bl.data(), (size_t)m.nb);
    if (centroids && !m.vert.empty())
        for (int64_t k = 0; k < m.n; ++k) {
            const double* x = &m.vert[(size_t)(6 * k)];
            centroids[2 * k] = ((x[0] + x[2]) + x[4]) / 3.0;
            centroids[2 * k + 1] = ((x[1] + x[3]) + x[5]) / 3.0;
        }
    if (vertices && !m.vert.empty()) std::memcpy(vertices, m.vert.data(), sizeof(double) * 6 * (size_t)m.n);
    return SWE_OK;
}

// Per-segment edge tasks of one instance whose cells start at `offset` in the
// context's arrays; appended to seg_ptr / seg_info / tasks. An inner edge with
// both cells in one segment is one task there; an edge between two segments is
// a task in both (each keeps its own side, so no segment waits for another). A
// boundary edge is a task in its cell's segment. Boundary tasks come first in a
// segment, then inner edges in stream (first-touch) order.
// Direction of the outward normal of local edge k (0..2) of a cell with plotter
// type p: 1 = along x, 2 = along y, 0 = diagonal.
// Direction of the outward normal of local edge k of a cell of plotter type p:
// 0 diagonal, 1 along x, 2 along y (a table built once, thread-safe).
static int normal_axis(int p, int k) {
    struct AxisTable {
        int8_t axis[17][3];
        AxisTable() {
            double normal[17][3][2], leg[kMaxDepth + 2], vol[kMaxDepth + 1];
            geometry_tables(leg, vol, normal);
            for (int q = 0; q < 17; ++q)
                for (int e = 0; e < 3; ++e) {
                    const double* nv = normal[q][e];
                    axis[q][e] = (nv[1] == 0.0 && nv[0] != 0.0) ? 1 : (nv[0] == 0.0 && nv[1] != 0.0) ? 2 : 0;
                }
        }
    };
    static const AxisTable table;
    return table.axis[p + 8][k];
}

// The segment lists: per segment the edges to compute, diagonal ones first, then
// the axis-aligned ones (so a warp's tasks mostly take the same branch of the
// flux's rotation), then the halo tasks, each class in input order (boundary
// edges, then inner edges). Placed by counting, no sort.
int build_tasks(const HostMesh& m, int64_t offset, int32_t inst, int32_t T, std::vector<int64_t>& seg_ptr,
                std::vector<SegInfo>& seg_info, hvec<Task>& tasks, hvec<Task>& xtasks) {
    const int64_t n = m.n_cells;
    const int64_t nseg = (n + T - 1) / T;
    if (seg_ptr.empty()) seg_ptr.push_back(0);
    // task kinds: boundary edges and the inner edges inside one segment are class 0
    // (diagonal) or 1 (axis-aligned); an inner edge between two segments is class 2
    // (a halo task) in both. Counted per part of the boundary and edge lists, then
    // placed in list order (boundary edges first, then inner edges; cross edges
    // numbered in edge order), so the lists do not depend on the number of parts.
    const int PB = host_parts(m.n_bnd), PE = host_parts(m.n_edges);
    const size_t ns = (size_t)(3 * nseg);
    std::vector<std::vector<int64_t>> cb((size_t)PB), ce((size_t)PE);
    std::vector<int64_t> xc((size_t)PE, 0);
    parallel_parts(m.n_bnd, PB, [&](int64_t j0, int64_t j1, int p) {
        std::vector<int64_t>& c = cb[(size_t)p];
        c.assign(ns, 0);
        for (int64_t j = j0; j < j1; ++j) {
            const int64_t cell = m.bc[(size_t)j];
            const int ax = normal_axis(m.plotter[(size_t)cell], m.bl[(size_t)j] - 1);
            c[(size_t)(3 * (cell / T) + (ax ? 1 : 0))]++;
        }
    });
    parallel_parts(m.n_edges, PE, [&](int64_t e0, int64_t e1, int p) {
        std::vector<int64_t>& c = ce[(size_t)p];
        c.assign(ns, 0);
        int64_t x = 0;
        for (int64_t e = e0; e < e1; ++e) {
            const int64_t a = m.ea[(size_t)e], b = m.eb[(size_t)e];
            const int64_t sa = a / T, sb = b / T;
            if (sa == sb) {
                const int ax = normal_axis(m.plotter[(size_t)a], m.la[(size_t)e] - 1);
                c[(size_t)(3 * sa + (ax ? 1 : 0))]++;
            } else {
                c[(size_t)(3 * sa + 2)]++;
                c[(size_t)(3 * sb + 2)]++;
                ++x;
            }
        }
        xc[(size_t)p] = x;
    });
    // slot starts: segments in order, classes 0, 1, 2 within a segment
    const int64_t base = seg_ptr.back();
    std::vector<int64_t> fill(ns);
    int64_t pos = base;
    for (int64_t sg = 0; sg < nseg; ++sg) {
        for (int k = 0; k < 3; ++k) {
            const size_t sl = (size_t)(3 * sg + k);
            fill[sl] = pos;
            int64_t cnt = 0;
            for (int p = 0; p < PB; ++p) cnt += cb[(size_t)p][sl];
            for (int p = 0; p < PE; ++p) cnt += ce[(size_t)p][sl];
            pos += cnt;
            if (k == 2) {
                SegInfo si;
                si.c0 = (int32_t)(offset + sg * T);
                si.cn = (int32_t)std::min<int64_t>(T, n - sg * T);
                si.inst = inst;
                si.halo = (int32_t)cnt;
                seg_info.push_back(si);
            }
        }
        seg_ptr.push_back(pos);
    }
    // each part's first position per slot (turn the counts into running starts)
    for (size_t sl = 0; sl < ns; ++sl) {
        int64_t at = fill[sl];
        for (int p = 0; p < PB; ++p) {
            const int64_t c = cb[(size_t)p][sl];
            cb[(size_t)p][sl] = at;
            at += c;
        }
        for (int p = 0; p < PE; ++p) {
            const int64_t c = ce[(size_t)p][sl];
            ce[(size_t)p][sl] = at;
            at += c;
        }
    }
    int64_t nx = (int64_t)xtasks.size();
    for (int p = 0; p < PE; ++p) {
        const int64_t c = xc[(size_t)p];
        xc[(size_t)p] = nx;
        nx += c;
    }
    if (nx > ((int64_t)1 << 31)) return set_error(SWE_E_INVALID, "too many cross-segment edges");
    tasks.resize((size_t)pos);
    xtasks.resize((size_t)nx);
    parallel_parts(m.n_bnd, PB, [&](int64_t j0, int64_t j1, int p) {
        std::vector<int64_t>& at = cb[(size_t)p];
        for (int64_t j = j0; j < j1; ++j) {
            const int64_t c = m.bc[(size_t)j];
            const int ax = normal_axis(m.plotter[(size_t)c], m.bl[(size_t)j] - 1);
            Task t;
            t.a = (int32_t)(offset + c);
            t.b = -1;
            t.meta = pack_meta(m.bl[(size_t)j] - 1, 0, m.plotter[(size_t)c], 1, true, ax);
            t.pad = 0;
            tasks[(size_t)at[(size_t)(3 * (c / T) + (ax ? 1 : 0))]++] = t;
        }
    });
    parallel_parts(m.n_edges, PE, [&](int64_t e0, int64_t e1, int p) {
        std::vector<int64_t>& at = ce[(size_t)p];
        int64_t xi = xc[(size_t)p];
        for (int64_t e = e0; e < e1; ++e) {
            const int64_t a = m.ea[(size_t)e], b = m.eb[(size_t)e];
            const int ax = normal_axis(m.plotter[(size_t)a], m.la[(size_t)e] - 1);
            Task t;
            t.a = (int32_t)(offset + a);
            t.b = (int32_t)(offset + b);
            t.meta = pack_meta(m.la[(size_t)e] - 1, m.lb[(size_t)e] - 1, m.plotter[(size_t)a], m.plotter[(size_t)b],
                               false, ax);
            t.pad = 0;
            const int64_t sa = a / T, sb = b / T;
            if (sb == sa) {
                tasks[(size_t)at[(size_t)(3 * sa + (ax ? 1 : 0))]++] = t;
                continue;
            }
            // an edge between two segments: computed once by the cross-edge pass,
            // each segment copies its own side's update
            Task h = t;
            h.meta |= kHaloBit;
            h.pad = (uint32_t)xi;
            t.pad = (uint32_t)inst;
            xtasks[(size_t)xi++] = t;
            tasks[(size_t)at[(size_t)(3 * sa + 2)]++] = h;
            tasks[(size_t)at[(size_t)(3 * sb + 2)]++] = h;
        }
    });
    return SWE_OK;
}

// Validate a mesh given through the C ABI and store it with a < b per edge, one
// item after the other: the first bad item in list order is the one reported.
static int ingest_serial(HostMesh& m, int64_t n_cells, const int8_t* depth, const int8_t* plotter, int64_t n_edges,
                const int64_t* edge_cells, const int8_t* edge_local, int64_t n_bnd, const int64_t* bnd_cell,
                const int8_t* bnd_local) {
    if (n_cells <= 0 || n_cells >= ((int64_t)1 << 31) - 1)
        return set_error(SWE_E_INVALID, "n_cells %lld out of range", (long long)n_cells);
    if (n_edges < 0 || n_bnd < 0 || 2 * n_edges + n_bnd != 3 * n_cells)
        return set_error(SWE_E_INVALID, "edge counts inconsistent: 2*%lld + %lld != 3*%lld", (long long)n_edges,
                         (long long)n_bnd, (long long)n_cells);
    if (!depth || !plotter || (n_edges && (!edge_cells || !edge_local)) || (n_bnd && (!bnd_cell || !bnd_local)))
        return set_error(SWE_E_INVALID, "null mesh array");
    m.n_cells = n_cells;
    m.n_edges = n_edges;
    m.n_bnd = n_bnd;
    m.depth.assign(depth, depth + n_cells);
    m.plotter.assign(plotter, plotter + n_cells);
    int dmin = 127, dmax = -1;
    for (int64_t c = 0; c < n_cells; ++c) {
        int d = depth[c], p = plotter[c];
        if (d < 0 || d > kMaxDepth) return set_error(SWE_E_INVALID, "cell %lld: depth %d", (long long)c, d);
        if (p == 0 || p < -8 || p > 8) return set_error(SWE_E_INVALID, "cell %lld: plotter type %d", (long long)c, p);
        if (d < dmin) dmin = d;
        if (d > dmax) dmax = d;
    }
    m.min_depth = dmin;
    m.max_depth = dmax;
    std::vector<uint8_t> used((size_t)n_cells, 0);
    auto claim = [&](int64_t c, int l) -> bool {
        uint8_t bit = (uint8_t)(1u << (l - 1));
        if (used[(size_t)c] & bit) return false;
        used[(size_t)c] |= bit;
        return true;
    };
    m.ea.resize((size_t)n_edges);
    m.eb.resize((size_t)n_edges);
    m.la.resize((size_t)n_edges);
    m.lb.resize((size_t)n_edges);
    for (int64_t e = 0; e < n_edges; ++e) {
        int64_t a = edge_cells[2 * e], b = edge_cells[2 * e + 1];
        int la = edge_local[2 * e], lb = edge_local[2 * e + 1];
        if (a < 0 || a >= n_cells || b < 0 || b >= n_cells || a == b)
            return set_error(SWE_E_INVALID, "edge %lld: cells (%lld, %lld) invalid", (long long)e, (long long)a,
                             (long long)b);
        if (la < 1 || la > 3 || lb < 1 || lb > 3)
            return set_error(SWE_E_INVALID, "edge %lld: local index out of 1..3", (long long)e);
        if (!claim(a, la) || !claim(b, lb))
            return set_error(SWE_E_INVALID, "edge %lld: a cell's local edge is used twice", (long long)e);
        if (b < a) {
            std::swap(a, b);
            std::swap(la, lb);
        }
        m.ea[(size_t)e] = a;
        m.eb[(size_t)e] = b;
        m.la[(size_t)e] = (int8_t)la;
        m.lb[(size_t)e] = (int8_t)lb;
    }
    m.bc.resize((size_t)n_bnd);
    m.bl.resize((size_t)n_bnd);
    for (int64_t j = 0; j < n_bnd; ++j) {
        int64_t c = bnd_cell[j];
        int l = bnd_local[j];
        if (c < 0 || c >= n_cells || l < 1 || l > 3)
            return set_error(SWE_E_INVALID, "boundary edge %lld invalid", (long long)j);
        if (!claim(c, l)) return set_error(SWE_E_INVALID, "boundary edge %lld: local edge used twice", (long long)j);
        m.bc[(size_t)j] = c;
        m.bl[(size_t)j] = (int8_t)l;
    }
    // 2*n_edges + n_bnd == 3*n_cells and no slot claimed twice => every slot used once
    return SWE_OK;
}

// Validate a mesh given through the C ABI and store it with a < b per edge. A
// large mesh is checked in parts on host threads without atomics: every claim
// of a (cell, local edge) slot writes its edge number into the slot, and a
// second pass checks that each claim still owns its slot (of two claims of one
// slot one loses). With 2 n_edges + n_bnd = 3 n_cells and no slot claimed
// twice, every slot is used once. On any failure the serial check runs again
// and reports the first bad item in list order.
int ingest_mesh(HostMesh& m, int64_t n_cells, const int8_t* depth, const int8_t* plotter, int64_t n_edges,
                const int64_t* edge_cells, const int8_t* edge_local, int64_t n_bnd, const int64_t* bnd_cell,
                const int8_t* bnd_local) {
    const int PE = host_parts(n_edges);
    if (PE == 1 || n_cells <= 0 || n_cells >= ((int64_t)1 << 30) || n_edges < 0 || n_bnd < 0 ||
        2 * n_edges + n_bnd != 3 * n_cells || !depth || !plotter || !edge_cells || !edge_local ||
        (n_bnd && (!bnd_cell || !bnd_local)))
        return ingest_serial(m, n_cells, depth, plotter, n_edges, edge_cells, edge_local, n_bnd, bnd_cell, bnd_local);
    m.n_cells = n_cells;
    m.n_edges = n_edges;
    m.n_bnd = n_bnd;
    m.depth.assign(depth, depth + n_cells);
    m.plotter.assign(plotter, plotter + n_cells);
    const int PC = host_parts(n_cells), PB = host_parts(n_bnd);
    std::vector<int> pmin((size_t)PC, 127), pmax((size_t)PC, -1);
    std::vector<uint8_t> ok((size_t)std::max({PC, PE, PB}), 1);
    parallel_parts(n_cells, PC, [&](int64_t c0, int64_t c1, int p) {
        int lo = 127, hi = -1;
        for (int64_t c = c0; c < c1; ++c) {
            const int d = depth[c], q = plotter[c];
            if (d < 0 || d > kMaxDepth || q == 0 || q < -8 || q > 8) {
                ok[(size_t)p] = 0;
                return;
            }
            lo = std::min(lo, d);
            hi = std::max(hi, d);
        }
        pmin[(size_t)p] = lo;
        pmax[(size_t)p] = hi;
    });
    auto all_ok = [&](int parts) {
        bool r = true;
        for (int p = 0; p < parts; ++p) r = r && ok[(size_t)p];
        return r;
    };
    auto serial = [&]() {
        return ingest_serial(m, n_cells, depth, plotter, n_edges, edge_cells, edge_local, n_bnd, bnd_cell, bnd_local);
    };
    if (!all_ok(PC)) return serial();
    m.min_depth = *std::min_element(pmin.begin(), pmin.end());
    m.max_depth = *std::max_element(pmax.begin(), pmax.end());
    // slot[3 c + l - 1]: the last claim of cell c's local edge l (edge e, or n_edges + j for boundary edge j)
    // (not initialised: every slot is written before it is read, or the check fails
    // earlier; the claims are relaxed atomic stores, plain stores on x86 and Arm)
    std::unique_ptr<uint32_t[]> slot(new uint32_t[(size_t)(3 * n_cells)]);
    auto put = [&](int64_t i, uint32_t v) { __atomic_store_n(&slot[(size_t)i], v, __ATOMIC_RELAXED); };
    m.ea.resize((size_t)n_edges);
    m.eb.resize((size_t)n_edges);
    m.la.resize((size_t)n_edges);
    m.lb.resize((size_t)n_edges);
    m.bc.resize((size_t)n_bnd);
    m.bl.resize((size_t)n_bnd);
    parallel_parts(n_edges, PE, [&](int64_t e0, int64_t e1, int p) {
        for (int64_t e = e0; e < e1; ++e) {
            int64_t a = edge_cells[2 * e], b = edge_cells[2 * e + 1];
            int la = edge_local[2 * e], lb = edge_local[2 * e + 1];
            if (a < 0 || a >= n_cells || b < 0 || b >= n_cells || a == b || la < 1 || la > 3 || lb < 1 || lb > 3) {
                ok[(size_t)p] = 0;
                return;
            }
            put(3 * a + la - 1, (uint32_t)e);
            put(3 * b + lb - 1, (uint32_t)e);
            if (b < a) {
                std::swap(a, b);
                std::swap(la, lb);
            }
            m.ea[(size_t)e] = a;
            m.eb[(size_t)e] = b;
            m.la[(size_t)e] = (int8_t)la;
            m.lb[(size_t)e] = (int8_t)lb;
        }
    });
    if (!all_ok(PE)) return serial();
    parallel_parts(n_bnd, PB, [&](int64_t j0, int64_t j1, int p) {
        for (int64_t j = j0; j < j1; ++j) {
            const int64_t c = bnd_cell[j];
            const int l = bnd_local[j];
            if (c < 0 || c >= n_cells || l < 1 || l > 3) {
                ok[(size_t)p] = 0;
                return;
            }
            put(3 * c + l - 1, (uint32_t)(n_edges + j));
            m.bc[(size_t)j] = c;
            m.bl[(size_t)j] = (int8_t)l;
        }
    });
    if (!all_ok(PB)) return serial();
    parallel_parts(n_edges, PE, [&](int64_t e0, int64_t e1, int p) {
        for (int64_t e = e0; e < e1; ++e)
            if (slot[(size_t)(3 * m.ea[(size_t)e] + m.la[(size_t)e] - 1)] != (uint32_t)e ||
                slot[(size_t)(3 * m.eb[(size_t)e] + m.lb[(size_t)e] - 1)] != (uint32_t)e) {
                ok[(size_t)p] = 0;
                return;
            }
    });
    if (!all_ok(PE)) return serial();
    parallel_parts(n_bnd, PB, [&](int64_t j0, int64_t j1, int p) {
        for (int64_t j = j0; j < j1; ++j)
            if (slot[(size_t)(3 * m.bc[(size_t)j] + m.bl[(size_t)j] - 1)] != (uint32_t)(n_edges + j)) {
                ok[(size_t)p] = 0;
                return;
            }
    });
    if (!all_ok(PB)) return serial();
    return SWE_OK;
}

}  // namespace swe
