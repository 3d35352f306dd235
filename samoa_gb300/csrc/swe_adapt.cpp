// Host adaptivity: one remesh of a conforming Sierpinski mesh from the step's
// refinement flags, a restatement of the adaption traversal's conformity and
// refine/coarsen rules (src/Conformity/Conformity.f90:1244-1317,
// src/SWE/SWE_adapt.f90:95-169) on the leaf-depth description of the tree.
//
// Edge flags: refine (initially false) and coarsen (initially true), shared by
// the two cells of an edge (refine merges with OR, coarsen with AND,
// Conformity.f90:1319-1331). Per cell: the hypotenuse never coarsens; flag 1
// marks the hypotenuse for refinement; flag 0 keeps both legs. Integrity, to a
// fixpoint over the mesh: a refined leg refines the hypotenuse; a cell coarsens
// only if its hypotenuse is not refined, both legs may coarsen and one leg is
// the edge it shares with its sibling, and it sets both legs' coarsen flag to
// that decision. A refined cell is bisected (the hypotenuse split); a child
// whose hypotenuse (one of the parent's legs) is marked is bisected again. Two
// siblings that both coarsen merge into their parent.
// State transfer of order 0 (src/Samoa/Tools_lagrange_basis.f90:139-220):
// split copies the cell's values to the children, merge averages h, hu, hv and b
// of the two siblings with 0.5 * (q1 + q2). The bathymetry of refined cells is
// copied; a host that samples b from data (get_bathymetry_at_element) replaces it.
#include "swe_internal.h"

#include <cstring>
#include <vector>

namespace swe {

int mesh_adapt(int64_t n, const int8_t* depth, const int8_t* flags, const double* const in[4], AdaptResult& out) {
    if (n < 2 || !depth || !flags) return set_error(SWE_E_INVALID, "bad mesh or flags");
    BuiltMesh m;
    int rc = build_mesh(n, depth, 0, kWantLegs, m);
    if (rc) return rc;
    const int64_t ne = m.ne, nb = m.nb;
    // edge ids: inner edges 0..ne-1, boundary edges ne..ne+nb-1
    std::vector<int64_t> slot((size_t)(3 * n), -1);
    for (int64_t e = 0; e < ne; ++e)
        for (int s = 0; s < 2; ++s) slot[(size_t)(3 * m.ec[(size_t)(2 * e + s)] + m.el[(size_t)(2 * e + s)] - 1)] = e;
    for (int64_t j = 0; j < nb; ++j) slot[(size_t)(3 * m.bc[(size_t)j] + m.bl[(size_t)j] - 1)] = ne + j;
    // per cell: hypotenuse, leg (x0, x1) = the first child's hypotenuse, leg (x1, x2)
    std::vector<int64_t> eh((size_t)n), ea((size_t)n), eb((size_t)n);
    for (int64_t k = 0; k < n; ++k) {
        const int la = m.leg[(size_t)k];  // local index of the leg (x0, x1)
        eh[(size_t)k] = slot[(size_t)(3 * k + 1)];
        ea[(size_t)k] = slot[(size_t)(3 * k + la)];
        eb[(size_t)k] = slot[(size_t)(3 * k + 2 - la)];
        if (eh[(size_t)k] < 0 || ea[(size_t)k] < 0 || eb[(size_t)k] < 0)
            return set_error(SWE_E_INVALID, "adapt: cell %lld has an unassigned edge", (long long)k);
        if (flags[k] < -1 || flags[k] > 1)
            return set_error(SWE_E_INVALID, "adapt: cell %lld: flag %d (expected -1, 0, 1)", (long long)k, flags[k]);
    }
    const size_t nt = (size_t)(ne + nb);
    std::vector<uint8_t> refine(nt, 0), coarsen(nt, 1), remove(nt, 0);
    for (int64_t e = 0; e < ne; ++e) {
        const int64_t a = m.ec[(size_t)(2 * e)], b = m.ec[(size_t)(2 * e + 1)];
        remove[(size_t)e] = m.parent[(size_t)a] >= 0 && m.parent[(size_t)a] == m.parent[(size_t)b];
    }
    for (int64_t k = 0; k < n; ++k) {
        coarsen[(size_t)eh[(size_t)k]] = 0;
        if (flags[k] == 1) refine[(size_t)eh[(size_t)k]] = 1;
        if (flags[k] == 0) coarsen[(size_t)ea[(size_t)k]] = coarsen[(size_t)eb[(size_t)k]] = 0;
    }
    // integrity to a fixpoint (refine only turns on, coarsen only turns off)
    for (bool changed = true; changed;) {
        changed = false;
        for (int64_t k = 0; k < n; ++k) {
            const size_t h = (size_t)eh[(size_t)k], a = (size_t)ea[(size_t)k], b = (size_t)eb[(size_t)k];
            if (!refine[h] && (refine[a] || refine[b])) {
                refine[h] = 1;
                changed = true;
            }
            const bool cc = !refine[h] && coarsen[a] && coarsen[b] && (remove[a] || remove[b]);
            if (!cc && (coarsen[a] || coarsen[b])) {
                coarsen[a] = coarsen[b] = 0;
                changed = true;
            }
        }
    }
    // new leaf sequence and state transfer
    out.depth.clear();
    out.source.clear();
    out.reserve_hint(n);
    for (int64_t k = 0; k < n; ++k) {
        const int d = depth[k];
        const size_t h = (size_t)eh[(size_t)k], a = (size_t)ea[(size_t)k], b = (size_t)eb[(size_t)k];
        if (refine[h]) {
            if (d + (refine[a] || refine[b] ? 2 : 1) > kMaxDepth)
                return set_error(SWE_E_INVALID, "adapt: cell %lld would exceed depth %d", (long long)k, kMaxDepth);
            for (int child = 0; child < 2; ++child) {
                const bool again = child == 0 ? refine[a] : refine[b];
                for (int q = 0; q < (again ? 2 : 1); ++q) {
                    out.depth.push_back((int8_t)(d + (again ? 2 : 1)));
                    out.source.push_back({k, -1});
                }
            }
            continue;
        }
        const bool cc = coarsen[a] && coarsen[b] && (remove[a] || remove[b]);
        if (cc && k + 1 < n && m.parent[(size_t)k] >= 0 && m.parent[(size_t)k] == m.parent[(size_t)(k + 1)]) {
            out.depth.push_back((int8_t)(d - 1));
            out.source.push_back({k, k + 1});
            ++k;  // the sibling merges into the same parent
            continue;
        }
        out.depth.push_back((int8_t)d);
        out.source.push_back({k, -1});
    }
    out.n = (int64_t)out.depth.size();
    for (int q = 0; q < 4; ++q) {
        out.state[q].clear();
        if (!in[q]) continue;
        out.state[q].resize((size_t)out.n);
        for (int64_t i = 0; i < out.n; ++i) {
            const auto& s = out.source[(size_t)i];
            out.state[q][(size_t)i] = s.second < 0 ? in[q][s.first] : 0.5 * (in[q][s.first] + in[q][s.second]);
        }
    }
    return SWE_OK;
}

}  // namespace swe

extern "C" {

int swe_mesh_build(int64_t n_cells, const int8_t* depth, int64_t* n_edges, int64_t* n_bnd, int8_t* plotter_out,
                   int64_t* edge_cells, int8_t* edge_local, int64_t* bnd_cell, int8_t* bnd_local, double* centroids,
                   double* vertices) {
    using namespace swe;
    if (!depth) return set_error(SWE_E_INVALID, "null depth array");
    const bool any = plotter_out || edge_cells || edge_local || bnd_cell || bnd_local || centroids || vertices;
    if (any && (!plotter_out || !edge_cells || !edge_local || !bnd_cell || !bnd_local))
        return set_error(SWE_E_INVALID, "mesh outputs must all be given (centroids, vertices optional)");
    BuiltMesh m;
    int rc = build_mesh(n_cells, depth, 0, (centroids || vertices) ? kWantVertices : 0, m);
    if (rc) return rc;
    if (n_edges) *n_edges = m.ne;
    if (n_bnd) *n_bnd = m.nb;
    if (!any) return SWE_OK;
    return export_mesh(m, nullptr, plotter_out, edge_cells, edge_local, bnd_cell, bnd_local, centroids, vertices);
}

int swe_mesh_adapt(int64_t n_cells, const int8_t* depth, const int8_t* flags, const double* h, const double* hu,
                   const double* hv, const double* b, int64_t capacity, int64_t* n_out, int8_t* depth_out,
                   int64_t* source_out, double* h_out, double* hu_out, double* hv_out, double* b_out) {
    using namespace swe;
    if (!n_out) return set_error(SWE_E_INVALID, "null n_out");
    const double* in[4] = {h, hu, hv, b};
    double* outp[4] = {h_out, hu_out, hv_out, b_out};
    for (int q = 0; q < 4; ++q)
        if (outp[q] && !in[q]) return set_error(SWE_E_INVALID, "state output %d without its input", q);
    AdaptResult r;
    int rc = mesh_adapt(n_cells, depth, flags, in, r);
    if (rc) return rc;
    *n_out = r.n;
    if (!depth_out) return SWE_OK;
    if (capacity < r.n)
        return set_error(SWE_E_INVALID, "adapt: %lld cells do not fit capacity %lld", (long long)r.n,
                         (long long)capacity);
    std::memcpy(depth_out, r.depth.data(), (size_t)r.n);
    if (source_out)
        for (int64_t i = 0; i < r.n; ++i) source_out[i] = r.source[(size_t)i].first;
    for (int q = 0; q < 4; ++q)
        if (outp[q]) std::memcpy(outp[q], r.state[q].data(), sizeof(double) * (size_t)r.n);
    return SWE_OK;
}

}  // extern "C"
