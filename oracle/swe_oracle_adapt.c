/*
 * ORACLE — test infrastructure only. Nothing in the product path may call this file.
 *
 * A plain-C restatement of one adaption step of sam(oa)^2's SWE scenario (the
 * remesh between two time steps) and of its bathymetry sampling, used by tests/
 * as the reference the product's host adaptivity is compared with. What it restates (paths
 * relative to the meistero/Samoa source tree):
 *   - the conformity traversal: edge flags refine (initially false), coarsen
 *     (initially true) and remove, set per cell by mark_edges and
 *     mark_edges_integrity (src/Conformity/Conformity.f90:1244-1317), merged
 *     across each edge by edge_merge_op_integrity (:1319-1331), repeated until
 *     both copies of every edge agree (conformity_check and
 *     update_conformity_traversal, :172-212,251-314);
 *   - the remove flag: set on the edge two children of one parent share
 *     (write_dest_element, src/SFC_generic_adaptive_traversal.f90:1177-1203);
 *   - transfer_op, refine_op and coarsen_op (src/SWE/SWE_adapt.f90:95-169) with
 *     the order-0 basis (split copies, merge averages 0.5 * (q1 + q2),
 *     src/Samoa/Tools_lagrange_basis.f90:139-210);
 *   - get_bathymetry_at_element with _ADAPT_INTEGRATE and
 *     refine_2D_recursive (src/SWE/SWE_initialize.f90:105-147): the mean of the
 *     bathymetry over 2^min(16, max_depth - depth) sub-triangles, sampled at
 *     each sub-triangle's centroid (x1 + x2 + x3) / 3 and mapped to world
 *     coordinates scaling * x + offset (get_bathymetry_at_position, :149-183;
 *     the synthetic bathymetry functions stand in for the ASAGI data).
 *
 * Independent of the product's adaptivity code by construction: the tree is
 * rebuilt here from the leaf depths with exact integer vertex coordinates, an
 * edge is found by the exact midpoint of its two end points (unique in a
 * conforming triangulation), the flags live on each cell's own copy of an edge
 * and are merged in passes as the reference's traversals do, not on a shared
 * edge record.
 *
 * Left and right leg: mark_edges clears the coarsen flag of the left leg only
 * for refinement 0, and mark_edges_integrity then gives both legs the same
 * coarsen flag, computed from both, so which leg is called left does not change
 * the result; the leg through the cell's first vertex is used.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORA_MAX_DEPTH 60
#define ORA_UNIT ((int64_t)1 << 31)      /* the unit square's side in integer coordinates */

/* A leaf: its vertices (x1, x2, x3) in integer coordinates, x2 the right angle,
 * hypotenuse x1-x3 (the vertex order of refine_2D_recursive). */
typedef struct {
    int64_t v[3][2];
    int64_t parent;      /* id of the parent node; roots: -1, -2 */
    int depth;
} ora_leaf;

typedef struct {
    ora_leaf* leaves;
    int64_t n, cap;
    int64_t next_node;
    const int8_t* depths;
} ora_tree;

/* The leaves of the tree whose leaf depths in traversal order are `depths`: a
 * cell is bisected (children (x1, m, x2) then (x2, m, x3), m the midpoint of the
 * hypotenuse) while it is shallower than the next leaf. */
static int ora_tree_rec(ora_tree* T, const int64_t v[3][2], int depth, int64_t parent)
{
    if (T->n >= T->cap) return -1;
    const int target = T->depths[T->n];
    if (depth == target) {
        ora_leaf* L = &T->leaves[T->n++];
        memcpy(L->v, v, sizeof(L->v));
        L->parent = parent;
        L->depth = depth;
        return 0;
    }
    if (depth > target || target > ORA_MAX_DEPTH) return -2;
    const int64_t id = T->next_node++;
    const int64_t m[2] = { (v[0][0] + v[2][0]) / 2, (v[0][1] + v[2][1]) / 2 };
    const int64_t a[3][2] = { { v[0][0], v[0][1] }, { m[0], m[1] }, { v[1][0], v[1][1] } };
    const int64_t b[3][2] = { { v[1][0], v[1][1] }, { m[0], m[1] }, { v[2][0], v[2][1] } };
    int rc = ora_tree_rec(T, a, depth + 1, id);
    if (rc) return rc;
    return ora_tree_rec(T, b, depth + 1, id);
}

static int ora_tree_build(ora_tree* T, int64_t n, const int8_t* depths)
{
    T->leaves = (ora_leaf*)malloc(sizeof(ora_leaf) * (size_t)(n > 0 ? n : 1));
    T->n = 0;
    T->cap = n;
    T->next_node = 0;
    T->depths = depths;
    const int64_t U = ORA_UNIT;
    const int64_t r1[3][2] = { { 0, 0 }, { U, 0 }, { U, U } };
    const int64_t r2[3][2] = { { U, U }, { 0, U }, { 0, 0 } };
    int rc = n >= 2 ? ora_tree_rec(T, r1, 0, -1) : -3;
    if (!rc) rc = ora_tree_rec(T, r2, 0, -2);
    if (!rc && T->n != n) rc = -3;
    return rc;
}

/* ---- bathymetry ---------------------------------------------------------- */

/* spec: {kind, p0, p1, scaling, offset_x, offset_y, max_depth};
 * kind 0: constant p0; kind 1: parabolic bowl -p0 * (1 - r^2 / p1^2). */
typedef struct {
    int kind;
    double p0, p1, scaling, ox, oy;
    int max_depth;
} ora_bath;

static double ora_bath_at(const ora_bath* B, const double x[2])
{
    /* get_bathymetry_at_position: xs = cfg%scaling * x + cfg%offset */
    const double xs = B->scaling * x[0] + B->ox;
    const double ys = B->scaling * x[1] + B->oy;
    if (B->kind == 1) {
        const double r2 = xs * xs + ys * ys;
        return -B->p0 * (1.0 - r2 / (B->p1 * B->p1));
    }
    return B->p0;
}

/* refine_2D_recursive (src/SWE/SWE_initialize.f90:105-117) */
static double ora_refine_2d(const ora_bath* B, const double x1[2], const double x2[2], const double x3[2],
                            int depth)
{
    if (depth > 0) {
        const double m[2] = { 0.5 * (x1[0] + x3[0]), 0.5 * (x1[1] + x3[1]) };
        return 0.5 * (ora_refine_2d(B, x1, m, x2, depth - 1) + ora_refine_2d(B, x2, m, x3, depth - 1));
    }
    const double c[2] = { (x1[0] + x2[0] + x3[0]) / 3.0, (x1[1] + x2[1] + x3[1]) / 3.0 };
    return ora_bath_at(B, c);
}

/* get_bathymetry_at_element with _ADAPT_INTEGRATE (:119-147, without ASAGI) */
static double ora_bath_element(const ora_bath* B, const int64_t v[3][2], int depth)
{
    int dd = B->max_depth - depth;
    if (dd > 16) dd = 16;
    const double s = 1.0 / (double)ORA_UNIT;  /* a power of two: exact */
    const double x1[2] = { (double)v[0][0] * s, (double)v[0][1] * s };
    const double x2[2] = { (double)v[1][0] * s, (double)v[1][1] * s };
    const double x3[2] = { (double)v[2][0] * s, (double)v[2][1] * s };
    return ora_refine_2d(B, x1, x2, x3, dd);
}

static void ora_bath_unpack(const double* spec, ora_bath* B)
{
    B->kind = (int)spec[0];
    B->p0 = spec[1];
    B->p1 = spec[2];
    B->scaling = spec[3];
    B->ox = spec[4];
    B->oy = spec[5];
    B->max_depth = (int)spec[6];
}

/*
 * b of every cell of the tree with the given leaf depths, as the initialisation
 * traversal sets it (Q%b = get_bathymetry_at_element, :102). spec as above.
 * Returns 0, or < 0 if the depths are not the leaves of a tree.
 */
int oracle_bathymetry_cells(int64_t n, const int8_t* depths, const double* spec, double* b_out)
{
    ora_tree T;
    int rc = ora_tree_build(&T, n, depths);
    if (!rc) {
        ora_bath B;
        ora_bath_unpack(spec, &B);
        for (int64_t k = 0; k < n; ++k) b_out[k] = ora_bath_element(&B, T.leaves[k].v, T.leaves[k].depth);
    }
    free(T.leaves);
    return rc;
}

/* ---- edges ----------------------------------------------------------------- */

/* Side 3k + r of leaf k: r = 0 hypotenuse (x1, x3), 1 leg (x1, x2) (the first
 * child's hypotenuse), 2 leg (x2, x3). */
static void ora_side_ends(const ora_leaf* L, int r, const int64_t** p, const int64_t** q)
{
    static const int ends[3][2] = { { 0, 2 }, { 0, 1 }, { 1, 2 } };
    *p = L->v[ends[r][0]];
    *q = L->v[ends[r][1]];
}

static int ora_on_border(const int64_t* p, const int64_t* q)
{
    const int64_t U = ORA_UNIT;
    return (p[0] == 0 && q[0] == 0) || (p[0] == U && q[0] == U) || (p[1] == 0 && q[1] == 0) ||
           (p[1] == U && q[1] == U);
}

typedef struct {
    int64_t mx, my;      /* twice the midpoint */
    int64_t side;        /* -1: empty */
} ora_slot;

static uint64_t ora_hash(int64_t a, int64_t b)
{
    uint64_t h = (uint64_t)a * 0x9E3779B97F4A7C15ull ^ ((uint64_t)b + 0x632BE59BD9B4E019ull);
    h ^= h >> 29;
    h *= 0xBF58476D1CE4E5B9ull;
    h ^= h >> 32;
    return h;
}

/* partner[s] = the other cell's side of the same edge, -1 on the domain
 * boundary. Returns 0, or -5 if an edge has no partner inside the domain or
 * more than one (the tree is not conforming). */
static int ora_match_edges(const ora_tree* T, int64_t* partner)
{
    const int64_t ns = 3 * T->n;
    size_t cap = 1;
    while (cap < (size_t)(2 * ns)) cap <<= 1;
    ora_slot* tab = (ora_slot*)malloc(sizeof(ora_slot) * cap);
    for (size_t i = 0; i < cap; ++i) tab[i].side = -1;
    int rc = 0;
    for (int64_t s = 0; s < ns && !rc; ++s) {
        partner[s] = -1;
        const int64_t *p, *q;
        ora_side_ends(&T->leaves[s / 3], (int)(s % 3), &p, &q);
        const int64_t mx = p[0] + q[0], my = p[1] + q[1];
        size_t i = (size_t)ora_hash(mx, my) & (cap - 1);
        while (tab[i].side >= 0 && (tab[i].mx != mx || tab[i].my != my)) i = (i + 1) & (cap - 1);
        if (tab[i].side < 0) {
            tab[i].mx = mx;
            tab[i].my = my;
            tab[i].side = s;
        } else {
            const int64_t o = tab[i].side;
            if (partner[o] >= 0) rc = -5;  /* a third cell on the same edge */
            partner[o] = s;
            partner[s] = o;
        }
    }
    for (int64_t s = 0; s < ns && !rc; ++s) {
        if (partner[s] >= 0) continue;
        const int64_t *p, *q;
        ora_side_ends(&T->leaves[s / 3], (int)(s % 3), &p, &q);
        if (!ora_on_border(p, q)) rc = -5;  /* a hanging node */
    }
    free(tab);
    return rc;
}

/* ---- one adaption step ------------------------------------------------------ */

enum { S_HYP = 0, S_LEG1 = 1, S_LEG2 = 2 };

/* mark_edges_integrity on one cell's own edge copies; returns 1 if a flag changed */
static int ora_integrity(uint8_t* refine, uint8_t* coarsen, const uint8_t* remove, int64_t k)
{
    const int64_t h = 3 * k + S_HYP, l = 3 * k + S_LEG1, r = 3 * k + S_LEG2;
    const uint8_t rh = refine[h] | refine[l] | refine[r];
    const uint8_t c = !rh && coarsen[l] && coarsen[r] && (remove[l] || remove[r]);
    const int changed = rh != refine[h] || c != coarsen[l] || c != coarsen[r];
    refine[h] = rh;
    coarsen[l] = c;
    coarsen[r] = c;
    return changed;
}

/*
 * One adaption step of the tree with leaf depths depth[n] from the time step's
 * refinement flags (-1 coarsen, 0 keep, 1 refine; src/SWE/SWE_euler_timestep.f90:336-344).
 * state: h, hu, hv, b (any may be NULL, then its output is not written).
 * bath_spec: NULL keeps the parent's b on refined cells (order-0 split);
 * else {kind, p0, p1, scaling, offset_x, offset_y, max_depth}: refined cells
 * take get_bathymetry_at_element (refine_op, src/SWE/SWE_adapt.f90:132).
 * Outputs (capacity cap): depth_out, source_out (first source cell), state.
 * Returns the new cell count, or < 0: -1/-2/-3 not a tree, -4 bad flag or a
 * coarsening cell without its sibling, -5 not conforming, -6 capacity, -7 depth.
 */
int64_t oracle_adapt(int64_t n, const int8_t* depth, const int8_t* flags, const double* h, const double* hu,
                     const double* hv, const double* b, const double* bath_spec, int64_t cap, int8_t* depth_out,
                     int64_t* source_out, double* h_out, double* hu_out, double* hv_out, double* b_out)
{
    ora_tree T;
    int64_t rc = ora_tree_build(&T, n, depth);
    const int64_t ns = 3 * n;
    int64_t* partner = (int64_t*)malloc(sizeof(int64_t) * (size_t)(ns > 0 ? ns : 1));
    uint8_t* refine = (uint8_t*)calloc((size_t)(ns > 0 ? ns : 1), 1);
    uint8_t* coarsen = (uint8_t*)malloc((size_t)(ns > 0 ? ns : 1));
    uint8_t* remove = (uint8_t*)calloc((size_t)(ns > 0 ? ns : 1), 1);
    if (!rc) rc = ora_match_edges(&T, partner);
    for (int64_t k = 0; k < n && !rc; ++k)
        if (flags[k] < -1 || flags[k] > 1) rc = -4;
    if (!rc) {
        /* the first touch of every edge copy: refine false, coarsen true; the
         * remove flag on the edge between two children of one parent */
        for (int64_t s = 0; s < ns; ++s) {
            coarsen[s] = 1;
            const int64_t o = partner[s];
            remove[s] = o >= 0 && T.leaves[s / 3].parent == T.leaves[o / 3].parent;
        }
        /* mark_edges (Conformity.f90:1244-1268) and its integrity call */
        for (int64_t k = 0; k < n; ++k) {
            coarsen[3 * k + S_HYP] = 0;
            if (flags[k] == 0) coarsen[3 * k + S_LEG1] = 0;
            if (flags[k] == 1) refine[3 * k + S_HYP] = 1;
            ora_integrity(refine, coarsen, remove, k);
        }
        /* the update traversals: merge both copies of each edge
         * (edge_merge_op_integrity: refine OR, coarsen AND), then integrity per
         * cell, until no flag changes */
        for (int changed = 1; changed;) {
            changed = 0;
            for (int64_t s = 0; s < ns; ++s) {
                const int64_t o = partner[s];
                if (o < s) continue;  /* boundary (-1) or the pair's second copy */
                const uint8_t r = refine[s] | refine[o], c = coarsen[s] & coarsen[o];
                if (r != refine[s] || r != refine[o] || c != coarsen[s] || c != coarsen[o]) changed = 1;
                refine[s] = refine[o] = r;
                coarsen[s] = coarsen[o] = c;
            }
            for (int64_t k = 0; k < n; ++k) changed |= ora_integrity(refine, coarsen, remove, k);
        }
    }
    /* refine_op / coarsen_op / transfer_op */
    ora_bath B;
    if (bath_spec) ora_bath_unpack(bath_spec, &B);
    const double* in[4] = { h, hu, hv, b };
    double* out[4] = { h_out, hu_out, hv_out, b_out };
    int64_t m = 0;
    for (int64_t k = 0; k < n && !rc; ++k) {
        const ora_leaf* L = &T.leaves[k];
        const int64_t s = 3 * k;
        if (refine[s + S_HYP]) {
            /* children (x1, m, x2) and (x2, m, x3); a child whose hypotenuse (the
             * parent's leg) is refined is bisected once more */
            const int64_t (*v)[2] = L->v;
            const int64_t mid[2] = { (v[0][0] + v[2][0]) / 2, (v[0][1] + v[2][1]) / 2 };
            int64_t ch[2][3][2] = { { { v[0][0], v[0][1] }, { mid[0], mid[1] }, { v[1][0], v[1][1] } },
                                    { { v[1][0], v[1][1] }, { mid[0], mid[1] }, { v[2][0], v[2][1] } } };
            for (int c = 0; c < 2 && !rc; ++c) {
                const int again = refine[s + (c == 0 ? S_LEG1 : S_LEG2)];
                const int d = L->depth + 1 + again;
                if (d > ORA_MAX_DEPTH) { rc = -7; break; }
                int64_t g[2][3][2];
                int ng = 1;
                memcpy(g[0], ch[c], sizeof(g[0]));
                if (again) {
                    const int64_t (*w)[2] = ch[c];
                    const int64_t mm[2] = { (w[0][0] + w[2][0]) / 2, (w[0][1] + w[2][1]) / 2 };
                    const int64_t g0[3][2] = { { w[0][0], w[0][1] }, { mm[0], mm[1] }, { w[1][0], w[1][1] } };
                    const int64_t g1[3][2] = { { w[1][0], w[1][1] }, { mm[0], mm[1] }, { w[2][0], w[2][1] } };
                    memcpy(g[0], g0, sizeof(g0));
                    memcpy(g[1], g1, sizeof(g1));
                    ng = 2;
                }
                for (int j = 0; j < ng; ++j) {
                    if (m >= cap) { rc = -6; break; }
                    depth_out[m] = (int8_t)d;
                    if (source_out) source_out[m] = k;
                    for (int q = 0; q < 3; ++q)
                        if (in[q] && out[q]) out[q][m] = in[q][k];
                    if (in[3] && out[3]) out[3][m] = bath_spec ? ora_bath_element(&B, g[j], d) : in[3][k];
                    ++m;
                }
            }
            continue;
        }
        if (coarsen[s + S_LEG1]) {
            /* merge with the sibling, which the fixpoint makes the next leaf */
            if (k + 1 >= n || !coarsen[s + 3 + S_LEG1] || refine[s + 3 + S_HYP] ||
                T.leaves[k + 1].parent != L->parent || T.leaves[k + 1].depth != L->depth) {
                rc = -4;
                break;
            }
            if (m >= cap) { rc = -6; break; }
            depth_out[m] = (int8_t)(L->depth - 1);
            if (source_out) source_out[m] = k;
            for (int q = 0; q < 4; ++q)
                if (in[q] && out[q]) out[q][m] = 0.5 * (in[q][k] + in[q][k + 1]);
            ++m;
            ++k;
            continue;
        }
        if (m >= cap) { rc = -6; break; }
        depth_out[m] = (int8_t)L->depth;
        if (source_out) source_out[m] = k;
        for (int q = 0; q < 4; ++q)
            if (in[q] && out[q]) out[q][m] = in[q][k];
        ++m;
    }
    free(partner);
    free(refine);
    free(coarsen);
    free(remove);
    free(T.leaves);
    return rc ? rc : m;
}
