/*
 * ORACLE — test infrastructure only. Nothing in the product path may call this file.
 *
 * A plain-C, strict-IEEE (no FMA contraction, no fast-math) restatement of the
 * sam(oa)^2 shallow-water (SWE) explicit Euler time step, used by tests/, by
 * __graft_entry__.smoke() and by bench.py's CPU-baseline leg, as the reference that results are compared with.
 *
 * What it restates (paths are relative to the meistero/Samoa source tree):
 *   - Sierpinski mesh generation and cell types ........ src/SFC_node_traversal.f90:85-292,
 *                                                        src/SFC_data_types.f90:370-507
 *   - geometry tables (volumes, edge lengths, normals) . src/SFC_data_types.f90:509-700
 *   - the static stack/stream traversal semantics ....... src/Tools_adaptive_traversal.f90:177-206,472-742,
 *     (which edge is first touched, update order)        src/SFC_generic_traversal_ringbuffer.f90:252-589
 *   - GeoClaw Riemann solvers (FP64) .................... src/geoclaw/c_bind_riemannsolvers.f90:16-176,
 *                                                        src/geoclaw/riemannsolvers.f:2-258,446-500,507-618
 *   - Lax-Friedrichs fluxes ............................. src/SWE/SWE_euler_timestep.f90:359-446
 *   - edge flux, boundary op, cell update, dt ........... src/SWE/SWE_euler_timestep.f90:89-140,196-355,449-481
 *
 * Parity status: the reference is Fortran and no Fortran compiler exists where
 * this was written, so this restatement could not be executed against the
 * reference itself; the reference ships no golden vectors for this path.
 * PARITY UNPINNED at the reference-test level. The anchors are analytic
 * invariants (lake at rest, mass balance, mirror symmetry) checked in tests/.
 *
 * Expression evaluation order follows Fortran's left-to-right rule for
 * operators of equal precedence; "dot_product"/"matmul" are restated as a
 * sum that starts from +0.0, which is what an inlined Fortran intrinsic does.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <float.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define OR_G 9.80665                      /* src/SWE/SWE_data_types.f90:34 */
#define OR_MAX_DEPTH 60                   /* bit_size(int64) - 4, src/SFC_data_types.f90:77 */

/* solver ids (GeoClaw numbering for the GeoClaw family, src/geoclaw/c_bind_riemannsolvers.f90:4-6) */
enum { OR_FWAVE = 1, OR_AUG_RIEMANN = 3, OR_LF = 10, OR_LF_BATH = 11, OR_LLF = 12, OR_LLF_BATH = 13 };
/* boundary conditions: OUTFLOW is the active one, SLIP/NOSLIP are the commented variants
 * at src/SWE/SWE_euler_timestep.f90:241-248 */
enum { OR_BC_OUTFLOW = 0, OR_BC_SLIP = 1, OR_BC_NOSLIP = 2 };

/* edge types and turtle types, src/SFC_data_types.f90:39-66 */
enum { T_K = 1, T_V = 2, T_H = 3 };
enum { E_OLD = 0, E_NEW = 1, E_OLD_BND = 2, E_NEW_BND = 3 };
enum { C_RED = -1, C_GREEN = 0 };

static double dmin_(double a, double b) { return (a < b) ? a : b; }
static double dmax_(double a, double b) { return (a > b) ? a : b; }

/* ------------------------------------------------------------------------- */
/* Geometry tables                                                             */
/* ------------------------------------------------------------------------- */

/* sqrt(0.5)**i is a Fortran PARAMETER (src/SFC_data_types.f90:535,557,584): the
 * compiler folds it as the correctly rounded power of the double fl(sqrt(0.5)).
 * Restated with exact big-integer arithmetic: x = m * 2^-53, x^i = m^i * 2^-53i,
 * rounded to 53 bits, half to even. */
static double or_pow_exact(double x, int i)
{
    if (i == 0) return 1.0;
    if (i < 0) return 1.0 / or_pow_exact(x, -i);      /* only i = -1 is used: one rounding */
    int e;
    double f = frexp(x, &e);                           /* x = f * 2^e, f in [0.5,1) */
    uint64_t m = (uint64_t)ldexp(f, 53);               /* x = m * 2^(e-53) */
    uint64_t limb[64];
    int n = 1;
    limb[0] = 1;
    for (int k = 0; k < i; ++k) {
        unsigned __int128 carry = 0;
        for (int j = 0; j < n; ++j) {
            unsigned __int128 p = (unsigned __int128)limb[j] * m + carry;
            limb[j] = (uint64_t)p;
            carry = p >> 64;
        }
        if (carry) limb[n++] = (uint64_t)carry;
    }
    int top = 63;
    while (!((limb[n - 1] >> top) & 1)) --top;
    int64_t bitlen = (int64_t)(n - 1) * 64 + top + 1;
    int64_t shift = bitlen - 53;                       /* keep the top 53 bits */
    uint64_t q = 0;
    for (int64_t b = bitlen - 1; b >= shift; --b)
        q = (q << 1) | ((limb[b / 64] >> (b % 64)) & 1);
    int round_bit = shift >= 1 ? (int)((limb[(shift - 1) / 64] >> ((shift - 1) % 64)) & 1) : 0;
    int sticky = 0;
    for (int64_t b = shift - 2; b >= 0 && !sticky; --b)
        if ((limb[b / 64] >> (b % 64)) & 1) sticky = 1;
    if (round_bit && (sticky || (q & 1))) q += 1;
    return ldexp((double)q, (int)(shift + (int64_t)i * (e - 53)));
}

static double g_leg[OR_MAX_DEPTH + 2];    /* g_leg[i+1] = sqrt(0.5)**i, i = -1..60 */
static double g_vol[OR_MAX_DEPTH + 1];    /* 0.5**(i+1), src/SFC_data_types.f90:524 */
static double g_normal[17][3][2];          /* [plotter+8][edge index-1][xy], src/SFC_data_types.f90:619-700 */
static int g_tables_ready = 0;

static void or_init_tables(void)
{
    if (g_tables_ready) return;
    double s = sqrt(0.5);
    for (int i = -1; i <= OR_MAX_DEPTH; ++i) g_leg[i + 1] = or_pow_exact(s, i);
    for (int i = 0; i <= OR_MAX_DEPTH; ++i) g_vol[i] = ldexp(1.0, -(i + 1));

    const double PI = 4.0 * atan(1.0);
    for (int p = -8; p <= 8; ++p) {
        if (p == 0) continue;
        double ang = PI / 4.0 * (double)abs(p);
        double J[2][2];                                 /* J[row][col] */
        if (p > 0) { J[0][0] = cos(ang); J[1][0] = sin(ang); J[0][1] = -sin(ang); J[1][1] = cos(ang); }
        else       { J[0][0] = -sin(ang); J[1][0] = cos(ang); J[0][1] = cos(ang); J[1][1] = sin(ang); }
        for (int r = 0; r < 2; ++r)
            for (int c = 0; c < 2; ++c) J[r][c] = trunc(1.5 * J[r][c]);
        double det = J[0][0] * J[1][1] - J[0][1] * J[1][0];
        double Ji[2][2];
        double rdet = 1.0 / det;
        Ji[0][0] = rdet * J[1][1]; Ji[1][0] = rdet * -J[1][0];
        Ji[0][1] = rdet * -J[0][1]; Ji[1][1] = rdet * J[0][0];
        const double ref[3][2] = { { -1.0, 0.0 }, { 1.0, 1.0 }, { 0.0, -1.0 } };
        for (int e = 0; e < 3; ++e) {
            double nv[2];
            for (int j = 0; j < 2; ++j) {                /* matmul(row vector, Jinv) */
                double acc = 0.0;
                acc = acc + ref[e][0] * Ji[0][j];
                acc = acc + ref[e][1] * Ji[1][j];
                nv[j] = acc;
            }
            double d = 0.0;
            d = d + nv[0] * nv[0];
            d = d + nv[1] * nv[1];
            double inv = 1.0 / sqrt(d);
            g_normal[p + 8][e][0] = inv * nv[0];
            g_normal[p + 8][e][1] = inv * nv[1];
        }
    }
    g_tables_ready = 1;
}

/* exported for tests: leg size sqrt(0.5)**i for i in -1..60, volume, normals */
double oracle_leg_size(int i) { or_init_tables(); return g_leg[i + 1]; }
double oracle_cell_volume(int i) { or_init_tables(); return g_vol[i]; }
void oracle_normal(int plotter, int edge_index, double* out)
{
    or_init_tables();
    out[0] = g_normal[plotter + 8][edge_index - 1][0];
    out[1] = g_normal[plotter + 8][edge_index - 1][1];
}

/* ------------------------------------------------------------------------- */
/* Cells and the Sierpinski mesh                                              */
/* ------------------------------------------------------------------------- */

typedef struct {
    int8_t entity;        /* i_entity_types */
    int8_t depth;
    int8_t plotter;
    int8_t turtle;
    int8_t color;         /* i_color_edge_color, RED = -1 / GREEN = 0 */
} or_cell;

/* get_edge_types, src/SFC_data_types.f90:402-414 */
static void cell_edge_types(const or_cell* c, int* prev, int* color, int* next)
{
    *prev = E_OLD | (((c->entity >> 3) & 1) << 1);
    *next = E_NEW | (((c->entity >> 2) & 1) << 1);
    *color = c->entity & 3;
}

/* set_edge_types, src/SFC_data_types.f90:440-450 */
static void cell_set_edge_types(or_cell* c, int prev, int color, int next)
{
    int e = 0;
    e |= ((prev >> 1) & 1) << 3;
    e |= ((next >> 1) & 1) << 2;
    e |= color & 3;
    c->entity = (int8_t)e;
}

/* get_edge_indices, src/SFC_data_types.f90:370-384: (previous, color, next) by turtle type */
static void cell_edge_indices(const or_cell* c, int* ip, int* ic, int* in)
{
    static const int tab[4][3] = { { 0, 0, 0 }, { 3, 1, 2 }, { 3, 2, 1 }, { 2, 3, 1 } };
    *ip = tab[c->turtle][0];
    *ic = tab[c->turtle][1];
    *in = tab[c->turtle][2];
}

/* cell_reverse, src/SFC_data_types.f90:473-486 */
static void cell_reverse(or_cell* c)
{
    unsigned v = (unsigned)(uint8_t)c->entity;
    unsigned low4 = v & 15u;
    low4 = ((low4 << 1) | (low4 >> 3)) & 15u;          /* ishftc(x, 1, 4) */
    v = (v & ~15u) | low4;
    unsigned low3 = v & 7u;
    low3 = ((low3 >> 1) | (low3 << 2)) & 7u;           /* ishftc(x, -1, 3) */
    v = (v & ~7u) | low3;
    v ^= 1u;
    c->entity = (int8_t)v;
    c->turtle = (int8_t)(4 - c->turtle);
    c->plotter = (int8_t)(-c->plotter);
}

/* create_child_cells, src/SFC_node_traversal.f90:252-292 */
static void create_child_cells(const or_cell* parent, or_cell* first, or_cell* second)
{
    static const int turtle_child[4][2] = { { 0, 0 }, { T_H, T_V }, { T_H, T_K }, { T_V, T_K } };
    static const int plotter_child[17] = { 3, 2, 1, 8, 7, 6, 5, 4, 0, -6, -7, -8, -1, -2, -3, -4, -5 };
    first->turtle = (int8_t)turtle_child[parent->turtle][0];
    second->turtle = (int8_t)turtle_child[parent->turtle][1];
    first->plotter = (int8_t)plotter_child[parent->plotter + 8];
    first->depth = (int8_t)(parent->depth + 1);
    second->plotter = (int8_t)(-plotter_child[-parent->plotter + 8]);
    second->depth = (int8_t)(parent->depth + 1);
    int p, c, n;
    cell_edge_types(parent, &p, &c, &n);
    int other = C_RED + C_GREEN - parent->color;
    switch (parent->turtle) {
    case T_K:
        cell_set_edge_types(first, p, n, E_NEW);
        cell_set_edge_types(second, E_OLD, c, n);
        first->color = (int8_t)other;
        second->color = parent->color;
        break;
    case T_V:
        cell_set_edge_types(first, p, c, E_NEW);
        cell_set_edge_types(second, E_OLD, c, n);
        first->color = parent->color;
        second->color = parent->color;
        break;
    default:
        cell_set_edge_types(first, p, c, E_NEW);
        cell_set_edge_types(second, E_OLD, p, n);
        first->color = parent->color;
        second->color = (int8_t)other;
        break;
    }
}

typedef struct {
    or_cell* cells;
    double* coords;       /* 6 per cell: node 1,2,3 (x,y) in the unit square */
    int64_t n;
    int64_t cap;
} or_mesh_builder;

static void sfc_recursion(or_mesh_builder* mb, const or_cell* cell, const double* co, int levels)
{
    if (levels == 0) {
        mb->cells[mb->n] = *cell;
        memcpy(mb->coords + 6 * mb->n, co, 6 * sizeof(double));
        mb->n++;
        return;
    }
    or_cell a, b;
    create_child_cells(cell, &a, &b);
    double mid[2] = { 0.5 * (co[0] + co[4]), 0.5 * (co[1] + co[5]) };
    double ca[6] = { co[0], co[1], mid[0], mid[1], co[2], co[3] };
    double cb[6] = { co[2], co[3], mid[0], mid[1], co[4], co[5] };
    sfc_recursion(mb, &a, ca, levels - 1);
    sfc_recursion(mb, &b, cb, levels - 1);
}

/*
 * Uniform Sierpinski mesh of the unit square at reference depth `depth`
 * (2^(depth+1) cells), in traversal order, init_section + sfc_init_recursion
 * (src/SFC_node_traversal.f90:85-145). Cells come out in the orientation of the
 * recursion ("forward"): the first step run on them traverses in this order.
 * Returns the number of cells; `cells_out` is int8[5*n] (entity, depth, plotter,
 * turtle, color) and `coords_out` double[6*n] (may be NULL).
 */
int64_t oracle_mesh_uniform(int depth, int8_t* cells_out, double* coords_out)
{
    int64_t n = (int64_t)1 << (depth + 1);
    or_mesh_builder mb;
    mb.cells = (or_cell*)malloc(sizeof(or_cell) * n);
    mb.coords = (double*)malloc(sizeof(double) * 6 * n);
    mb.n = 0;
    mb.cap = n;
    or_cell first = { 8 + 2 + E_OLD, 0, -2, T_K, C_RED };      /* FIRST_OLD_BND */
    or_cell second = { 4 + 2 + E_NEW, 0, -6, T_H, C_RED };     /* LAST_NEW_BND */
    const double c1[6] = { 0.0, 0.0, 1.0, 0.0, 1.0, 1.0 };
    const double c2[6] = { 1.0, 1.0, 0.0, 1.0, 0.0, 0.0 };
    sfc_recursion(&mb, &first, c1, depth);
    sfc_recursion(&mb, &second, c2, depth);
    for (int64_t i = 0; i < n; ++i) {
        cells_out[5 * i + 0] = mb.cells[i].entity;
        cells_out[5 * i + 1] = mb.cells[i].depth;
        cells_out[5 * i + 2] = mb.cells[i].plotter;
        cells_out[5 * i + 3] = mb.cells[i].turtle;
        cells_out[5 * i + 4] = mb.cells[i].color;
    }
    if (coords_out) memcpy(coords_out, mb.coords, sizeof(double) * 6 * n);
    free(mb.cells);
    free(mb.coords);
    return n;
}

/* The same recursion over a tree given by its leaf depths in traversal order
 * (an adaptive conforming mesh): a cell is bisected while it is shallower than
 * the next leaf's depth. */
static int sfc_recursion_depths(or_mesh_builder* mb, const or_cell* cell, const double* co, const int8_t* depths)
{
    if (mb->n >= mb->cap) return -1;
    const int target = depths[mb->n];
    if (cell->depth == target) {
        mb->cells[mb->n] = *cell;
        memcpy(mb->coords + 6 * mb->n, co, 6 * sizeof(double));
        mb->n++;
        return 0;
    }
    if (cell->depth > target || target > OR_MAX_DEPTH) return -2;
    or_cell a, b;
    create_child_cells(cell, &a, &b);
    double mid[2] = { 0.5 * (co[0] + co[4]), 0.5 * (co[1] + co[5]) };
    double ca[6] = { co[0], co[1], mid[0], mid[1], co[2], co[3] };
    double cb[6] = { co[2], co[3], mid[0], mid[1], co[4], co[5] };
    int rc = sfc_recursion_depths(mb, &a, ca, depths);
    if (rc) return rc;
    return sfc_recursion_depths(mb, &b, cb, depths);
}

/*
 * Mesh of the tree whose n leaves, in traversal order, have the given depths
 * (init_section + the recursion of sfc_init_recursion applied to that tree).
 * Outputs as oracle_mesh_uniform. Returns n, or < 0 if the depths are not the
 * leaves of such a tree.
 */
int64_t oracle_mesh_from_depths(int64_t n, const int8_t* depths, int8_t* cells_out, double* coords_out)
{
    or_mesh_builder mb;
    mb.cells = (or_cell*)malloc(sizeof(or_cell) * (size_t)n);
    mb.coords = (double*)malloc(sizeof(double) * 6 * (size_t)n);
    mb.n = 0;
    mb.cap = n;
    or_cell first = { 8 + 2 + E_OLD, 0, -2, T_K, C_RED };      /* FIRST_OLD_BND */
    or_cell second = { 4 + 2 + E_NEW, 0, -6, T_H, C_RED };     /* LAST_NEW_BND */
    const double c1[6] = { 0.0, 0.0, 1.0, 0.0, 1.0, 1.0 };
    const double c2[6] = { 1.0, 1.0, 0.0, 1.0, 0.0, 0.0 };
    int rc = sfc_recursion_depths(&mb, &first, c1, depths);
    if (!rc) rc = sfc_recursion_depths(&mb, &second, c2, depths);
    if (!rc && mb.n != n) rc = -3;
    if (!rc) {
        for (int64_t i = 0; i < n; ++i) {
            cells_out[5 * i + 0] = mb.cells[i].entity;
            cells_out[5 * i + 1] = mb.cells[i].depth;
            cells_out[5 * i + 2] = mb.cells[i].plotter;
            cells_out[5 * i + 3] = mb.cells[i].turtle;
            cells_out[5 * i + 4] = mb.cells[i].color;
        }
        if (coords_out) memcpy(coords_out, mb.coords, sizeof(double) * 6 * (size_t)n);
    }
    free(mb.cells);
    free(mb.coords);
    return rc ? rc : n;
}

/* ------------------------------------------------------------------------- */
/* Static traversal: which edge a cell's local edge index refers to            */
/* ------------------------------------------------------------------------- */

/*
 * Walks the cells in the given order with red/green colour-edge stacks the way
 * the read_* hooks do (src/Tools_adaptive_traversal.f90:472-531):
 *   previous edge OLD  -> the crossed edge shared with the previous cell,
 *   colour edge NEW    -> a new inner edge pushed on stack[colour],
 *   colour edge OLD    -> popped from stack[colour],
 *   next edge NEW      -> a new crossed edge shared with the next cell,
 *   *_BND              -> a domain-boundary edge.
 * Inner edges are numbered in first-touch order (colour edge before next
 * edge, src/Tools_adaptive_traversal.f90:585-603, the numbering of
 * src/Generic/Generic_initialize.f90:205-213); boundary edges are numbered in
 * walk order (previous, colour, next).
 *
 * Outputs (cells indexed by position k in `order`):
 *   slot_edge[3*k + (i-1)] = inner edge id (>= 0) or -(boundary id) - 1
 *   edge_cells[2*e], edge_local[2*e]: first-touch cell position and its local
 *       index, then the second cell.
 *   bnd_cell[b], bnd_local[b].
 * Returns 0 or a negative error code (stack underflow / inconsistent types).
 */
static int or_walk_edges(const or_cell* cells, int64_t n, int64_t* slot_edge, int64_t* edge_cells,
                         int8_t* edge_local, int64_t* n_edges, int64_t* bnd_cell, int8_t* bnd_local,
                         int64_t* n_bnd)
{
    int64_t* stack[2];
    int64_t sp[2] = { 0, 0 };
    stack[0] = (int64_t*)malloc(sizeof(int64_t) * (size_t)(n + 4));
    stack[1] = (int64_t*)malloc(sizeof(int64_t) * (size_t)(n + 4));
    int64_t ne = 0, nb = 0, crossed = -1;
    int rc = 0;
    for (int64_t k = 0; k < n && rc == 0; ++k) {
        const or_cell* c = &cells[k];
        int tp, tc, tn, ip, ic, in;
        cell_edge_types(c, &tp, &tc, &tn);
        cell_edge_indices(c, &ip, &ic, &in);
        int s = c->color + 1;                              /* RED -> 0, GREEN -> 1 */
        /* previous */
        if (tp == E_OLD) {
            if (crossed < 0) { rc = -1; break; }
            slot_edge[3 * k + ip - 1] = crossed;
            edge_cells[2 * crossed + 1] = k;
            edge_local[2 * crossed + 1] = (int8_t)ip;
        } else {
            bnd_cell[nb] = k; bnd_local[nb] = (int8_t)ip;
            slot_edge[3 * k + ip - 1] = -nb - 1;
            nb++;
        }
        crossed = -1;
        /* colour */
        if (tc == E_OLD) {
            if (sp[s] == 0) { rc = -2; break; }
            int64_t e = stack[s][--sp[s]];
            slot_edge[3 * k + ic - 1] = e;
            edge_cells[2 * e + 1] = k;
            edge_local[2 * e + 1] = (int8_t)ic;
        } else if (tc == E_NEW) {
            int64_t e = ne++;
            stack[s][sp[s]++] = e;
            slot_edge[3 * k + ic - 1] = e;
            edge_cells[2 * e] = k;
            edge_local[2 * e] = (int8_t)ic;
        } else {
            bnd_cell[nb] = k; bnd_local[nb] = (int8_t)ic;
            slot_edge[3 * k + ic - 1] = -nb - 1;
            nb++;
        }
        /* next */
        if (tn == E_NEW) {
            int64_t e = ne++;
            slot_edge[3 * k + in - 1] = e;
            edge_cells[2 * e] = k;
            edge_local[2 * e] = (int8_t)in;
            crossed = e;
        } else {
            bnd_cell[nb] = k; bnd_local[nb] = (int8_t)in;
            slot_edge[3 * k + in - 1] = -nb - 1;
            nb++;
        }
    }
    if (rc == 0 && (sp[0] != 0 || sp[1] != 0 || crossed >= 0)) rc = -3;
    free(stack[0]);
    free(stack[1]);
    *n_edges = ne;
    *n_bnd = nb;
    return rc;
}

/*
 * Edge streams of a mesh in the C-ABI format (first cell, second cell, local
 * indices 1..3), for comparison with the product's own mesh builder.
 * cells: int8[5*n] as produced by oracle_mesh_uniform. Returns 0 or < 0.
 */
int oracle_mesh_edges(const int8_t* cells5, int64_t n, int64_t* edge_cells, int8_t* edge_local,
                      int64_t* n_edges, int64_t* bnd_cell, int8_t* bnd_local, int64_t* n_bnd)
{
    or_cell* cells = (or_cell*)malloc(sizeof(or_cell) * (size_t)n);
    for (int64_t i = 0; i < n; ++i) {
        cells[i].entity = cells5[5 * i]; cells[i].depth = cells5[5 * i + 1];
        cells[i].plotter = cells5[5 * i + 2]; cells[i].turtle = cells5[5 * i + 3];
        cells[i].color = cells5[5 * i + 4];
    }
    int64_t* slot = (int64_t*)malloc(sizeof(int64_t) * 3 * (size_t)n);
    int rc = or_walk_edges(cells, n, slot, edge_cells, edge_local, n_edges, bnd_cell, bnd_local, n_bnd);
    free(slot);
    free(cells);
    return rc;
}

/* ------------------------------------------------------------------------- */
/* GeoClaw Riemann solvers (double precision)                                  */
/* ------------------------------------------------------------------------- */

/* riemanntype, src/geoclaw/riemannsolvers.f:507-618 (maxiter = 1 at every call site) */
static void riemanntype(double hL, double hR, double uL, double uR, double* hm_out, double* s1m_out,
                        double* s2m_out, int* rare1, int* rare2, int maxiter, double drytol, double g)
{
    double hm, s1m, s2m, h0, F0, slope, gL, gR, dfdh, u1m, u2m;
    double h_min = dmin_(hR, hL);
    double h_max = dmax_(hR, hL);
    double delu = uR - uL;
    if (h_min <= drytol) {
        hm = 0.0;
        s1m = ((uR + uL) - 2.0 * sqrt(g * hR)) + 2.0 * sqrt(g * hL);
        s2m = ((uR + uL) - 2.0 * sqrt(g * hR)) + 2.0 * sqrt(g * hL);
        if (hL <= 0.0) { *rare2 = 1; *rare1 = 0; }
        else { *rare1 = 1; *rare2 = 0; }
    } else {
        double F_min = delu + 2.0 * (sqrt(g * h_min) - sqrt(g * h_max));
        double F_max = delu + (h_max - h_min) * sqrt(((0.5 * g) * (h_max + h_min)) / (h_max * h_min));
        if (F_min > 0.0) {
            double t = dmax_(0.0, -delu + 2.0 * (sqrt(g * hL) + sqrt(g * hR)));
            hm = (1.0 / (16.0 * g)) * (t * t);
            s1m = (uL + 2.0 * sqrt(g * hL)) - 3.0 * sqrt(g * hm);
            s2m = (uR - 2.0 * sqrt(g * hR)) + 3.0 * sqrt(g * hm);
            *rare1 = 1; *rare2 = 1;
        } else if (F_max <= 0.0) {
            h0 = h_max;
            for (int it = 0; it < maxiter; ++it) {
                gL = sqrt((0.5 * g) * (1.0 / h0 + 1.0 / hL));
                gR = sqrt((0.5 * g) * (1.0 / h0 + 1.0 / hR));
                F0 = (delu + (h0 - hL) * gL) + (h0 - hR) * gR;
                dfdh = ((gL - (g * (h0 - hL)) / ((4.0 * (h0 * h0)) * gL)) + gR)
                       - (g * (h0 - hR)) / ((4.0 * (h0 * h0)) * gR);
                slope = (2.0 * sqrt(h0)) * dfdh;
                double t = sqrt(h0) - F0 / slope;
                h0 = t * t;
            }
            hm = h0;
            u1m = uL - (hm - hL) * sqrt((0.5 * g) * (1.0 / hm + 1.0 / hL));
            u2m = uR + (hm - hR) * sqrt((0.5 * g) * (1.0 / hm + 1.0 / hR));
            s1m = u1m - sqrt(g * hm);
            s2m = u2m + sqrt(g * hm);
            *rare1 = 0; *rare2 = 0;
        } else {
            h0 = h_min;
            for (int it = 0; it < maxiter; ++it) {
                F0 = (delu + 2.0 * (sqrt(g * h0) - sqrt(g * h_max)))
                     + (h0 - h_min) * sqrt((0.5 * g) * (1.0 / h0 + 1.0 / h_min));
                slope = (F_max - F0) / (h_max - h_min);
                h0 = h0 - F0 / slope;
            }
            hm = h0;
            if (hL > hR) {
                s1m = (uL + 2.0 * sqrt(g * hL)) - 3.0 * sqrt(g * hm);
                s2m = (uL + 2.0 * sqrt(g * hL)) - sqrt(g * hm);
                *rare1 = 1; *rare2 = 0;
            } else {
                s2m = (uR - 2.0 * sqrt(g * hR)) + 3.0 * sqrt(g * hm);
                s1m = (uR - 2.0 * sqrt(g * hR)) + sqrt(g * hm);
                *rare2 = 1; *rare1 = 0;
            }
        }
    }
    *hm_out = hm; *s1m_out = s1m; *s2m_out = s2m;
}

/* riemann_fwave, src/geoclaw/riemannsolvers.f:446-500 */
static void riemann_fwave(double hL, double hR, double huL, double huR, double bL, double bR, double vL,
                          double vR, double delphi, double s1, double s2, double g, double sw[3],
                          double fw[3][3])
{
    double delhu = huR - huL;
    double delb = bR - bL;
    double deldelphi = -(((g * 0.5) * (hR + hL)) * delb);
    double delphidecomp = delphi - deldelphi;
    double beta1 = (s2 * delhu - delphidecomp) / (s2 - s1);
    double beta2 = (delphidecomp - s1 * delhu) / (s2 - s1);
    sw[0] = s1;
    sw[1] = 0.5 * (s1 + s2);
    sw[2] = s2;
    fw[0][0] = beta1; fw[1][0] = beta1 * s1; fw[2][0] = beta1 * vL;
    fw[0][2] = beta2; fw[1][2] = beta2 * s2; fw[2][2] = beta2 * vR;
    fw[0][1] = 0.0; fw[1][1] = 0.0;
    fw[2][1] = ((huR * vR - huL * vL) - fw[2][0]) - fw[2][2];
}

static double det3(const double A[3][3])
{
    double d1 = A[0][0] * (A[1][1] * A[2][2] - A[1][2] * A[2][1]);
    double d2 = A[0][1] * (A[1][0] * A[2][2] - A[1][2] * A[2][0]);
    double d3 = A[0][2] * (A[1][0] * A[2][1] - A[1][1] * A[2][0]);
    return (d1 - d2) + d3;
}

/* riemann_aug_JCP with maxiter = 1, src/geoclaw/riemannsolvers.f:2-258. The
 * entropy corrector is disabled in the source (rarecorrectortest = .false.),
 * and with one iteration the star-state update after the Cramer solve does
 * not reach the outputs. */
static void riemann_aug_jcp(double hL, double hR, double huL, double huR, double bL, double bR,
                            double uL, double uR, double vL, double vR, double delphi, double sE1,
                            double sE2, double drytol, double g, double sw[3], double fw[3][3])
{
    double lambda[3], r[3][3], A[3][3], del[3], beta[3];
    double delh = hR - hL;
    double delhu = huR - huL;
    double delb = bR - bL;
    double hm, s1m, s2m;
    int rare1, rare2;
    riemanntype(hL, hR, uL, uR, &hm, &s1m, &s2m, &rare1, &rare2, 1, drytol, g);
    lambda[0] = dmin_(sE1, s2m);
    lambda[2] = dmax_(sE2, s1m);
    sE1 = lambda[0];
    sE2 = lambda[2];
    double hstarHLL = dmax_((((huL - huR) + sE2 * hR) - sE1 * hL) / (sE2 - sE1), 0.0);
    lambda[1] = 0.5 * (lambda[0] + lambda[2]);
    if (fabs(lambda[1]) < 1e-20) lambda[1] = 0.0;
    for (int mw = 0; mw < 3; ++mw) { r[0][mw] = 1.0; r[1][mw] = lambda[mw]; r[2][mw] = lambda[mw] * lambda[mw]; }
    r[0][1] = 0.0; r[1][1] = 0.0; r[2][1] = 1.0;

    const double criticaltol = 1e-6;
    double hLstar = hL, hRstar = hR, uLstar = uL, uRstar = uR;
    double hbar = dmax_(0.5 * (hLstar + hRstar), 0.0);
    double su = uLstar + uRstar;
    double s1s2bar = 0.25 * (su * su) - g * hbar;
    double s1s2tilde = dmax_(0.0, uLstar * uRstar) - g * hbar;
    int sonic = 0;
    if (fabs(s1s2bar) <= criticaltol) sonic = 1;
    if (s1s2bar * s1s2tilde <= criticaltol) sonic = 1;
    if ((s1s2bar * sE1) * sE2 <= criticaltol) sonic = 1;
    if (dmin_(fabs(sE1), fabs(sE2)) < criticaltol) sonic = 1;
    if (sE1 < 0.0 && s1m > 0.0) sonic = 1;
    if (sE2 > 0.0 && s2m < 0.0) sonic = 1;
    if ((uL + sqrt(g * hL)) * (uR + sqrt(g * hR)) < 0.0) sonic = 1;
    if ((uL - sqrt(g * hL)) * (uR - sqrt(g * hR)) < 0.0) sonic = 1;

    double deldelh = sonic ? -delb : ((delb * g) * hbar) / s1s2bar;
    if (sE1 < -criticaltol && sE2 > criticaltol) {
        deldelh = dmin_(deldelh, (hstarHLL * (sE2 - sE1)) / sE2);
        deldelh = dmax_(deldelh, (hstarHLL * (sE2 - sE1)) / sE1);
    } else if (sE1 >= criticaltol) {
        deldelh = dmin_(deldelh, (hstarHLL * (sE2 - sE1)) / sE1);
        deldelh = dmax_(deldelh, -hL);
    } else if (sE2 <= -criticaltol) {
        deldelh = dmin_(deldelh, hR);
        deldelh = dmax_(deldelh, (hstarHLL * (sE2 - sE1)) / sE2);
    }
    double deldelphi = sonic ? -((g * hbar) * delb) : -((((delb * g) * hbar) * s1s2tilde) / s1s2bar);
    deldelphi = dmin_(deldelphi, g * dmax_(-(hLstar * delb), -(hRstar * delb)));
    deldelphi = dmax_(deldelphi, g * dmin_(-(hLstar * delb), -(hRstar * delb)));
    del[0] = delh - deldelh;
    del[1] = delhu;
    del[2] = delphi - deldelphi;
    double determinant = det3(r);
    for (int k = 0; k < 3; ++k) {
        for (int mw = 0; mw < 3; ++mw)
            for (int m = 0; m < 3; ++m) A[m][mw] = (mw == k) ? del[m] : r[m][mw];
        beta[k] = det3(A) / determinant;
    }
    for (int mw = 0; mw < 3; ++mw) {
        sw[mw] = lambda[mw];
        fw[0][mw] = beta[mw] * r[1][mw];
        fw[1][mw] = beta[mw] * r[2][mw];
        fw[2][mw] = beta[mw] * r[1][mw];
    }
    fw[2][0] = fw[2][0] * vL;
    fw[2][2] = fw[2][2] * vR;
    fw[2][1] = ((((hR * uR) * vR) - ((hL * uL) * vL)) - fw[2][0]) - fw[2][2];
}

/* c_bind_geoclaw_solver_dp, src/geoclaw/c_bind_riemannsolvers.f90:16-176 */
void oracle_geoclaw_solver(int solver, double hL, double hR, double huL, double huR, double hvL,
                           double hvR, double bL, double bR, double drytol, double g, double netL[3],
                           double netR[3], double* maxspeed)
{
    double sw[3] = { 0.0, 0.0, 0.0 };
    double fw[3][3] = { { 0.0, 0.0, 0.0 }, { 0.0, 0.0, 0.0 }, { 0.0, 0.0, 0.0 } };
    double wall[3] = { 1.0, 1.0, 1.0 };
    double uL, uR, vL, vR, hstar, s1m, s2m, hstartest;
    int rare1, rare2;
    *maxspeed = 0.0;
    netL[0] = netL[1] = netL[2] = 0.0;
    netR[0] = netR[1] = netR[2] = 0.0;
    if (hL <= drytol && hR <= drytol) return;
    if (hR > drytol) { uR = huR / hR; vR = hvR / hR; }
    else { hR = 0.0; huR = 0.0; hvR = 0.0; uR = 0.0; vR = 0.0; }
    if (hL > drytol) { uL = huL / hL; vL = hvL / hL; }
    else { hL = 0.0; huL = 0.0; hvL = 0.0; uL = 0.0; vL = 0.0; }
    if (hR <= drytol) {
        riemanntype(hL, hL, uL, -uL, &hstar, &s1m, &s2m, &rare1, &rare2, 1, drytol, g);
        hstartest = dmax_(hL, hstar);
        if (hstartest + bL < bR) {
            wall[1] = 0.0; wall[2] = 0.0;
            hR = hL; huR = -huL; bR = bL; uR = -uL; vR = vL;
        } else if (hL + bL < bR) {
            bR = hL + bL;
        }
    } else if (hL <= drytol) {
        riemanntype(hR, hR, -uR, uR, &hstar, &s1m, &s2m, &rare1, &rare2, 1, drytol, g);
        hstartest = dmax_(hR, hstar);
        if (hstartest + bR < bL) {
            wall[0] = 0.0; wall[1] = 0.0;
            hL = hR; huL = -huR; bL = bR; uL = -uR; vL = vR;
        } else if (hR + bR < bL) {
            bL = hR + bR;
        }
    }
    double delphi = ((((huR - huL) * (uL + uR)) - ((uL * uR) * (hR - hL)))
                     + (((0.5 * g) * (((bR + hR) - bL) - hL)) * (hR + hL)))
                    - (((0.5 * g) * (hR + hL)) * (bR - bL));
    double sqL = sqrt(g * hL), sqR = sqrt(g * hR);
    double sL = uL - sqL;
    double sR = uR + sqR;
    double uhat = (sqL * uL + sqR * uR) / (sqR + sqL);
    double chat = sqrt((g * 0.5) * (hR + hL));
    double sRoe1 = uhat - chat;
    double sRoe2 = uhat + chat;
    double sE1 = dmin_(sL, sRoe1);
    double sE2 = dmax_(sR, sRoe2);
    if (solver == OR_AUG_RIEMANN)
        riemann_aug_jcp(hL, hR, huL, huR, bL, bR, uL, uR, vL, vR, delphi, sE1, sE2, drytol, g, sw, fw);
    else
        riemann_fwave(hL, hR, huL, huR, bL, bR, vL, vR, delphi, sE1, sE2, g, sw, fw);
    for (int w = 0; w < 3; ++w) {
        if (wall[w] != 1.0) {
            sw[w] = sw[w] * wall[w];
            for (int e = 0; e < 3; ++e) fw[e][w] = fw[e][w] * wall[w];
        }
    }
    for (int e = 0; e < 3; ++e) {
        for (int w = 0; w < 3; ++w) {
            if (sw[w] < 0.0) netL[e] = netL[e] + fw[e][w];
            else if (sw[w] > 0.0) netR[e] = netR[e] + fw[e][w];
            else { netL[e] = netL[e] + 0.5 * fw[e][w]; netR[e] = netR[e] + 0.5 * fw[e][w]; }
        }
    }
    double m = fabs(sw[0]);
    if (fabs(sw[1]) > m) m = fabs(sw[1]);
    if (fabs(sw[2]) > m) m = fabs(sw[2]);
    *maxspeed = m;
}

/* ------------------------------------------------------------------------- */
/* Edge fluxes                                                                 */
/* ------------------------------------------------------------------------- */

typedef struct { double h, p1, p2, b; } or_state;
typedef struct { double h, p1, p2, s; } or_update;

/* compute_geoclaw_flux, src/SWE/SWE_euler_timestep.f90:449-481 */
static void geoclaw_flux(int solver, const double n[2], const or_state* QL, const or_state* QR,
                         double drytol, or_update* fL, or_update* fR)
{
    double T[2][2] = { { n[0], n[1] }, { -n[1], n[0] } };
    double pL[2], pR[2];
    for (int i = 0; i < 2; ++i) {
        double a = 0.0, b = 0.0;
        a = a + T[i][0] * QL->p1; a = a + T[i][1] * QL->p2;
        b = b + T[i][0] * QR->p1; b = b + T[i][1] * QR->p2;
        pL[i] = a; pR[i] = b;
    }
    double hL = QL->h - QL->b, hR = QR->h - QR->b;
    double netL[3], netR[3], ms;
    oracle_geoclaw_solver(solver, hL, hR, pL[0], pR[0], pL[1], pR[1], QL->b, QR->b, drytol, OR_G, netL, netR,
                          &ms);
    double a1 = 0.0, a2 = 0.0, b1 = 0.0, b2 = 0.0;
    a1 = a1 + netL[1] * T[0][0]; a1 = a1 + netL[2] * T[1][0];
    a2 = a2 + netL[1] * T[0][1]; a2 = a2 + netL[2] * T[1][1];
    b1 = b1 + netR[1] * T[0][0]; b1 = b1 + netR[2] * T[1][0];
    b2 = b2 + netR[1] * T[0][1]; b2 = b2 + netR[2] * T[1][1];
    fL->h = netL[0]; fL->p1 = a1; fL->p2 = a2; fL->s = ms;
    fR->h = netR[0]; fR->p1 = b1; fR->p2 = b2; fR->s = ms;
}

/* compute_lf_flux, src/SWE/SWE_euler_timestep.f90:359-446 */
static void lf_flux(int solver, const double n[2], const or_state* QL, const or_state* QR, double drytol,
                    or_update* fL, or_update* fR)
{
    const double g = OR_G;
    double vL, vR, hL, hR, alpha;
    if (solver == OR_LF_BATH || solver == OR_LLF_BATH) {
        if (QL->h - QL->b < drytol || QR->h - QR->b < drytol) {
            hL = 0.0; hR = 0.0; vL = 0.0; vR = 0.0;
            fL->s = 0.0; fR->s = 0.0;
            fL->h = 0.0; fR->h = 0.0;
            fL->p1 = 0.0; fL->p2 = 0.0; fR->p1 = 0.0; fR->p2 = 0.0;
            if (QL->h - QL->b < drytol && QR->h - QR->b < drytol) {
            } else if (QL->h - QL->b < drytol) {
                hR = dmax_(QR->h - QR->b, 0.0);
                double d = QR->h - QR->b;
                double t = 0.0; t = t + n[0] * (QR->p1 / d); t = t + n[1] * (QR->p2 / d);
                vR = t;
                fR->s = sqrt(g * hR) + fabs(vR);
                fR->p1 = (-((0.5 * vR) * QR->p1) - (((0.5 * g) * hR) * hR) * n[0]) + (0.5 * fR->s) * QR->p1;
                fR->p2 = (-((0.5 * vR) * QR->p2) - (((0.5 * g) * hR) * hR) * n[1]) + (0.5 * fR->s) * QR->p2;
            } else {
                hL = dmax_(QL->h - QL->b, 0.0);
                double d = QL->h - QL->b;
                double t = 0.0; t = t + n[0] * (QL->p1 / d); t = t + n[1] * (QL->p2 / d);
                vL = t;
                fL->s = sqrt(g * hL) + fabs(vL);
                fL->p1 = ((0.5 * vL) * QL->p1 + (((0.5 * g) * hL) * hL) * n[0]) + (0.5 * fL->s) * QL->p1;
                fL->p2 = ((0.5 * vL) * QL->p2 + (((0.5 * g) * hL) * hL) * n[1]) + (0.5 * fL->s) * QL->p2;
            }
            return;
        }
        hL = dmax_(QL->h - QL->b, 0.0);
        hR = dmax_(QR->h - QR->b, 0.0);
        double dL = QL->h - QL->b, dR = QR->h - QR->b;
        double t = 0.0; t = t + n[0] * (QL->p1 / dL); t = t + n[1] * (QL->p2 / dL); vL = t;
        t = 0.0; t = t + n[0] * (QR->p1 / dR); t = t + n[1] * (QR->p2 / dR); vR = t;
        fL->s = sqrt(g * hL) + fabs(vL);
        fR->s = sqrt(g * hR) + fabs(vR);
        alpha = (solver == OR_LLF_BATH) ? dmax_(fL->s, fR->s) : 100.0;
        fL->h = 0.5 * ((hL * vL + hR * vR) + alpha * (QL->h - QR->h));
        fR->h = -fL->h;
        double pr = (0.5 * g) * (hL * hL + hR * hR);
        fL->p1 = 0.5 * (((QL->p1 * vL + QR->p1 * vR) + pr * n[0]) + alpha * (QL->p1 - QR->p1));
        fL->p2 = 0.5 * (((QL->p2 * vL + QR->p2 * vR) + pr * n[1]) + alpha * (QL->p2 - QR->p2));
        fR->p1 = -fL->p1;
        fR->p2 = -fL->p2;
        double src = ((0.25 * g) * (hL + hR)) * (QR->b - QL->b);
        fL->p1 = fL->p1 + src * n[0];
        fL->p2 = fL->p2 + src * n[1];
        fR->p1 = fR->p1 + src * n[0];
        fR->p2 = fR->p2 + src * n[1];
    } else {
        const double b = 0.0;
        hL = dmax_(QL->h - b, 0.0);
        hR = dmax_(QR->h - b, 0.0);
        double dL = QL->h - b, dR = QR->h - b;
        double t = 0.0; t = t + n[0] * (QL->p1 / dL); t = t + n[1] * (QL->p2 / dL); vL = t;
        t = 0.0; t = t + n[0] * (QR->p1 / dR); t = t + n[1] * (QR->p2 / dR); vR = t;
        fL->s = sqrt(g * (QL->h - b)) + fabs(vL);
        fR->s = sqrt(g * (QR->h - b)) + fabs(vR);
        alpha = (solver == OR_LLF) ? dmax_(fL->s, fR->s) : 100.0;
        fL->h = 0.5 * ((vL * hL + vR * hR) + alpha * (QL->h - QR->h));
        fR->h = -fL->h;
        double sc = (vL * vL) * hL + (vR * vR) * hR;
        double pr = (0.5 * g) * (hL * hL + hR * hR);
        fL->p1 = 0.5 * ((sc + pr * n[0]) + alpha * (QL->p1 - QR->p1));
        fL->p2 = 0.5 * ((sc + pr * n[1]) + alpha * (QL->p2 - QR->p2));
        fR->p1 = -fL->p1;
        fR->p2 = -fL->p2;
    }
}

static void edge_flux(int solver, const double n[2], const or_state* QL, const or_state* QR, double drytol,
                      or_update* fL, or_update* fR)
{
    if (solver == OR_FWAVE || solver == OR_AUG_RIEMANN)
        geoclaw_flux(solver, n, QL, QR, drytol, fL, fR);
    else
        lf_flux(solver, n, QL, QR, drytol, fL, fR);
}

/* exported for solver-level tests: one edge, left/right states (h = surface, p, b) */
void oracle_edge_flux(int solver, const double* normal, const double* qL, const double* qR, double drytol,
                      double* upd_left, double* upd_right)
{
    or_state L = { qL[0], qL[1], qL[2], qL[3] }, R = { qR[0], qR[1], qR[2], qR[3] };
    or_update a, b;
    edge_flux(solver, normal, &L, &R, drytol, &a, &b);
    upd_left[0] = a.h; upd_left[1] = a.p1; upd_left[2] = a.p2; upd_left[3] = a.s;
    upd_right[0] = b.h; upd_right[1] = b.p1; upd_right[2] = b.p2; upd_right[3] = b.s;
}

/* bnd_skeleton_scalar_op, src/SWE/SWE_euler_timestep.f90:231-255 */
static void boundary_ghost(int bc, const double n[2], const or_state* Q, or_state* ghost)
{
    *ghost = *Q;
    if (bc == OR_BC_SLIP) {
        double d = 0.0;
        d = d + Q->p1 * n[0];
        d = d + Q->p2 * n[1];
        ghost->p1 = Q->p1 - d * n[0];
        ghost->p2 = Q->p2 - d * n[1];
    } else if (bc == OR_BC_NOSLIP) {
        ghost->p1 = -Q->p1;
        ghost->p2 = -Q->p2;
    }
}

/* ------------------------------------------------------------------------- */
/* The time step                                                               */
/* ------------------------------------------------------------------------- */

typedef struct {
    int solver, bc;
    double dry_tolerance, courant, scaling;
    int min_depth, max_depth;
    double max_time, output_time_step;
} or_params;

/* volume_op + cell_update_op, src/SWE/SWE_euler_timestep.f90:257-284,307-355.
 * upd[0..2] are the three edge updates in local edge index order. */
static void cell_update(const or_params* P, int depth, or_state* Q, const or_update upd[3], double dt,
                        double* dt_new, int8_t* flag, int64_t* n_refine)
{
    double volume = (P->scaling * P->scaling) * g_vol[depth];
    double len[3] = { P->scaling * g_leg[depth + 1], P->scaling * g_leg[depth], P->scaling * g_leg[depth + 1] };
    double dh = 0.0, dp1 = 0.0, dp2 = 0.0, ds = 0.0;
    for (int i = 0; i < 3; ++i) dh = dh + len[i] * upd[i].h;
    for (int i = 0; i < 3; ++i) dp1 = dp1 + len[i] * upd[i].p1;
    for (int i = 0; i < 3; ++i) dp2 = dp2 + len[i] * upd[i].p2;
    double thr = (5.0 * P->scaling) * g_leg[P->max_depth + 1];
    int8_t f = 0;
    double nrm = fabs(dh);
    if (depth < P->max_depth && nrm > thr) { f = 1; (*n_refine)++; }
    else if (depth > P->min_depth && nrm < thr / 8.0) f = -1;
    *flag = f;
    for (int i = 0; i < 3; ++i) ds = ds + len[i] * upd[i].s;
    double c = volume / ds;
    *dt_new = dmin_(*dt_new, c);
    double sc = -dt / volume;
    dh = sc * dh; dp1 = sc * dp1; dp2 = sc * dp2;
    if (Q->h < Q->b + P->dry_tolerance && dh > 0.0) {
        Q->h = Q->b + P->dry_tolerance;
        Q->p1 = 0.0; Q->p2 = 0.0;
    }
    Q->h = Q->h + dh;
    Q->p1 = Q->p1 + dp1;
    Q->p2 = Q->p2 + dp2;
    Q->b = Q->b + 0.0;
    if (Q->h < Q->b + P->dry_tolerance) {
        Q->h = dmin_(Q->b, 0.0);
        Q->p1 = 0.0; Q->p2 = 0.0;
    }
}

/*
 * The sequential walk, step by step as the static traversal runs with one
 * thread and one section (src/SFC_generic_traversal_ringbuffer.f90:252-453):
 *   1. boundary skeleton: boundary edges, ghost from the cell (boundary_skeleton,
 *      src/Tools_adaptive_traversal.f90:177-206),
 *   2. for each cell in the current order: the skeleton op on its newly
 *      touched edges (colour, then next) with this cell as the left side and
 *      its own outward normal, then the cell update with the three edge
 *      updates in local edge index order,
 *   3. the grid is reversed: order flips and every cell is reversed (entity
 *      bits, turtle, plotter type), src/Tools_adaptive_traversal.f90:733-739.
 * Cell data arrays are indexed by the cell's position in the ORIGINAL order.
 *
 * cells5: int8[5*n] in the original order, updated in place to the reversed
 * types after an odd number of steps. `reversed` tells whether the current
 * traversal order is the reverse of the original; it is flipped per step.
 * state: h, hu, hv, b (double[n] each), updated in place.
 * flags: int8[n], refinement flags of the last step.
 * scal: [time, dt] in/out; out_dt_new receives min(volume / sum(len*speed)).
 * Returns 0 or negative on an inconsistent mesh.
 */
int oracle_steps(const void* params_v, int64_t n, int8_t* cells5, int* reversed, double* h, double* hu,
                 double* hv, double* b, int8_t* flags, double* scal, int64_t n_steps, int64_t* n_refine_out,
                 double* dt_new_out)
{
    or_init_tables();
    const or_params* P = (const or_params*)params_v;
    or_cell* cells = (or_cell*)malloc(sizeof(or_cell) * (size_t)n);
    or_cell* cur = (or_cell*)malloc(sizeof(or_cell) * (size_t)n);
    int64_t* slot = (int64_t*)malloc(sizeof(int64_t) * 3 * (size_t)n);
    int64_t* ecell = (int64_t*)malloc(sizeof(int64_t) * 2 * (size_t)(2 * n + 8));
    int8_t* eloc = (int8_t*)malloc(2 * (size_t)(2 * n + 8));
    int64_t* bcell = (int64_t*)malloc(sizeof(int64_t) * (size_t)(n + 8));
    int8_t* bloc = (int8_t*)malloc((size_t)(n + 8));
    or_update* upd = (or_update*)malloc(sizeof(or_update) * 3 * (size_t)n);
    or_state* Q0 = (or_state*)malloc(sizeof(or_state) * (size_t)n);
    int rc = 0;
    for (int64_t i = 0; i < n; ++i) {
        cells[i].entity = cells5[5 * i]; cells[i].depth = cells5[5 * i + 1];
        cells[i].plotter = cells5[5 * i + 2]; cells[i].turtle = cells5[5 * i + 3];
        cells[i].color = cells5[5 * i + 4];
    }
    double time = scal[0], dt = scal[1];
    int64_t nref = 0;
    double dtn = DBL_MAX;
    for (int64_t step = 0; step < n_steps && rc == 0; ++step) {
        int rev = *reversed;
        /* pre_traversal_grid_op, :89-109 */
        if (P->max_time > 0.0) dt = dmin_(P->max_time, dt);
        if (P->output_time_step > 0.0) dt = dmin_(P->output_time_step, dt);
        /* cells in the current traversal order */
        for (int64_t k = 0; k < n; ++k) cur[k] = cells[rev ? n - 1 - k : k];
        int64_t ne, nb;
        rc = or_walk_edges(cur, n, slot, ecell, eloc, &ne, bcell, bloc, &nb);
        if (rc) break;
        for (int64_t i = 0; i < n; ++i) {
            Q0[i].h = h[i]; Q0[i].p1 = hu[i]; Q0[i].p2 = hv[i]; Q0[i].b = b[i];
        }
#define ID(k) (rev ? n - 1 - (k) : (k))
        /* 1. boundary skeleton */
        for (int64_t j = 0; j < nb; ++j) {
            int64_t k = bcell[j];
            int li = bloc[j];
            const double* nn = g_normal[cur[k].plotter + 8][li - 1];
            or_state ghost;
            boundary_ghost(P->bc, nn, &Q0[ID(k)], &ghost);
            or_update dummy;
            edge_flux(P->solver, nn, &Q0[ID(k)], &ghost, P->dry_tolerance, &upd[3 * ID(k) + li - 1], &dummy);
        }
        /* 2. the walk */
        nref = 0;
        dtn = DBL_MAX;
        for (int64_t k = 0; k < n; ++k) {
            int64_t c = ID(k);
            int ip, ic, in, tp, tc, tn;
            cell_edge_indices(&cur[k], &ip, &ic, &in);
            cell_edge_types(&cur[k], &tp, &tc, &tn);
            int newl[2], cnt = 0;
            if (tc == E_NEW) newl[cnt++] = ic;
            if (tn == E_NEW) newl[cnt++] = in;
            for (int q = 0; q < cnt; ++q) {
                int li = newl[q];
                int64_t e = slot[3 * k + li - 1];
                int64_t k2 = ecell[2 * e + 1];
                int lj = eloc[2 * e + 1];
                const double* nn = g_normal[cur[k].plotter + 8][li - 1];
                edge_flux(P->solver, nn, &Q0[c], &Q0[ID(k2)], P->dry_tolerance, &upd[3 * c + li - 1],
                          &upd[3 * ID(k2) + lj - 1]);
            }
            or_state Q = Q0[c];
            cell_update(P, cur[k].depth, &Q, &upd[3 * c], dt, &dtn, &flags[c], &nref);
            h[c] = Q.h; hu[c] = Q.p1; hv[c] = Q.p2; b[c] = Q.b;
        }
#undef ID
        /* 3. reverse the grid */
        for (int64_t i = 0; i < n; ++i) cell_reverse(&cells[i]);
        *reversed = !rev;
        /* post_traversal_grid_op, :111-131 */
        time = time + dt;
        dt = P->courant * dtn;
    }
    for (int64_t i = 0; i < n; ++i) {
        cells5[5 * i] = cells[i].entity; cells5[5 * i + 1] = cells[i].depth;
        cells5[5 * i + 2] = cells[i].plotter; cells5[5 * i + 3] = cells[i].turtle;
        cells5[5 * i + 4] = cells[i].color;
    }
    scal[0] = time;
    scal[1] = dt;
    if (n_refine_out) *n_refine_out = nref;
    if (dt_new_out) *dt_new_out = dtn;
    free(cells); free(cur); free(slot); free(ecell); free(eloc); free(bcell); free(bloc); free(upd); free(Q0);
    return rc;
}

/*
 * OpenMP CPU step over the C-ABI mesh format (the same format the GPU takes:
 * cells in upload order, inner edges (a < b) with local indices in the upload
 * orientation, boundary edges). Jacobi form of the same step: on a step with
 * parity 0 the lower-numbered cell of an edge is the first-touched (left)
 * one, on parity 1 the higher-numbered one, and the leg updates are summed in
 * the reversed local order. Used as the timed CPU baseline; tests check it
 * against oracle_steps bit for bit.
 * flux_buf: caller-provided scratch of 8*n_edges + 4*n_bnd doubles.
 */
int oracle_steps_omp(const void* params_v, int64_t n, const int8_t* depth, const int8_t* plotter,
                     int64_t n_edges, const int64_t* edge_cells, const int8_t* edge_local, int64_t n_bnd,
                     const int64_t* bnd_cell, const int8_t* bnd_local, const int64_t* cell_slots,
                     double* h, double* hu, double* hv, const double* b, double* h_out, double* hu_out,
                     double* hv_out, int8_t* flags, double* scal, int64_t* parity_io, int64_t n_steps,
                     double* flux_buf, int64_t* n_refine_out, double* dt_new_out, int threads)
{
    or_init_tables();
    const or_params* P = (const or_params*)params_v;
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#else
    (void)threads;
#endif
    double time = scal[0], dt = scal[1];
    int64_t parity = *parity_io;
    int64_t nref = 0;
    double dtn = DBL_MAX;
    double *hi = h, *hui = hu, *hvi = hv, *ho = h_out, *huo = hu_out, *hvo = hv_out;
    double* ef = flux_buf;                       /* 8 per inner edge: left update, right update */
    double* bf = flux_buf + 8 * n_edges;         /* 4 per boundary edge */
    for (int64_t step = 0; step < n_steps; ++step) {
        int odd = (int)(parity & 1);
        if (P->max_time > 0.0) dt = dmin_(P->max_time, dt);
        if (P->output_time_step > 0.0) dt = dmin_(P->output_time_step, dt);
#pragma omp parallel for schedule(static)
        for (int64_t e = 0; e < n_edges; ++e) {
            int64_t cl = edge_cells[2 * e + odd], cr = edge_cells[2 * e + 1 - odd];
            int ll = edge_local[2 * e + odd];
            const double* nn = g_normal[plotter[cl] + 8][ll - 1];
            or_state QL = { hi[cl], hui[cl], hvi[cl], b[cl] }, QR = { hi[cr], hui[cr], hvi[cr], b[cr] };
            or_update a, c;
            edge_flux(P->solver, nn, &QL, &QR, P->dry_tolerance, &a, &c);
            double* o = ef + 8 * e;
            /* stored by side: [0..3] for edge_cells[2e], [4..7] for edge_cells[2e+1] */
            double* oa = o + 4 * odd;
            double* ob = o + 4 * (1 - odd);
            oa[0] = a.h; oa[1] = a.p1; oa[2] = a.p2; oa[3] = a.s;
            ob[0] = c.h; ob[1] = c.p1; ob[2] = c.p2; ob[3] = c.s;
        }
#pragma omp parallel for schedule(static)
        for (int64_t j = 0; j < n_bnd; ++j) {
            int64_t cc = bnd_cell[j];
            int ll = bnd_local[j];
            const double* nn = g_normal[plotter[cc] + 8][ll - 1];
            or_state Q = { hi[cc], hui[cc], hvi[cc], b[cc] }, ghost;
            boundary_ghost(P->bc, nn, &Q, &ghost);
            or_update a, c;
            edge_flux(P->solver, nn, &Q, &ghost, P->dry_tolerance, &a, &c);
            double* o = bf + 4 * j;
            o[0] = a.h; o[1] = a.p1; o[2] = a.p2; o[3] = a.s;
        }
        double dmin_all = DBL_MAX;
        int64_t nr = 0;
#pragma omp parallel for schedule(static) reduction(min : dmin_all) reduction(+ : nr)
        for (int64_t c = 0; c < n; ++c) {
            or_update u3[3];
            for (int i = 0; i < 3; ++i) {
                int li = odd ? 2 - i : i;                 /* local index order of this traversal */
                int64_t s = cell_slots[3 * c + li];
                const double* src = (s >= 0) ? ef + 8 * (s >> 1) + 4 * (s & 1) : bf + 4 * (-s - 1);
                u3[i].h = src[0]; u3[i].p1 = src[1]; u3[i].p2 = src[2]; u3[i].s = src[3];
            }
            or_state Q = { hi[c], hui[c], hvi[c], b[c] };
            double dl = DBL_MAX;
            int64_t r = 0;
            cell_update(P, depth[c], &Q, u3, dt, &dl, &flags[c], &r);
            ho[c] = Q.h; huo[c] = Q.p1; hvo[c] = Q.p2;
            if (dl < dmin_all) dmin_all = dl;
            nr += r;
        }
        dtn = dmin_all;
        nref = nr;
        time = time + dt;
        dt = P->courant * dtn;
        parity++;
        double* t;
        t = hi; hi = ho; ho = t;
        t = hui; hui = huo; huo = t;
        t = hvi; hvi = hvo; hvo = t;
    }
    /* leave the newest state in h/hu/hv */
    if (hi != h) {
        memcpy(h, hi, sizeof(double) * (size_t)n);
        memcpy(hu, hui, sizeof(double) * (size_t)n);
        memcpy(hv, hvi, sizeof(double) * (size_t)n);
    }
    scal[0] = time;
    scal[1] = dt;
    *parity_io = parity;
    if (n_refine_out) *n_refine_out = nref;
    if (dt_new_out) *dt_new_out = dtn;
    return 0;
}

/* For each cell and local edge index (1..3, stored at [3*c + i-1]) the slot of its
 * edge update: (e << 1) | side for inner edge e (side 0 = edge_cells[2e]), or
 * -(j) - 1 for boundary edge j. Returns 0, or -1 if a slot is claimed twice or left empty. */
int oracle_cell_slots(int64_t n, int64_t n_edges, const int64_t* edge_cells, const int8_t* edge_local,
                      int64_t n_bnd, const int64_t* bnd_cell, const int8_t* bnd_local, int64_t* out)
{
    const int64_t EMPTY = INT64_MIN;
    for (int64_t i = 0; i < 3 * n; ++i) out[i] = EMPTY;
    for (int64_t e = 0; e < n_edges; ++e)
        for (int s = 0; s < 2; ++s) {
            int64_t idx = 3 * edge_cells[2 * e + s] + edge_local[2 * e + s] - 1;
            if (out[idx] != EMPTY) return -1;
            out[idx] = (e << 1) | s;
        }
    for (int64_t j = 0; j < n_bnd; ++j) {
        int64_t idx = 3 * bnd_cell[j] + bnd_local[j] - 1;
        if (out[idx] != EMPTY) return -1;
        out[idx] = -j - 1;
    }
    for (int64_t i = 0; i < 3 * n; ++i)
        if (out[i] == EMPTY) return -1;
    return 0;
}

int oracle_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
