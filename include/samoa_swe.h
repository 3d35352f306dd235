/*
 * samoa_swe.h — C ABI of the GB300-native shallow-water (SWE) time step.
 *
 * A drop-in for sam(oa)^2's SWE Euler time-step traversal
 * `call swe%euler%traverse(grid)` (src/SWE/SWE.f90:393, also :339), i.e. the
 * traversal t_swe_euler_timestep_traversal of src/SWE/SWE_euler_timestep.f90.
 * Mesh generation, adaptivity and I/O stay on the host. After each remesh
 * the host hands the Sierpinski-ordered cells and the edge streams to the
 * device (swe_mesh_upload), uploads the cell state, and calls swe_traverse
 * once per time step (or once for many steps).
 *
 * Conventions (all follow the reference):
 *   - h is the water SURFACE elevation, depth = h - b (src/SWE/SWE_data_types.f90:42-65);
 *   - cells are in the host's current traversal order; the first step after
 *     an upload traverses them in that order, and every step reverses the
 *     traversal direction like grid%reverse() does
 *     (src/SFC_generic_traversal_ringbuffer.f90:420);
 *   - local edge indices are 1 = right leg, 2 = hypotenuse, 3 = left leg in the
 *     cell's current orientation (src/SFC_data_types.f90:47-49);
 *   - indices are int64 like src/Generic/samoa.h; the device narrows to int32
 *     (n_cells < 2^31).
 * Every function returns 0 on success or a negative SWE_E* code; nothing
 * aborts. swe_last_error() gives the message of the last failure on the
 * calling thread. A context is not thread-safe; use one context per stream.
 */
#ifndef SAMOA_SWE_H
#define SAMOA_SWE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define SWE_OK 0
#define SWE_E_INVALID -1      /* bad argument / inconsistent mesh */
#define SWE_E_CUDA -2         /* CUDA runtime error */
#define SWE_E_NOMESH -3       /* no mesh uploaded */
#define SWE_E_NOMEM -4        /* device allocation failed */
#define SWE_E_STATE -5        /* state or time step not set */
#define SWE_E_DEVICE -6       /* a kernel reported an error (timeout, bad index) */

/* flux solvers: GeoClaw numbering for the GeoClaw family
 * (src/geoclaw/c_bind_riemannsolvers.f90:4-6), then the Lax-Friedrichs family of
 * compute_lf_flux (src/SWE/SWE_euler_timestep.f90:359-446). The reference picks
 * one at compile time (SConstruct:223-237); here it is a runtime parameter. */
#define SWE_SOLVER_FWAVE 1
#define SWE_SOLVER_AUG_RIEMANN 3
#define SWE_SOLVER_LF 10
#define SWE_SOLVER_LF_BATH 11
#define SWE_SOLVER_LLF 12
#define SWE_SOLVER_LLF_BATH 13

/* domain-boundary conditions of bnd_skeleton_scalar_op
 * (src/SWE/SWE_euler_timestep.f90:241-248): OUTFLOW is the active one in the
 * reference; SLIP and NOSLIP are its commented-out alternatives. */
#define SWE_BC_OUTFLOW 0
#define SWE_BC_SLIP 1
#define SWE_BC_NOSLIP 2

/* Runtime parameters the step reads from cfg (src/Config.f90:30-121). */
typedef struct swe_params {
    int32_t solver;            /* SWE_SOLVER_* */
    int32_t bc;                /* SWE_BC_* */
    double dry_tolerance;      /* cfg%dry_tolerance [m] */
    double courant;            /* cfg%courant_number */
    double scaling;            /* cfg%scaling: domain edge length */
    int32_t min_depth;         /* cfg%i_min_depth */
    int32_t max_depth;         /* cfg%i_max_depth */
    double max_time;           /* cfg%r_max_time, <= 0 disables the dt clamp */
    double output_time_step;   /* cfg%r_output_time_step, <= 0 disables the dt clamp */
} swe_params;

typedef struct swe_ctx swe_ctx;

/* Create a context on CUDA device `device`. Replaces the creation of the
 * euler traversal in t_swe%create (src/SWE/SWE.f90:52-88). */
int swe_create(swe_ctx** ctx, int device);

/* Free all device memory of the context. Replaces swe_destroy (src/SWE/SWE.f90:173-203). */
int swe_destroy(swe_ctx* ctx);

/* Launch work on this stream (a cudaStream_t, NULL = the context's own stream). */
int swe_set_stream(swe_ctx* ctx, void* stream);

/* Set the runtime parameters (the cfg fields of src/Config.f90:30-121 and the
 * compile-time flux choice of SConstruct:223-237). */
int swe_set_params(swe_ctx* ctx, const swe_params* params);

/* Upload a mesh after a remesh. Replaces the cell and edge streams the
 * traversal reads (t_grid_section, src/Tools_grid.f90:480-515); the layout
 * follows the index maps of samoa_get_grid (src/Generic/samoa.h:25-57).
 *   depth[n_cells], plotter[n_cells]   cell depth and plotter-grammar type (+-1..+-8)
 *   edge_cells[2*n_edges]              the two cells of each inner edge
 *   edge_local[2*n_edges]              the edge's local index (1..3) in each cell
 *   bnd_cell[n_bnd], bnd_local[n_bnd]  domain-boundary edges
 * Every (cell, local index) must be used exactly once. Invalidates the state. */
int swe_mesh_upload(swe_ctx* ctx, int64_t n_cells, const int8_t* depth, const int8_t* plotter,
                    int64_t n_edges, const int64_t* edge_cells, const int8_t* edge_local, int64_t n_bnd,
                    const int64_t* bnd_cell, const int8_t* bnd_local);

/* Copy the cell state in/out (host pointers, n_cells doubles each; b is read-only
 * for the step). Replaces gv_Q%read/write on the cells' data_pers%Q
 * (src/Tools_grid_variable.f90:146-193). Download synchronises. */
int swe_state_upload(swe_ctx* ctx, const double* h, const double* hu, const double* hv, const double* b);
int swe_state_download(swe_ctx* ctx, double* h, double* hu, double* hv, double* b);

/* Device pointers of the current state (valid until the next step or upload). */
int swe_state_device(swe_ctx* ctx, double** h, double** hu, double** hv, const double** b);

/* grid%r_time and grid%r_dt (src/SWE/SWE_data_types.f90:126-130). The step
 * uses dt (clamped by max_time / output_time_step) and leaves
 * dt = courant * min_cells(volume / sum(len * max_wave_speed)) for the next
 * step (src/SWE/SWE_euler_timestep.f90:89-131). swe_get_time synchronises. */
int swe_set_time(swe_ctx* ctx, double time, double dt);
int swe_get_time(swe_ctx* ctx, double* time, double* dt, double* dt_new);

/* Run n_steps time steps, asynchronously on the context's stream.
 * Replaces n_steps calls of swe%euler%traverse(grid) (src/SWE/SWE.f90:393). */
int swe_traverse(swe_ctx* ctx, int64_t n_steps);

/* Refinement flags of the last step (-1 coarsen, 0 keep, 1 refine; int8 per
 * cell in upload order) and the number of refinements it issued
 * (src/SWE/SWE_euler_timestep.f90:117,336-344). Synchronises. */
int swe_get_refinements(swe_ctx* ctx, int8_t* flags, int64_t* n_refinements);

/* Number of steps run since the last mesh upload (its parity is the current
 * traversal direction: odd = reversed). Synchronises. */
int swe_get_step_count(swe_ctx* ctx, int64_t* steps);

/* Block until all work of the context has finished; reports device errors. */
int swe_synchronize(swe_ctx* ctx);

/* Message of the last failure on this thread (always NUL-terminated). */
int swe_last_error(char* buf, size_t n);

/* Kernel tuning: cells per segment (even, 64..1536; 18 doubles of shared
 * memory per cell, 22 with staging depth 2, at most 227 KB in all) and threads
 * per block (multiple of 32, 64..256); 0 keeps
 * the current value. A mesh upload or
 * this call rebuilds the segment task lists. Until a segment length is set
 * here, each mesh upload picks it by size: 384 cells from 2^20 cells on, 256
 * below (more segments than resident CTAs on small meshes). */
int swe_set_tiling(swe_ctx* ctx, int32_t segment_cells, int32_t block_threads);

/* Staging depth of the step kernel: 1 = a CTA stages a segment's state into
 * shared memory, then works on it; 2 = it stages the next segment (bulk copies
 * in flight) while it works on the current one, at 4 * segment_cells doubles
 * more shared memory. Default 1; SWE_E_INVALID if the tiling then exceeds
 * shared memory. No counterpart in the reference. */
int swe_set_staging(swe_ctx* ctx, int32_t depth);

/* Arithmetic of the step kernel. STRICT (the default): every FP64 operation
 * rounded separately, in the reference's evaluation order, so results are bit
 * identical to a strict-IEEE CPU evaluation of the reference step. FMA: the
 * same kernel with multiply-adds fused by the compiler; faster on GB300's FP64
 * pipe, results within a few ulps per step of STRICT (not bit identical). No
 * reference counterpart (the reference's precision is a compile-time choice,
 * SConstruct:272-278). Adjoint steps always use STRICT. */
#define SWE_ARITH_STRICT 0
#define SWE_ARITH_FMA 1
int swe_set_arith(swe_ctx* ctx, int32_t mode);
int swe_get_tiling(swe_ctx* ctx, int32_t* segment_cells, int32_t* block_threads);

/* How the edges between two segments are solved. PASS: once per step by a
 * kernel before the step kernel, which copies the updates. INKERNEL: by both
 * segments' CTAs, each keeping its side (no extra launch). AUTO (the default):
 * PASS for steps on device-resident state (swe_traverse and the calls built on
 * it), INKERNEL for swe_step_host, whose state is in host memory. The results
 * are bit identical. No reference counterpart. */
#define SWE_CROSS_AUTO 0
#define SWE_CROSS_PASS 1
#define SWE_CROSS_INKERNEL 2
int swe_set_cross_pass(swe_ctx* ctx, int32_t mode);

/* The order the step kernel hands its segments out in. CURVE: along the
 * space-filling curve. SPREAD: each instance's segments in bit-reversed index
 * order, so that the CTAs working at one time hold segments from all over the
 * domain and mix cheap (dry) and FP64-heavy (wet) work. AUTO (the default):
 * SPREAD from 2048 segments on, CURVE below. The results are bit identical.
 * No reference counterpart. */
#define SWE_ORDER_CURVE 0
#define SWE_ORDER_SPREAD 1
#define SWE_ORDER_AUTO 2
int swe_set_segment_order(swe_ctx* ctx, int32_t mode);

/* Sizes of the uploaded mesh's work lists: segments, edge tasks in the segment
 * lists (an edge between two segments counted once per segment), edges between
 * two segments (computed once per step by a pass before the step kernel) and
 * kernel launches per device-resident step (1, or 2 with that pass). Any pointer may be null.
 * No reference counterpart (the reference's sections, src/SFC_edge_traversal.f90). */
int swe_get_task_counts(swe_ctx* ctx, int64_t* n_segments, int64_t* n_tasks, int64_t* n_cross_edges,
                        int32_t* launches_per_step);

/* Vertices of the cells of swe_mesh_uniform(depth) in the unit square, in the
 * same cell order: vertices[6 k + 2 v + {0, 1}] = (x, y) of vertex v of cell k
 * (exact dyadic values). The node coordinates samoa_get_grid hands out
 * (src/Generic/samoa.h:25-57), per cell; used by the headless VTK writer. */
int swe_mesh_uniform_vertices(int32_t depth, double* vertices);

/* Mesh of the unit square from its leaf depths: the cells of a conforming
 * Sierpinski tree in traversal order given by their depths (depth[k] of cell
 * k); the same walk as swe_mesh_uniform (init_grid with the tree's own
 * bisections) gives the plotter types, the edge streams in the swe_mesh_upload
 * layout, and optionally centroids[2n] and vertices[6n]. With plotter_out and
 * the edge arrays NULL only the counts *n_edges, *n_bnd are returned (sizes:
 * edge_cells, edge_local 2 * n_edges; bnd_cell, bnd_local n_bnd). Since every
 * cell has three edges, 2 * n_edges + n_bnd = 3 * n_cells: arrays of 3 * n_cells
 * entries each always suffice, and one call with them returns counts and streams.
 * SWE_E_INVALID if the depths are not the leaves of such a tree or the tree is
 * not conforming. The host side of the remesh handoff. */
int swe_mesh_build(int64_t n_cells, const int8_t* depth, int64_t* n_edges, int64_t* n_bnd, int8_t* plotter_out,
                   int64_t* edge_cells, int8_t* edge_local, int64_t* bnd_cell, int8_t* bnd_local, double* centroids,
                   double* vertices);

/* One remesh from the step's refinement flags (-1 coarsen, 0 keep, 1 refine):
 * the adaption traversal's conformity closure and refine/coarsen rules
 * (src/Conformity/Conformity.f90:1244-1317, src/SWE/SWE_adapt.f90:95-169).
 * Input: the mesh as leaf depths in traversal order, the flags, and optionally
 * the state h, hu, hv, b (host arrays, n_cells). Output: *n_out cells; with
 * depth_out non-NULL (capacity >= *n_out) the new leaf depths, optionally the
 * source cell of each new cell (source_out: the parent of a refined cell, the
 * first of two merged siblings; compare depths to tell which), and for each
 * given input the transferred state (refined cells copy their parent's values,
 * merged siblings average them, order 0). Call once with depth_out = NULL for
 * the count. The new mesh's streams come from swe_mesh_build. */
int swe_mesh_adapt(int64_t n_cells, const int8_t* depth, const int8_t* flags, const double* h, const double* hu,
                   const double* hv, const double* b, int64_t capacity, int64_t* n_out, int8_t* depth_out,
                   int64_t* source_out, double* h_out, double* hu_out, double* hv_out, double* b_out);

/* Uniform Sierpinski mesh of the unit square at reference depth `depth`
 * (2^(depth+1) cells) in traversal order, restating init_grid
 * (src/SFC_node_traversal.f90:22-145). Call with NULL outputs to get the sizes.
 * Inner edges are numbered in first-touch order (colour edge before next
 * edge, src/Tools_adaptive_traversal.f90:585-603), boundary edges in walk order.
 * centroids (optional, may be NULL): 2 doubles per cell, the mean of the
 * three corners in the unit square. */
int swe_mesh_uniform(int32_t depth, int64_t* n_cells, int64_t* n_edges, int64_t* n_bnd, int8_t* depth_out,
                     int8_t* plotter_out, int64_t* edge_cells, int8_t* edge_local, int64_t* bnd_cell,
                     int8_t* bnd_local, double* centroids);

/* ---- ensembles: many independent instances stepped together ------------ */
/* An ensemble is a context with n_instances meshes that advance together, one
 * kernel launch per time step for all of them, each instance with its own
 * parameters, time and dt. No reference counterpart: sam(oa)^2 runs one
 * scenario per process. Arrays are concatenated in instance order; cell
 * indices in edge_cells / bnd_cell are local to their instance. State arrays
 * (swe_state_upload/download) and flags are concatenated the same way
 * (sum of n_cells entries). All instances must use the same solver. */
int swe_ensemble_mesh_upload(swe_ctx* ctx, int64_t n_instances, const int64_t* n_cells, const int64_t* n_edges,
                             const int64_t* n_bnd, const int8_t* depth, const int8_t* plotter,
                             const int64_t* edge_cells, const int8_t* edge_local, const int64_t* bnd_cell,
                             const int8_t* bnd_local);
int swe_ensemble_set_params(swe_ctx* ctx, const swe_params* params /* [n_instances] */);
int swe_ensemble_set_time(swe_ctx* ctx, const double* time, const double* dt);
int swe_ensemble_get_time(swe_ctx* ctx, double* time, double* dt, double* dt_new);
int swe_ensemble_get_refinements(swe_ctx* ctx, int8_t* flags, int64_t* n_refinements /* [n_instances] */);

/* Run n_steps time steps as one CUDA graph: the first call with a given
 * n_steps captures the launches, later calls replay the graph. No reference
 * counterpart (the reference loop is host-driven, src/SWE/SWE.f90:380-429). */
int swe_traverse_graph(swe_ctx* ctx, int64_t n_steps);

/* Freeze the time-step sequence: the k-th step after this call uses
 * dts[k * n_instances + i] for instance i instead of the CFL dt (for adjoint
 * and finite-difference runs, where dt must not depend on the state);
 * n_steps = 0 clears it. No reference counterpart. */
int swe_set_dt_sequence(swe_ctx* ctx, int64_t n_steps, const double* dts);

/* ---- discrete adjoint (single-instance contexts; the f-wave and augmented
 * solvers and the four Lax-Friedrichs fluxes) ------------------------------ */
/* No reference counterpart: sam(oa)^2 has no adjoint. Cotangent buffers are
 * device pointers with n_cells doubles each. */

/* Copy the current state (h, hu, hv) to caller device buffers and return the
 * step count (its parity is the traversal direction); restore sets the state
 * and the step count back (time is not restored). For checkpointing. */
int swe_snapshot_store(swe_ctx* ctx, double* h, double* hu, double* hv, int64_t* step);
int swe_snapshot_restore(swe_ctx* ctx, const double* h, const double* hu, const double* hv, int64_t step);

/* Surface elevation h of the current state at the given cells (device arrays;
 * NaN for an index out of range), asynchronously: a gauge sampler on the
 * device (the point output of src/SWE/SWE_point_output.f90:226-266 at order 0). */
int swe_sample_gauges(swe_ctx* ctx, int64_t n_gauges, const int64_t* cells, double* out);

/* Branch-frozen forward run for checking the adjoint (f-wave, single
 * instance): mode 1 runs n_steps steps recording every edge's decisions
 * (edges[s * edge_stride + k], edge_stride >= the task count plus the
 * cross-segment edge count of swe_get_task_counts) and every cell's wet/dry
 * fixes (branch[s * branch_stride + cell]); mode 2 runs them again taking
 * every decision from those records instead of the comparisons, so the run is
 * a smooth function of its inputs near the recorded one (finite differences of
 * it approximate the discrete adjoint's gradient without crossing a kink).
 * With n_gauges > 0 the gauge cells' surface after every step goes to
 * out[s * n_gauges + g] (device memory). No reference counterpart. */
int swe_traverse_frozen(swe_ctx* ctx, int64_t n_steps, int32_t mode, uint8_t* branch, int64_t branch_stride,
                        uint16_t* edges, int64_t edge_stride, int64_t n_gauges, const int64_t* cells, double* out);

/* Run n_steps steps like swe_traverse and record each step's wet/dry branches
 * (per cell: bit 0 wetting fix, bit 1 drying clamp) at branch + i * stride
 * for the i-th step (device buffer, stride >= n_cells). */
int swe_traverse_branches(swe_ctx* ctx, int64_t n_steps, uint8_t* branch, int64_t stride);

/* Undo the last step: valid right after a step, whose input state is still in
 * the other state buffer; sets the step count back by one (time is kept). */
int swe_step_back(swe_ctx* ctx);

/* One reverse step. The context is at step t with state x_t. Given
 * lam = dJ/dx_{t+1}, writes out = dJ/dx_t and adds dJ/db of step t to bbar,
 * differentiating every branch on the side the forward step took; dt is the
 * frozen value of swe_set_dt_sequence, which is required. `branch` holds the
 * branches recorded when step t ran forward (swe_traverse_branches); with
 * branch = NULL the step first runs forward itself to record them and the
 * context is left at step t+1, else it stays at step t. */
int swe_adjoint_step(swe_ctx* ctx, const uint8_t* branch, const double* lam_h, const double* lam_hu,
                     const double* lam_hv, double* out_h, double* out_hu, double* out_hv, double* bbar);

/* n_steps steps, each followed by the gauge sample of swe_sample_gauges into
 * out[step * n_gauges + g] (device): the forward operator of the gauge misfit,
 * with no host round trip between steps. No counterpart in the reference. */
int swe_traverse_gauges(swe_ctx* ctx, int64_t n_steps, int64_t n_gauges, const int64_t* cells, double* out);

/* Gradient of the gauge misfit J = sum_t sum_g (h_{t+1}[gauges[g]] - obs[t][g])^2
 * over n_steps f-wave steps with the frozen dt sequence dts (host, n_steps),
 * from the context's current state x_0, by one checkpointed reverse sweep run
 * entirely in the library: binomial checkpointing (revolve's offline schedule)
 * with `snapshots` device snapshot slots, each forward step recording its
 * branches, the first visit of each step sampling the gauges, each reverse step
 * adding the gauge residuals and calling the step's discrete adjoint. Device
 * arrays: gauges[n_gauges] (cells), obs[n_steps * n_gauges]; outputs
 * gauge_values[n_steps * n_gauges] (may be NULL), grad_h (dJ/dh of x_0),
 * grad_hu, grad_hv (may be NULL), grad_b (dJ/db); J and forward_steps (may be
 * NULL) on the host. The context is left at x_0 and its step count; the dt
 * sequence stays set. Synchronises before returning. Allocates
 * snapshots * 24 * n_cells + n_steps * n_cells bytes for the sweep.
 * No counterpart in the reference. */
int swe_gauge_gradient(swe_ctx* ctx, int64_t n_steps, const double* dts, int32_t snapshots, int64_t n_gauges,
                       const int64_t* gauges, const double* obs, double* gauge_values, double* grad_h,
                       double* grad_hu, double* grad_hv, double* grad_b, double* J, int64_t* forward_steps);

/* Check a mesh in the swe_mesh_upload layout on the host without a context
 * (same checks as the upload): 0 if valid, SWE_E_INVALID with a message otherwise. */
int swe_mesh_validate(int64_t n_cells, const int8_t* depth, const int8_t* plotter, int64_t n_edges,
                      const int64_t* edge_cells, const int8_t* edge_local, int64_t n_bnd, const int64_t* bnd_cell,
                      const int8_t* bnd_local);

/* Evaluate the edge flux of one solver on n independent edges on the device:
 * the skeleton operator of src/SWE/SWE_euler_timestep.f90:196-215 with
 * compute_geoclaw_flux / compute_lf_flux. Host arrays: normals[2n],
 * q_left[4n], q_right[4n] as (h, hu, hv, b); out_left[4n], out_right[4n] as
 * (h, hu, hv, max_wave_speed) net updates. For solver-level checks. */
int swe_riemann_batch(int32_t solver, int64_t n, const double* normals, const double* q_left, const double* q_right,
                      double dry_tolerance, double* out_left, double* out_right);

/* One step on state arrays the caller keeps in host memory (or device memory):
 * the step reads h, hu, hv and b where they are and writes h_out, hu_out,
 * hv_out and the refinement flags (flags_out may be NULL: the context's
 * buffer) directly, with no staging copies; on a Grace-Blackwell node the
 * kernel streams them over the coherent CPU-GPU link. Replaces the upload /
 * traverse / download round trip a host that owns the arrays (the Fortran grid)
 * would otherwise make around swe%euler%traverse (src/SWE/SWE.f90:393). Arrays:
 * n_cells doubles in the mesh order; pinned (cudaHostAlloc / cudaHostRegister)
 * or device memory, or pageable memory where the device reads it coherently
 * (cudaDevAttrPageableMemoryAccess); inputs and outputs must not overlap.
 * b = NULL uses the uploaded bathymetry. Time, dt, the step counter (traversal
 * direction) and the refinement count advance as in swe_traverse; the
 * context's own state buffers are left as they were. Single-instance contexts
 * only. Returns without synchronising (swe_synchronize before reading). */
int swe_step_host(swe_ctx* ctx, const double* h, const double* hu, const double* hv, const double* b,
                  double* h_out, double* hu_out, double* hv_out, int8_t* flags_out);

/* Device self-check of the step's correctly rounded division with a shared
 * reciprocal (the quotients u = hu / h and v = hv / h, which share h, and the
 * two f-wave coefficients, which share s2 - s1): on 2n seeded random pairs
 * (a, b) with exponents in [-exponent_span, exponent_span], one in 16 with
 * a = 0, counts the quotients that differ from IEEE a / b in any bit.
 * No counterpart in the reference (the Fortran step divides directly). */
int swe_division_check(int64_t n, uint64_t seed, int32_t exponent_span, int64_t* mismatches);

/* Test-only device fault injection, off by default. No counterpart in the
 * reference (it has no bounded waits: it asserts). SWE_INJECT_STAGING_TX: the
 * step kernel arms each staging mbarrier for 16 bytes more than its bulk copies
 * deliver, so the phase never completes; every copy still lands, and the
 * kernel's bounded wait (shortened to 20 ms) gives up, the CTA leaves its
 * segment and the step reports SWE_E_DEVICE at the next swe_synchronize. The
 * report clears the device flag; the failed step's state is undefined, so
 * upload a state (or a mesh) before stepping on. Applies to device-resident
 * steps (swe_traverse); stays set until SWE_INJECT_NONE. */
#define SWE_INJECT_NONE 0
#define SWE_INJECT_STAGING_TX 1
int swe_set_fault_injection(swe_ctx* ctx, int32_t kind);

/* One time step on caller-owned device memory, allocating nothing. No
 * counterpart in the reference. For callers that cannot allocate device memory
 * at the point where they step (a host code whose device memory all comes from
 * its own pool, or that steps where an allocation would synchronise the device):
 * every argument after `params` is a device pointer the caller owns, in the
 * layout of swe_mesh_upload / swe_state_upload; the step reads (h, hu, hv, b),
 * writes (h_out, hu_out, hv_out) and the refinement flags (flags may be NULL),
 * uses dt as given (no clamps), the traversal parity `parity` (0 = the given
 * cell order, 1 = reversed, as on the odd steps after an upload), and writes
 * min(volume / sum(len * speed)) to *dt_new and the refinement count to
 * *n_refinements, both device pointers. *n_refinements is -1 (and the outputs
 * undefined) when the mesh is invalid: an index or a local edge number out of
 * range, a plotter type or depth out of range, or a (cell, local edge) slot that
 * no edge or more than one edge claims; the next call starts clean.
 * The work goes on `stream` (a cudaStream_t; NULL = the legacy default stream)
 * and the call returns without synchronising.
 * Limits: n_cells <= 65,536. The scratch (edge updates, per-slot claim counts
 * and reduction accumulators, 7.1 MB) is one fixed array in device memory that
 * every GPU which loads the library keeps until exit; all calls share it, so
 * calls that overlap on the GPU (different streams, or without ordering) race.
 * The first call on a
 * device, and the first after that device's context was replaced (a device
 * reset), sets it up (cudaGetSymbolAddress, geometry tables, clearing the
 * accumulators and claim counts, one device synchronisation): make that first
 * call before any stream capture. */
int swe_step_noalloc(const swe_params* params, int64_t n_cells, const int8_t* depth, const int8_t* plotter,
                     int64_t n_edges, const int64_t* edge_cells, const int8_t* edge_local, int64_t n_bnd,
                     const int64_t* bnd_cell, const int8_t* bnd_local, const double* h, const double* hu,
                     const double* hv, const double* b, double* h_out, double* hu_out, double* hv_out, int8_t* flags,
                     double dt, int32_t parity, double* dt_new, int64_t* n_refinements, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* SAMOA_SWE_H */
