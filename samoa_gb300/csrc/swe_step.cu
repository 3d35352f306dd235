// Context management and the C ABI of the SWE time step (include/samoa_swe.h).
//
// A context holds one or more instances (an ensemble). Instance i's cells sit
// at offset[i] in the device arrays (offsets even, so every segment starts on
// a 16-byte boundary for the TMA bulk copies); segments never span two
// instances. The plain C-ABI calls work on a one-instance context; the
// swe_ensemble_* calls set up many instances that step together in one
// launch per time step, each with its own dt.
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <vector>

#include "swe_internal.h"
#include "swe_adjoint.cuh"

namespace swe {

static thread_local char g_err[512] = "";

int set_error(int code, const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
    return code;
}

#define CUDA_TRY(x)                                                                                     \
    do {                                                                                                \
        cudaError_t e_ = (x);                                                                           \
        if (e_ != cudaSuccess)                                                                          \
            return set_error(SWE_E_CUDA, "%s failed: %s (%s:%d)", #x, cudaGetErrorString(e_), __FILE__, \
                             __LINE__);                                                                 \
    } while (0)

template <int SOLVER>
__global__ void riemann_batch_kernel(int64_t n, const double* nrm, const double* ql, const double* qr, double drytol,
                                     double* ol, double* orr) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        State L{ql[4 * i], ql[4 * i + 1], ql[4 * i + 2], ql[4 * i + 3]};
        State R{qr[4 * i], qr[4 * i + 1], qr[4 * i + 2], qr[4 * i + 3]};
        double dL, dR, sqL, sqR, yL, yR;
        depth_terms(L, drytol, dL, sqL, yL);
        depth_terms(R, drytol, dR, sqR, yR);
        Update fL, fR;
        edge_flux<SOLVER>(nrm[2 * i], nrm[2 * i + 1], L, R, dL, dR, sqL, sqR, yL, yR, drytol, fL, fR);
        ol[4 * i] = fL.h; ol[4 * i + 1] = fL.p1; ol[4 * i + 2] = fL.p2; ol[4 * i + 3] = fL.s;
        orr[4 * i] = fR.h; orr[4 * i + 1] = fR.p1; orr[4 * i + 2] = fR.p2; orr[4 * i + 3] = fR.s;
    }
}

// splitmix64 (Steele, Lea, Flood, OOPSLA 2014): a counter-based stream of
// 64-bit values for the division self-check.
__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
    z += 0x9e3779b97f4a7c15ULL;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}

// A double with a random significand, random sign and an exponent drawn from
// [-e_span, e_span]; every 8th value gets an all-ones or all-zeros low
// significand, which exercises the tie and boundary cases of the rounding.
__device__ __forceinline__ double draw_double(unsigned long long z, int e_span) {
    const unsigned long long w = mix64(z);
    unsigned long long mant = w & 0x000fffffffffffffULL;
    const int sel = (int)((w >> 52) & 7);
    if (sel == 0) mant |= 0x000ffffffff00000ULL;
    if (sel == 1) mant &= 0x000ffffff0000000ULL;
    const unsigned long long r = mix64(z ^ 0x5555555555555555ULL);
    const int e = (int)(r % (unsigned long long)(2 * e_span + 1)) - e_span;
    const unsigned long long sign = (r >> 63) << 63;
    return __longlong_as_double((long long)(sign | ((unsigned long long)(e + 1023) << 52) | mant));
}

// Compares div_rn(a, recip_rn(b)) and div_rn(c, recip_rn(b)) with the IEEE
// quotients bit for bit (a NaN matches any NaN); counts mismatches.
__global__ void division_check_kernel(int64_t n, unsigned long long seed, int e_span,
                                      unsigned long long* mismatches) {
    unsigned long long bad = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const unsigned long long z = seed + 3ULL * (unsigned long long)i;
        const double b = draw_double(z, e_span);
        const double a = draw_double(z + 1, e_span);
        const double c = (i & 15) == 0 ? 0.0 : draw_double(z + 2, e_span);
        const Recip r = recip_rn(b);
        const double q1 = div_rn(a, r), q2 = div_rn(c, r), e1 = a / b, e2 = c / b;
        const bool ok1 = (q1 != q1 && e1 != e1) || __double_as_longlong(q1) == __double_as_longlong(e1);
        const bool ok2 = (q2 != q2 && e2 != e2) || __double_as_longlong(q2) == __double_as_longlong(e2);
        bad += (ok1 ? 0 : 1) + (ok2 ? 0 : 1);
    }
    if (bad) atomicAdd(mismatches, bad);
}

__global__ void set_times_kernel(InstScalars* S, const double* t, const double* dt, int n) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        S[i].time = t[i];
        S[i].dt = dt[i];
        S[i].dt_acc = (unsigned long long)__double_as_longlong(DBL_MAX);
        S[i].ds_acc = 0;
        S[i].refine_acc = 0;
    }
}

__global__ void reset_scalars_kernel(InstScalars* S, GlobalScalars* G, int n) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        S[i].time = 0.0;
        S[i].dt = 0.0;
        S[i].dt_new = DBL_MAX;
        S[i].dt_acc = (unsigned long long)__double_as_longlong(DBL_MAX);
        S[i].ds_acc = 0;
        S[i].refine_acc = 0;
        S[i].n_refine = 0;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        G->done = 0;
        G->error = 0;
        G->next_seg = 0;
        G->step = 0;
        G->dt_seq_base = 0;
    }
}

__global__ void mark_seq_base_kernel(GlobalScalars* G) { G->dt_seq_base = G->step; }

__global__ void set_step_kernel(GlobalScalars* G, long long step) { G->step = step; }

__global__ void gauge_kernel(const GlobalScalars* G, const double* h0, const double* h1, int64_t n,
                             const int64_t* cells, int64_t n_cells, double* out) {
    const double* h = (G->step & 1) ? h1 : h0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t c = cells[i];
        out[i] = (c >= 0 && c < n_cells) ? h[c] : __longlong_as_double(0x7ff8000000000000LL);
    }
}

// lam_h[gauge g] += 2 (value[g] - obs[g]) for the gauges in order: a gauge listed
// twice adds twice, in list order. Up to kResidualParallel gauges, the thread of
// a cell's first listing adds all of its listings in list order (the same sums
// in the same order as one thread walking the list, without its chain of
// dependent loads); beyond that, one thread walks the list.
constexpr int64_t kResidualParallel = 4096;
__global__ void gauge_residual_kernel(double* lam_h, const int64_t* cells, int64_t n, const double* value,
                                      const double* obs) {
    if (n > kResidualParallel) {
        if (blockIdx.x == 0 && threadIdx.x == 0)
            for (int64_t i = 0; i < n; ++i) lam_h[cells[i]] += 2.0 * (value[i] - obs[i]);
        return;
    }
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
        const int64_t c = cells[i];
        bool first = true;
        for (int64_t j = 0; j < i && first; ++j) first = cells[j] != c;
        if (!first) continue;
        double acc = lam_h[c];
        for (int64_t j = i; j < n; ++j)
            if (cells[j] == c) acc += 2.0 * (value[j] - obs[j]);
        lam_h[c] = acc;
    }
}

// J = sum over all entries of (value - obs)^2, one block, fixed order per thread
// then a fixed tree: deterministic from run to run
__global__ void misfit_kernel(const double* value, const double* obs, int64_t n, double* J) {
    __shared__ double part[256];
    double acc = 0.0;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
        const double r = value[i] - obs[i];
        acc += r * r;
    }
    part[threadIdx.x] = acc;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) part[threadIdx.x] += part[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) *J = part[0];
}

typedef void (*StepKernel)(StepArgs);

static StepKernel kernel_for(int solver) {
    switch (solver) {
        case FWAVE: return step_kernel<FWAVE>;
        case AUG_RIEMANN: return step_kernel<AUG_RIEMANN>;
        case LF: return step_kernel<LF>;
        case LF_BATH: return step_kernel<LF_BATH>;
        case LLF: return step_kernel<LLF>;
        case LLF_BATH: return step_kernel<LLF_BATH>;
        default: return nullptr;
    }
}

static void* cross_kernel_for(int solver) {
    switch (solver) {
        case FWAVE: return (void*)cross_edges_kernel<FWAVE>;
        case AUG_RIEMANN: return (void*)cross_edges_kernel<AUG_RIEMANN>;
        case LF: return (void*)cross_edges_kernel<LF>;
        case LF_BATH: return (void*)cross_edges_kernel<LF_BATH>;
        case LLF: return (void*)cross_edges_kernel<LLF>;
        case LLF_BATH: return (void*)cross_edges_kernel<LLF_BATH>;
        default: return nullptr;
    }
}

void* fma_step_kernel(int solver);
void* fma_cross_kernel(int solver);
cudaError_t fma_upload_tables();

static int upload_tables() {
    // __constant__ symbols are per device: every context uploads for its device
    double leg[kMaxDepth + 2], vol[kMaxDepth + 1], nrm[17][3][2];
    geometry_tables(leg, vol, nrm);
    CUDA_TRY(cudaMemcpyToSymbol(c_leg, leg, sizeof(leg)));
    CUDA_TRY(cudaMemcpyToSymbol(c_vol, vol, sizeof(vol)));
    CUDA_TRY(cudaMemcpyToSymbol(c_normal, nrm, sizeof(nrm)));
    CUDA_TRY(fma_upload_tables());
    return SWE_OK;
}

}  // namespace swe

using namespace swe;

struct swe_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t own_stream = nullptr;
    int num_sms = 0;
    // instances
    std::vector<HostMesh> mesh;
    std::vector<swe_params> params;
    std::vector<int64_t> offset;   // device cell offset of each instance (even)
    int64_t cells_total = 0;       // padded length of the device arrays
    int64_t cells_packed = 0;      // sum of the instances' cells (host layout)
    bool has_mesh = false, has_state = false;
    // tiling
    // 384 x 128 until the caller sets a tiling: the best on GB300 where most water
    // is at rest (2^26 basin 1.16e10 against 1.07e10 at 512; 2^22 adjoint step
    // 1.15 against 1.17 ms), within 2 % of 512 where it moves (2^22 bowls).
    // Meshes below 2^20 cells get 256-cell segments: with more cells per segment a
    // 2^18-cell mesh has too few segments for the ~600 resident CTAs, and a step
    // takes two segment-times (measured at 2^18: forward step 0.170 -> 0.145 ms,
    // adjoint step 0.242 -> 0.222 ms against 512).
    int32_t seg_cells = 384, block_threads = 128;
    bool tiling_set = false;
    int32_t stage_depth = 1;                        // segments staged ahead per CTA (1 or 2)
    int32_t arith = SWE_ARITH_STRICT;
    int32_t cross_mode = SWE_CROSS_AUTO;
    int32_t seg_order_mode = SWE_ORDER_AUTO;
    int32_t inject = SWE_INJECT_NONE;               // test-only device fault injection
    int64_t n_seg = 0, n_tasks = 0;
    int grid = 0, max_ndepth = 1;
    size_t smem = 0;
    // device memory
    double* h[2] = {nullptr, nullptr};
    double* hu[2] = {nullptr, nullptr};
    double* hv[2] = {nullptr, nullptr};
    double* b = nullptr;
    int8_t* depth = nullptr;
    int8_t* flags = nullptr;
    Task* tasks = nullptr;
    Task* xtasks = nullptr;         // cross-segment edges
    double* xflux = nullptr;        // their updates, [n_xtasks][2][4]
    int64_t n_xtasks = 0;
    long long* seg_ptr = nullptr;
    SegInfo* seg_info = nullptr;
    int32_t* seg_order = nullptr;   // hand-out order of the segments (spread over each instance's domain)
    InstParams* ip = nullptr;
    InstScalars* is = nullptr;
    GlobalScalars* gs = nullptr;
    double* dt_seq = nullptr;
    int64_t dt_seq_len = 0;
    std::vector<double> dt_seq_host;
    uint8_t* branch = nullptr;      // wet/dry branch flags of the last forward step (adjoint)
    // per cell (d, sqrt(g d)) of the last depth the step kernel took a square root of: a
    // cache of a function of d (any entry is a valid pair, so nothing ever invalidates it;
    // all bits set, a NaN key, when allocated)
    double2* memo = nullptr;
    // allocated sizes (elements) of the per-cell, per-instance and task buffers: a re-upload that
    // fits reuses them, so remeshing every step does not pay cudaMalloc / cudaFree each time
    size_t cap_cells = 0, cap_inst = 0, cap_tasks = 0, cap_segs = 0, cap_xtasks = 0;
    // host mirror of the device step counter and dt-sequence base: every change
    // goes through this library (launches, graph replays, restores), so the host
    // knows the traversal parity without reading the device
    long long step_mirror = 0, seq_base_mirror = 0;
    bool capturing = false;
    std::vector<InstParams> ip_host;
    int adj_grid = 0;               // adjoint launch shape for the current tiling (0 = not configured)
    int32_t adj_seg_cells = 0;
    int adj_solver = 0;
    // CUDA graphs of n steps
    std::map<int64_t, cudaGraphExec_t> graphs;
    double leg[kMaxDepth + 2], vol[kMaxDepth + 1], nrm[17][3][2];
};

namespace {

int n_inst(const swe_ctx* c) { return (int)c->mesh.size(); }

void drop_graphs(swe_ctx* c) {
    for (auto& kv : c->graphs) cudaGraphExecDestroy(kv.second);
    c->graphs.clear();
}

// Forget the mesh: graphs, the frozen dt sequence and the adjoint's branch
// buffer always go; the cell, instance and task buffers are released only with
// `release` (else kept for a re-upload that fits them).
void free_mesh_buffers(swe_ctx* c, bool release = true) {
    drop_graphs(c);
    cudaFree(c->dt_seq); cudaFree(c->branch);
    c->branch = nullptr;
    c->dt_seq = nullptr;
    c->dt_seq_len = 0;
    c->dt_seq_host.clear();
    c->has_mesh = c->has_state = false;
    if (!release) return;
    for (int k = 0; k < 2; ++k) {
        cudaFree(c->h[k]); cudaFree(c->hu[k]); cudaFree(c->hv[k]);
        c->h[k] = c->hu[k] = c->hv[k] = nullptr;
    }
    cudaFree(c->b); cudaFree(c->depth); cudaFree(c->flags); cudaFree(c->tasks); cudaFree(c->seg_ptr);
    cudaFree(c->seg_info); cudaFree(c->seg_order); cudaFree(c->ip); cudaFree(c->is); cudaFree(c->xtasks); cudaFree(c->xflux);
    cudaFree(c->memo);
    c->memo = nullptr;
    c->b = nullptr; c->depth = nullptr; c->flags = nullptr; c->tasks = nullptr; c->seg_ptr = nullptr;
    c->seg_info = nullptr; c->seg_order = nullptr; c->ip = nullptr; c->is = nullptr; c->xtasks = nullptr; c->xflux = nullptr;
    c->n_xtasks = 0;
    c->cap_cells = c->cap_inst = c->cap_tasks = c->cap_segs = c->cap_xtasks = 0;
}

int device_alloc(void** p, size_t bytes) {
    cudaError_t e = cudaMalloc(p, bytes ? bytes : 16);
    if (e != cudaSuccess) {
        cudaGetLastError();
        *p = nullptr;
        return set_error(SWE_E_NOMEM, "cudaMalloc(%zu) failed: %s", bytes, cudaGetErrorString(e));
    }
    return SWE_OK;
}

size_t smem_bytes_for(int64_t seg_cells, int stage_depth, int max_ndepth) {
    // staging [depth][4][T], RN(1/depth) and sqrt(g depth) [2][T], edge slots [12][T], depth tables [6][nd]
    return (size_t)(14 + 4 * stage_depth) * (size_t)seg_cells * sizeof(double) + (size_t)6 * max_ndepth * sizeof(double);
}

size_t smem_bytes(const swe_ctx* c) { return smem_bytes_for(c->seg_cells, c->stage_depth, c->max_ndepth); }

constexpr size_t kMaxSmem = 227 * 1024;

int check_params(const swe_params* p) {
    if (!kernel_for(p->solver)) return set_error(SWE_E_INVALID, "unknown solver %d", p->solver);
    if (p->bc < SWE_BC_OUTFLOW || p->bc > SWE_BC_NOSLIP) return set_error(SWE_E_INVALID, "unknown bc %d", p->bc);
    if (!(p->scaling > 0.0)) return set_error(SWE_E_INVALID, "scaling must be > 0");
    if (!(p->dry_tolerance >= 0.0)) return set_error(SWE_E_INVALID, "dry tolerance must be >= 0");
    if (p->min_depth < 0 || p->max_depth > kMaxDepth || p->min_depth > p->max_depth)
        return set_error(SWE_E_INVALID, "depth limits %d..%d invalid", p->min_depth, p->max_depth);
    return SWE_OK;
}

int upload_inst_params(swe_ctx* c) {
    const int n = n_inst(c);
    std::vector<InstParams> v((size_t)n);
    for (int i = 0; i < n; ++i) {
        const swe_params& p = c->params[(size_t)i];
        InstParams& q = v[(size_t)i];
        q.drytol = p.dry_tolerance;
        q.courant = p.courant;
        q.scaling = p.scaling;
        // refinement_threshold * scaling * get_edge_size(dmax) (src/SWE/SWE_euler_timestep.f90:339,342)
        q.thr_refine = (5.0 * p.scaling) * c->leg[p.max_depth + 1];
        q.thr_coarsen = q.thr_refine / 8.0;
        q.max_time = p.max_time;
        q.tout = p.output_time_step;
        q.min_depth = p.min_depth;
        q.max_depth = p.max_depth;
        q.dmin = c->mesh[(size_t)i].min_depth;
        q.ndepth = c->mesh[(size_t)i].max_depth - c->mesh[(size_t)i].min_depth + 1;
        q.bc = p.bc;
        // RN(scaling^2) * 2^-(d+1) must stay a normal number for the deepest cell
        const double v0 = p.scaling * p.scaling;
        const int dmax = c->mesh[(size_t)i].max_depth;
        q.dt_by_max = (std::isfinite(v0) && v0 > 0.0 && std::ldexp(v0, -(dmax + 1)) >= DBL_MIN) ? 1 : 0;
    }
    CUDA_TRY(cudaMemcpyAsync(c->ip, v.data(), sizeof(InstParams) * v.size(), cudaMemcpyHostToDevice, c->stream));
    c->ip_host = v;
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    return SWE_OK;
}

// A kernel's dynamic shared-memory limit is an attribute of the function, shared
// by every context of the process: contexts with different tilings only ever
// raise it (the limit does not change the resources of a launch that asks for
// less), so a context never finds it lowered by another.
int raise_smem_limit(const void* k, size_t bytes) {
    static std::mutex mu;
    std::lock_guard<std::mutex> lock(mu);
    cudaFuncAttributes fa;
    CUDA_TRY(cudaFuncGetAttributes(&fa, k));
    if ((size_t)fa.maxDynamicSharedSizeBytes < bytes)
        CUDA_TRY(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
    return SWE_OK;
}

int configure_launch(swe_ctx* c) {
    c->smem = smem_bytes(c);
    StepKernel k = kernel_for(c->params.empty() ? FWAVE : c->params[0].solver);
    if (!k) return set_error(SWE_E_INVALID, "unknown solver");
    int rc;
    for (int s : {FWAVE, AUG_RIEMANN, LF, LF_BATH, LLF, LLF_BATH}) {
        if ((rc = raise_smem_limit((const void*)kernel_for(s), c->smem)) ||
            (rc = raise_smem_limit((const void*)fma_step_kernel(s), c->smem)))
            return rc;
    }
    if ((rc = raise_smem_limit((const void*)step_kernel<FWAVE, 1>, c->smem)) ||
        (rc = raise_smem_limit((const void*)step_kernel<FWAVE, 2>, c->smem)))
        return rc;
    int per_sm = 0;
    CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, c->block_threads, c->smem));
    if (per_sm < 1)
        return set_error(SWE_E_INVALID, "tiling %d cells x %d threads does not fit an SM", c->seg_cells,
                         c->block_threads);
    int64_t g = (int64_t)per_sm * c->num_sms;
    c->grid = (int)std::max<int64_t>(1, std::min<int64_t>(g, c->n_seg));
    drop_graphs(c);
    return SWE_OK;
}

// The order the step kernel hands segments out in: each instance's segments in
// bit-reversed order of their index (the reversal over the next power of two,
// skipping indices past the end), instances one after the other. The CTAs that
// run at one time then work on segments spread over the instance's domain, so
// an SM rarely holds only dry land (integer work, the FP64 pipe idle) or only
// wet cells. Results do not depend on the order: the step's reductions are a
// min, a max and an integer sum.
static std::vector<int32_t> spread_order(const std::vector<SegInfo>& seg_info) {
    std::vector<int32_t> order;
    order.reserve(seg_info.size());
    size_t s0 = 0;
    while (s0 < seg_info.size()) {
        size_t s1 = s0 + 1;
        while (s1 < seg_info.size() && seg_info[s1].inst == seg_info[s0].inst) ++s1;
        const uint64_t n = s1 - s0;
        int bits = 0;
        while (((uint64_t)1 << bits) < n) ++bits;
        for (uint64_t k = 0; k < ((uint64_t)1 << bits); ++k) {
            uint64_t r = 0;
            for (int i = 0; i < bits; ++i) r |= ((k >> i) & 1u) << (bits - 1 - i);
            if (r < n) order.push_back((int32_t)(s0 + r));
        }
        s0 = s1;
    }
    return order;
}

int rebuild_tasks(swe_ctx* c) {
    std::vector<int64_t> seg_ptr;
    std::vector<SegInfo> seg_info;
    hvec<Task> tasks, xtasks;
    for (int i = 0; i < n_inst(c); ++i) {
        int rc = build_tasks(c->mesh[(size_t)i], c->offset[(size_t)i], i, c->seg_cells, seg_ptr, seg_info, tasks,
                             xtasks);
        if (rc) return rc;
    }
    c->n_xtasks = (int64_t)xtasks.size();
    c->n_seg = (int64_t)seg_info.size();
    c->adj_seg_cells = 0;  // the adjoint's grid depends on the segment count
    c->n_tasks = (int64_t)tasks.size();
    if (c->n_seg >= ((int64_t)1 << 31)) return set_error(SWE_E_INVALID, "too many segments");
    int rc;
    if (tasks.size() > c->cap_tasks) {
        cudaFree(c->tasks);
        c->tasks = nullptr;
        c->cap_tasks = 0;
        const size_t cap = tasks.size() + tasks.size() / 8 + 64;
        if ((rc = device_alloc((void**)&c->tasks, sizeof(Task) * cap))) return rc;
        c->cap_tasks = cap;
    }
    if (seg_info.size() + 1 > c->cap_segs) {
        cudaFree(c->seg_ptr);
        cudaFree(c->seg_info);
        cudaFree(c->seg_order);
        c->seg_ptr = nullptr;
        c->seg_info = nullptr;
        c->seg_order = nullptr;
        c->cap_segs = 0;
        const size_t cap = seg_info.size() + seg_info.size() / 8 + 16;
        if ((rc = device_alloc((void**)&c->seg_ptr, sizeof(long long) * (cap + 1)))) return rc;
        if ((rc = device_alloc((void**)&c->seg_info, sizeof(SegInfo) * cap))) return rc;
        if ((rc = device_alloc((void**)&c->seg_order, sizeof(int32_t) * cap))) return rc;
        c->cap_segs = cap;
    }
    if (xtasks.size() > c->cap_xtasks) {
        cudaFree(c->xtasks);
        cudaFree(c->xflux);
        c->xtasks = nullptr;
        c->xflux = nullptr;
        c->cap_xtasks = 0;
        const size_t cap = xtasks.size() + xtasks.size() / 8 + 64;
        if ((rc = device_alloc((void**)&c->xtasks, sizeof(Task) * cap))) return rc;
        if ((rc = device_alloc((void**)&c->xflux, 8 * sizeof(double) * cap))) return rc;
        c->cap_xtasks = cap;
    }
    CUDA_TRY(cudaMemcpyAsync(c->tasks, tasks.data(), sizeof(Task) * tasks.size(), cudaMemcpyHostToDevice, c->stream));
    if (!xtasks.empty())
        CUDA_TRY(cudaMemcpyAsync(c->xtasks, xtasks.data(), sizeof(Task) * xtasks.size(), cudaMemcpyHostToDevice,
                                 c->stream));
    CUDA_TRY(cudaMemcpyAsync(c->seg_ptr, seg_ptr.data(), sizeof(long long) * seg_ptr.size(), cudaMemcpyHostToDevice,
                             c->stream));
    CUDA_TRY(cudaMemcpyAsync(c->seg_info, seg_info.data(), sizeof(SegInfo) * seg_info.size(),
                             cudaMemcpyHostToDevice, c->stream));
    const std::vector<int32_t> order = spread_order(seg_info);
    if (order.size() != seg_info.size()) return set_error(SWE_E_INVALID, "segment order is not a permutation");
    CUDA_TRY(cudaMemcpyAsync(c->seg_order, order.data(), sizeof(int32_t) * order.size(), cudaMemcpyHostToDevice,
                             c->stream));
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    return configure_launch(c);
}

int check_device_error(swe_ctx* c) {
    unsigned int err = 0;
    CUDA_TRY(cudaMemcpyAsync(&err, &c->gs->error, sizeof(err), cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    if (err) {
        // reported once: the flag is cleared so that the context steps on after
        // the caller has uploaded a state again (the failed step's is undefined)
        CUDA_TRY(cudaMemsetAsync(&c->gs->error, 0, sizeof(err), c->stream));
        CUDA_TRY(cudaStreamSynchronize(c->stream));
        return set_error(SWE_E_DEVICE, "step kernel reported error 0x%x (%s)", err,
                         (err & 2u) ? "TMA wait ran out" : "edge task index out of range");
    }
    return SWE_OK;
}

int current_index(swe_ctx* c, int* idx) {
    *idx = (int)(c->step_mirror & 1);
    return SWE_OK;
}

// Ingest and upload the instances' meshes (arrays concatenated, indices local to each instance).
int upload_meshes(swe_ctx* c, int64_t ni, const int64_t* n_cells, const int64_t* n_edges, const int64_t* n_bnd,
                  const int8_t* depth, const int8_t* plotter, const int64_t* edge_cells, const int8_t* edge_local,
                  const int64_t* bnd_cell, const int8_t* bnd_local) {
    if (ni < 1 || ni > (1 << 20)) return set_error(SWE_E_INVALID, "instance count %lld", (long long)ni);
    if (!n_cells || !n_edges || !n_bnd) return set_error(SWE_E_INVALID, "null size arrays");
    cudaSetDevice(c->device);
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    free_mesh_buffers(c, false);
    std::vector<HostMesh> meshes((size_t)ni);
    std::vector<int64_t> offset((size_t)ni);
    int64_t pc = 0, pe = 0, pb = 0, off = 0;
    int dmin = kMaxDepth, dmax = 0, max_nd = 1;
    for (int64_t i = 0; i < ni; ++i) {
        int rc = ingest_mesh(meshes[(size_t)i], n_cells[i], depth + pc, plotter + pc, n_edges[i],
                             edge_cells ? edge_cells + 2 * pe : nullptr, edge_local ? edge_local + 2 * pe : nullptr,
                             n_bnd[i], bnd_cell ? bnd_cell + pb : nullptr, bnd_local ? bnd_local + pb : nullptr);
        if (rc) {
            char why[512];
            snprintf(why, sizeof(why), "%s", g_err);
            return set_error(rc, "instance %lld: %s", (long long)i, why);
        }
        offset[(size_t)i] = off;
        off += (n_cells[i] + 1) & ~(int64_t)1;
        pc += n_cells[i];
        pe += n_edges[i];
        pb += n_bnd[i];
        dmin = std::min(dmin, meshes[(size_t)i].min_depth);
        dmax = std::max(dmax, meshes[(size_t)i].max_depth);
        max_nd = std::max(max_nd, meshes[(size_t)i].max_depth - meshes[(size_t)i].min_depth + 1);
    }
    if (off >= ((int64_t)1 << 31) - 1) return set_error(SWE_E_INVALID, "total cells %lld >= 2^31", (long long)off);
    c->mesh.swap(meshes);
    c->offset.swap(offset);
    c->cells_total = off;
    c->cells_packed = pc;
    if (!c->tiling_set) c->seg_cells = off < ((int64_t)1 << 20) ? 256 : 384;
    c->max_ndepth = max_nd;
    swe_params p0 = c->params.empty() ? swe_params{} : c->params[0];
    c->params.assign((size_t)ni, p0);
    const size_t n = (size_t)off;
    int rc = SWE_OK;
    if (n > c->cap_cells || (size_t)ni > c->cap_inst) {  // grow (with headroom for a remesh that refines)
        free_mesh_buffers(c, true);
        const size_t cap = n + n / 8 + 64, capi = (size_t)ni;
        for (int k = 0; k < 2 && !rc; ++k)
            if ((rc = device_alloc((void**)&c->h[k], cap * 8)) || (rc = device_alloc((void**)&c->hu[k], cap * 8)) ||
                (rc = device_alloc((void**)&c->hv[k], cap * 8)))
                break;
        if (!rc && !(rc = device_alloc((void**)&c->b, cap * 8)) && !(rc = device_alloc((void**)&c->depth, cap)) &&
            !(rc = device_alloc((void**)&c->flags, cap)) && !(rc = device_alloc((void**)&c->ip, sizeof(InstParams) * capi)) &&
            !(rc = device_alloc((void**)&c->memo, cap * sizeof(double2))))
            rc = device_alloc((void**)&c->is, sizeof(InstScalars) * capi);
        if (rc) {
            free_mesh_buffers(c);
            return rc;
        }
        CUDA_TRY(cudaMemsetAsync(c->memo, 0xff, cap * sizeof(double2), c->stream));
        c->cap_cells = cap;
        c->cap_inst = capi;
    }
    // zero the padding cells; copy depths per instance
    for (int k = 0; k < 2; ++k) {
        CUDA_TRY(cudaMemsetAsync(c->h[k], 0, n * 8, c->stream));
        CUDA_TRY(cudaMemsetAsync(c->hu[k], 0, n * 8, c->stream));
        CUDA_TRY(cudaMemsetAsync(c->hv[k], 0, n * 8, c->stream));
    }
    CUDA_TRY(cudaMemsetAsync(c->b, 0, n * 8, c->stream));
    CUDA_TRY(cudaMemsetAsync(c->depth, 0, n, c->stream));
    CUDA_TRY(cudaMemsetAsync(c->flags, 0, n, c->stream));
    for (int64_t i = 0; i < ni; ++i)
        CUDA_TRY(cudaMemcpyAsync(c->depth + c->offset[(size_t)i], c->mesh[(size_t)i].depth.data(),
                                 (size_t)c->mesh[(size_t)i].n_cells, cudaMemcpyHostToDevice, c->stream));
    c->has_mesh = true;
    if ((rc = upload_inst_params(c)) || (rc = rebuild_tasks(c))) {
        free_mesh_buffers(c);
        return rc;
    }
    reset_scalars_kernel<<<(int)((ni + 255) / 256), 256, 0, c->stream>>>(c->is, c->gs, (int)ni);
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    c->step_mirror = 0;
    c->seq_base_mirror = 0;
    return SWE_OK;
}

// host packed layout <-> device padded layout
int copy_state(swe_ctx* c, int to_device, double* h, double* hu, double* hv, double* b) {
    int k, rc;
    if ((rc = current_index(c, &k))) return rc;
    int64_t p = 0;
    for (int i = 0; i < n_inst(c); ++i) {
        const size_t bytes = (size_t)c->mesh[(size_t)i].n_cells * 8;
        const int64_t o = c->offset[(size_t)i];
        double* dev[4] = {c->h[k] + o, c->hu[k] + o, c->hv[k] + o, c->b + o};
        double* host[4] = {h ? h + p : nullptr, hu ? hu + p : nullptr, hv ? hv + p : nullptr, b ? b + p : nullptr};
        for (int q = 0; q < 4; ++q) {
            if (!host[q]) continue;
            if (to_device)
                CUDA_TRY(cudaMemcpyAsync(dev[q], host[q], bytes, cudaMemcpyHostToDevice, c->stream));
            else
                CUDA_TRY(cudaMemcpyAsync(host[q], dev[q], bytes, cudaMemcpyDeviceToHost, c->stream));
        }
        p += c->mesh[(size_t)i].n_cells;
    }
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    return SWE_OK;
}

// io: optional caller buffers {h, hu, hv, h_out, hu_out, hv_out} (device-accessible
// addresses), b and flags: optional replacements of the context's arrays.
// fz: 0 a plain step; 1 records every edge decision into erec (and the cells'
// fixes into branch); 2 replays them (the f-wave only).
int launch_steps(swe_ctx* c, int64_t n_steps, uint8_t* branch = nullptr, double* const* io = nullptr,
                 const double* b = nullptr, int8_t* flags = nullptr, int use_tma = 1, int fz = 0,
                 uint16_t* erec = nullptr) {
    StepArgs A;
    A.branch = branch;
    for (int k = 0; k < 2; ++k) {
        A.h[k] = c->h[k];
        A.hu[k] = c->hu[k];
        A.hv[k] = c->hv[k];
    }
    A.b = c->b;
    A.depth = c->depth;
    A.flags = c->flags;
    A.tasks = reinterpret_cast<const int4*>(c->tasks);
    A.seg_ptr = c->seg_ptr;
    A.seg_info = reinterpret_cast<const int4*>(c->seg_info);
    // AUTO: spread from 2048 segments on; on fewer (a step of one or two waves of
    // CTAs) the curve order measured faster (2^18-cell bowl: 0.167 against 0.172 ms)
    const bool spread = c->seg_order_mode == SWE_ORDER_SPREAD ||
                        (c->seg_order_mode == SWE_ORDER_AUTO && c->n_seg >= 2048);
    A.seg_order = spread ? c->seg_order : nullptr;
    A.xtasks = reinterpret_cast<const int4*>(c->xtasks);
    A.xflux = c->xflux;
    A.n_xtasks = c->n_xtasks;
    A.ip = c->ip;
    A.is = c->is;
    A.gs = c->gs;
    A.dt_seq = c->dt_seq;
    A.dt_seq_len = c->dt_seq_len;
    A.n_seg = (int32_t)c->n_seg;
    A.n_inst = n_inst(c);
    A.seg_cells = c->seg_cells;
    A.max_ndepth = c->max_ndepth;
    A.n_cells_total = (int32_t)c->cells_total;
    A.use_tma = use_tma;
    A.stage_depth = c->stage_depth;
    A.fixed_io = 0;
    // fault injection (tests): the staging barrier expects 16 bytes that no copy
    // delivers, so its phase never completes and the bounded wait, shortened to
    // 20 ms, gives up; every issued copy still lands before the CTA leaves
    A.memo = c->memo;
    A.extra_tx = c->inject == SWE_INJECT_STAGING_TX ? 16u : 0u;
    A.wait_ns = c->inject == SWE_INJECT_STAGING_TX ? 20000000ull : kWaitNs;
    // edges between two segments: a pass before the step kernel for device-resident
    // steps; solved by both segments' CTAs when the state is in host memory (the
    // pass's scattered reads of host memory cost more than the duplicated solves)
    const bool pass = c->n_xtasks > 0 && (c->cross_mode == SWE_CROSS_PASS || (c->cross_mode == SWE_CROSS_AUTO && !io));
    A.halo_solve = pass ? 0 : 1;
    if (io) {
        A.h[0] = io[0]; A.hu[0] = io[1]; A.hv[0] = io[2];
        A.h[1] = io[3]; A.hu[1] = io[4]; A.hv[1] = io[5];
        A.fixed_io = 1;
    }
    if (b) A.b = b;
    if (flags) A.flags = flags;
    // the adjoint's forward step (branch output) always runs the strict kernel,
    // so its branches are the ones the reverse sweep re-evaluates
    const bool fma = c->arith == SWE_ARITH_FMA && !branch;
    void* k = fma ? fma_step_kernel(c->params[0].solver) : (void*)kernel_for(c->params[0].solver);
    void* kx = fma ? fma_cross_kernel(c->params[0].solver) : cross_kernel_for(c->params[0].solver);
    A.erec = erec;
    A.xrec = erec ? erec + c->n_tasks : nullptr;
    if (fz == 1) {
        k = (void*)step_kernel<FWAVE, 1>;
        kx = (void*)cross_edges_kernel<FWAVE, 1>;
    } else if (fz == 2) {
        k = (void*)step_kernel<FWAVE, 2>;
        kx = (void*)cross_edges_kernel<FWAVE, 2>;
    }
    // the cross-edge pass waits mostly on its scattered cell reads: 128-thread CTAs
    // (90 registers) fit 5 per SM, 20 warps, against 2 CTAs of 256 threads
    constexpr int kCrossThreads = 128;
    const unsigned xblocks = pass ? (unsigned)((c->n_xtasks + kCrossThreads - 1) / kCrossThreads) : 0u;
    void* args[] = {&A};
    for (int64_t s = 0; s < n_steps; ++s) {
        if (xblocks) CUDA_TRY(cudaLaunchKernel(kx, dim3(xblocks), dim3(kCrossThreads), args, 0, c->stream));
        CUDA_TRY(cudaLaunchKernel(k, dim3(c->grid), dim3(c->block_threads), args, c->smem, c->stream));
        if (!c->capturing) ++c->step_mirror;
    }
    return SWE_OK;
}

int ready(swe_ctx* c) {
    if (!c) return set_error(SWE_E_INVALID, "null context");
    if (!c->has_mesh) return set_error(SWE_E_NOMESH, "upload a mesh first");
    if (!c->has_state) return set_error(SWE_E_STATE, "upload a state first");
    return SWE_OK;
}

}  // namespace

extern "C" {

int swe_last_error(char* buf, size_t n) {
    if (!buf || n == 0) return SWE_E_INVALID;
    snprintf(buf, n, "%s", g_err);
    return SWE_OK;
}

int swe_create(swe_ctx** out, int device) {
    if (!out) return set_error(SWE_E_INVALID, "null context pointer");
    *out = nullptr;
    int ndev = 0;
    CUDA_TRY(cudaGetDeviceCount(&ndev));
    if (device < 0 || device >= ndev) return set_error(SWE_E_INVALID, "device %d of %d", device, ndev);
    CUDA_TRY(cudaSetDevice(device));
    int rc = upload_tables();
    if (rc) return rc;
    swe_ctx* c = new swe_ctx();
    c->device = device;
    cudaError_t e = cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete c;
        return set_error(SWE_E_CUDA, "stream: %s", cudaGetErrorString(e));
    }
    c->stream = c->own_stream;
    cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device);
    if ((rc = device_alloc((void**)&c->gs, sizeof(GlobalScalars)))) {
        cudaStreamDestroy(c->own_stream);
        delete c;
        return rc;
    }
    cudaMemsetAsync(c->gs, 0, sizeof(GlobalScalars), c->stream);
    geometry_tables(c->leg, c->vol, c->nrm);
    swe_params p;
    p.solver = SWE_SOLVER_FWAVE;
    p.bc = SWE_BC_OUTFLOW;
    p.dry_tolerance = 0.01;
    p.courant = 0.45;
    p.scaling = 1.0;
    p.min_depth = 0;
    p.max_depth = 14;
    p.max_time = -1.0;
    p.output_time_step = -1.0;
    c->params.assign(1, p);
    e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) {
        swe_destroy(c);
        return set_error(SWE_E_CUDA, "init: %s", cudaGetErrorString(e));
    }
    *out = c;
    return SWE_OK;
}

int swe_destroy(swe_ctx* c) {
    if (!c) return SWE_OK;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    free_mesh_buffers(c);
    cudaFree(c->gs);
    if (c->own_stream) cudaStreamDestroy(c->own_stream);
    delete c;
    return SWE_OK;
}

int swe_set_stream(swe_ctx* c, void* stream) {
    if (!c) return set_error(SWE_E_INVALID, "null context");
    c->stream = stream ? (cudaStream_t)stream : c->own_stream;
    drop_graphs(c);
    return SWE_OK;
}

int swe_set_params(swe_ctx* c, const swe_params* p) {
    if (!c || !p) return set_error(SWE_E_INVALID, "null argument");
    int rc = check_params(p);
    if (rc) return rc;
    const int old_solver = c->params.empty() ? -1 : c->params[0].solver;
    c->params.assign(std::max<size_t>(1, c->mesh.size()), *p);
    if (!c->has_mesh) return SWE_OK;
    cudaSetDevice(c->device);
    if ((rc = upload_inst_params(c))) return rc;
    if (old_solver != p->solver) return configure_launch(c);
    return SWE_OK;
}

int swe_ensemble_set_params(swe_ctx* c, const swe_params* p) {
    if (!c || !p) return set_error(SWE_E_INVALID, "null argument");
    if (!c->has_mesh) return set_error(SWE_E_NOMESH, "upload the ensemble meshes first");
    const int ni = n_inst(c);
    for (int i = 0; i < ni; ++i) {
        int rc = check_params(&p[i]);
        if (rc) {
            char why[512];
            snprintf(why, sizeof(why), "%s", g_err);
            return set_error(rc, "instance %d: %s", i, why);
        }
        if (p[i].solver != p[0].solver)
            return set_error(SWE_E_INVALID, "all instances of an ensemble use one solver (instance %d differs)", i);
    }
    const int old_solver = c->params[0].solver;
    c->params.assign(p, p + ni);
    cudaSetDevice(c->device);
    int rc = upload_inst_params(c);
    if (rc) return rc;
    if (old_solver != p[0].solver) return configure_launch(c);
    return SWE_OK;
}

int swe_set_tiling(swe_ctx* c, int32_t seg_cells, int32_t block_threads) {
    if (!c) return set_error(SWE_E_INVALID, "null context");
    if (seg_cells && (seg_cells < 64 || seg_cells > 1536 || (seg_cells & 1)))
        return set_error(SWE_E_INVALID, "segment_cells %d: need an even value in 64..1536", seg_cells);
    if (block_threads && (block_threads < 64 || block_threads > 256 || (block_threads & 31)))
        return set_error(SWE_E_INVALID, "block_threads %d: need a multiple of 32 in 64..256", block_threads);
    if (seg_cells && smem_bytes_for(seg_cells, c->stage_depth, kMaxDepth + 1) > kMaxSmem)
        return set_error(SWE_E_INVALID, "segment_cells %d with staging depth %d exceeds shared memory", seg_cells,
                         c->stage_depth);
    if (seg_cells) {
        c->seg_cells = seg_cells;
        c->tiling_set = true;
    }
    if (block_threads) c->block_threads = block_threads;
    if (!c->has_mesh) return SWE_OK;
    cudaSetDevice(c->device);
    return rebuild_tasks(c);
}

int swe_set_staging(swe_ctx* c, int32_t depth) {
    if (!c) return set_error(SWE_E_INVALID, "null context");
    if (depth != 1 && depth != 2) return set_error(SWE_E_INVALID, "staging depth %d: need 1 or 2", depth);
    if (smem_bytes_for(c->seg_cells, depth, std::max(c->max_ndepth, kMaxDepth + 1)) > kMaxSmem)
        return set_error(SWE_E_INVALID, "staging depth %d with %d-cell segments exceeds shared memory", depth,
                         c->seg_cells);
    c->stage_depth = depth;
    if (!c->has_mesh) return SWE_OK;
    cudaSetDevice(c->device);
    return configure_launch(c);
}

int swe_set_arith(swe_ctx* c, int32_t mode) {
    if (!c) return set_error(SWE_E_INVALID, "null context");
    if (mode != SWE_ARITH_STRICT && mode != SWE_ARITH_FMA) return set_error(SWE_E_INVALID, "unknown arith mode %d", mode);
    c->arith = mode;
    drop_graphs(c);
    return SWE_OK;
}

int swe_get_tiling(swe_ctx* c, int32_t* seg_cells, int32_t* block_threads) {
    if (!c) return set_error(SWE_E_INVALID, "null context");
    if (seg_cells) *seg_cells = c->seg_cells;
    if (block_threads) *block_threads = c->block_threads;
    return SWE_OK;
}

int swe_set_cross_pass(swe_ctx* c, int32_t mode) {
    if (!c) return set_error(SWE_E_INVALID, "null context");
    if (mode < SWE_CROSS_AUTO || mode > SWE_CROSS_INKERNEL) return set_error(SWE_E_INVALID, "cross mode %d", mode);
    c->cross_mode = mode;
    drop_graphs(c);
    return SWE_OK;
}

int swe_set_segment_order(swe_ctx* c, int32_t mode) {
    if (!c) return set_error(SWE_E_INVALID, "null context");
    if (mode != SWE_ORDER_CURVE && mode != SWE_ORDER_SPREAD && mode != SWE_ORDER_AUTO)
        return set_error(SWE_E_INVALID, "segment order %d", mode);
    c->seg_order_mode = mode;
    drop_graphs(c);
    return SWE_OK;
}

int swe_get_task_counts(swe_ctx* c, int64_t* n_segments, int64_t* n_tasks, int64_t* n_cross_edges,
                        int32_t* launches_per_step) {
    if (!c) return set_error(SWE_E_INVALID, "null context");
    if (!c->has_mesh) return set_error(SWE_E_NOMESH, "upload a mesh first");
    if (n_segments) *n_segments = c->n_seg;
    if (n_tasks) *n_tasks = c->n_tasks;
    if (n_cross_edges) *n_cross_edges = c->n_xtasks;
    if (launches_per_step)
        *launches_per_step = (c->n_xtasks > 0 && c->cross_mode != SWE_CROSS_INKERNEL) ? 2 : 1;
    return SWE_OK;
}

int swe_mesh_upload(swe_ctx* c, int64_t n_cells, const int8_t* depth, const int8_t* plotter, int64_t n_edges,
                    const int64_t* edge_cells, const int8_t* edge_local, int64_t n_bnd, const int64_t* bnd_cell,
                    const int8_t* bnd_local) {
    if (!c) return set_error(SWE_E_INVALID, "null context");
    return upload_meshes(c, 1, &n_cells, &n_edges, &n_bnd, depth, plotter, edge_cells, edge_local, bnd_cell,
                         bnd_local);
}

int swe_ensemble_mesh_upload(swe_ctx* c, int64_t n_instances, const int64_t* n_cells, const int64_t* n_edges,
                             const int64_t* n_bnd, const int8_t* depth, const int8_t* plotter,
                             const int64_t* edge_cells, const int8_t* edge_local, const int64_t* bnd_cell,
                             const int8_t* bnd_local) {
    if (!c) return set_error(SWE_E_INVALID, "null context");
    return upload_meshes(c, n_instances, n_cells, n_edges, n_bnd, depth, plotter, edge_cells, edge_local, bnd_cell,
                         bnd_local);
}

int swe_state_upload(swe_ctx* c, const double* h, const double* hu, const double* hv, const double* b) {
    if (!c || !h || !hu || !hv || !b) return set_error(SWE_E_INVALID, "null argument");
    if (!c->has_mesh) return set_error(SWE_E_NOMESH, "upload a mesh first");
    cudaSetDevice(c->device);
    int rc = copy_state(c, 1, const_cast<double*>(h), const_cast<double*>(hu), const_cast<double*>(hv),
                        const_cast<double*>(b));
    if (rc) return rc;
    c->has_state = true;
    return SWE_OK;
}

int swe_state_download(swe_ctx* c, double* h, double* hu, double* hv, double* b) {
    if (!c) return set_error(SWE_E_INVALID, "null context");
    if (!c->has_state) return set_error(SWE_E_STATE, "no state uploaded");
    cudaSetDevice(c->device);
    return copy_state(c, 0, h, hu, hv, b);
}

int swe_state_device(swe_ctx* c, double** h, double** hu, double** hv, const double** b) {
    if (!c) return set_error(SWE_E_INVALID, "null context");
    if (!c->has_mesh) return set_error(SWE_E_NOMESH, "upload a mesh first");
    cudaSetDevice(c->device);
    int k, rc;
    if ((rc = current_index(c, &k))) return rc;
    if (h) *h = c->h[k];
    if (hu) *hu = c->hu[k];
    if (hv) *hv = c->hv[k];
    if (b) *b = c->b;
    c->has_state = true;  // the caller may write the state in place
    return SWE_OK;
}

int swe_ensemble_set_time(swe_ctx* c, const double* time, const double* dt) {
    if (!c || !time || !dt) return set_error(SWE_E_INVALID, "null argument");
    if (!c->has_mesh) return set_error(SWE_E_NOMESH, "upload a mesh first");
    cudaSetDevice(c->device);
    const int ni = n_inst(c);
    double* tmp = nullptr;
    int rc = device_alloc((void**)&tmp, sizeof(double) * 2 * ni);
    if (rc) return rc;
    cudaError_t e = cudaMemcpyAsync(tmp, time, sizeof(double) * ni, cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(tmp + ni, dt, sizeof(double) * ni, cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) {
        set_times_kernel<<<(ni + 255) / 256, 256, 0, c->stream>>>(c->is, tmp, tmp + ni, ni);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    cudaFree(tmp);
    if (e != cudaSuccess) return set_error(SWE_E_CUDA, "set time: %s", cudaGetErrorString(e));
    return SWE_OK;
}

int swe_set_time(swe_ctx* c, double time, double dt) {
    if (!c) return set_error(SWE_E_INVALID, "null context");
    if (!c->has_mesh) return set_error(SWE_E_NOMESH, "upload a mesh first");
    std::vector<double> t((size_t)n_inst(c), time), d((size_t)n_inst(c), dt);
    return swe_ensemble_set_time(c, t.data(), d.data());
}

int swe_ensemble_get_time(swe_ctx* c, double* time, double* dt, double* dt_new) {
    if (!c) return set_error(SWE_E_INVALID, "null context");
    if (!c->has_mesh) return set_error(SWE_E_NOMESH, "upload a mesh first");
    cudaSetDevice(c->device);
    std::vector<InstScalars> s((size_t)n_inst(c));
    CUDA_TRY(cudaMemcpyAsync(s.data(), c->is, sizeof(InstScalars) * s.size(), cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    for (size_t i = 0; i < s.size(); ++i) {
        if (time) time[i] = s[i].time;
        if (dt) dt[i] = s[i].dt;
        if (dt_new) dt_new[i] = s[i].dt_new;
    }
    return SWE_OK;
}

int swe_get_time(swe_ctx* c, double* time, double* dt, double* dt_new) {
    if (!c) return set_error(SWE_E_INVALID, "null context");
    if (!c->has_mesh) return set_error(SWE_E_NOMESH, "upload a mesh first");
    std::vector<double> t((size_t)n_inst(c)), d(t.size()), dn(t.size());
    int rc = swe_ensemble_get_time(c, t.data(), d.data(), dn.data());
    if (rc) return rc;
    if (time) *time = t[0];
    if (dt) *dt = d[0];
    if (dt_new) *dt_new = dn[0];
    return SWE_OK;
}

int swe_traverse(swe_ctx* c, int64_t n_steps) {
    int rc = ready(c);
    if (rc) return rc;
    if (n_steps < 0) return set_error(SWE_E_INVALID, "n_steps < 0");
    cudaSetDevice(c->device);
    return launch_steps(c, n_steps);
}

}  // extern "C"

namespace {
// The address the device uses for a caller's array: device or managed memory
// as is, pinned host memory through its device alias, pageable host memory
// only where the device reads it coherently (pageable memory access).
int device_view(const swe_ctx* c, const void* p, const char* name, const void** out, bool* on_device) {
    cudaPointerAttributes at;
    cudaError_t e = cudaPointerGetAttributes(&at, p);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return set_error(SWE_E_INVALID, "%s: cannot query the pointer (%s)", name, cudaGetErrorString(e));
    }
    *on_device = false;
    if (at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged) {
        if (at.type == cudaMemoryTypeDevice && at.device != c->device)
            return set_error(SWE_E_INVALID, "%s is memory of device %d, the context runs on %d", name, at.device,
                             c->device);
        *out = p;
        *on_device = at.type == cudaMemoryTypeDevice;
        return SWE_OK;
    }
    if (at.type == cudaMemoryTypeHost) {
        if (!at.devicePointer) return set_error(SWE_E_INVALID, "%s: pinned memory without a device mapping", name);
        *out = at.devicePointer;
        return SWE_OK;
    }
    int pageable = 0;
    cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, c->device);
    if (!pageable)
        return set_error(SWE_E_INVALID, "%s is pageable host memory and device %d cannot read it; pin it "
                         "(cudaHostRegister) or pass device memory", name, c->device);
    *out = p;
    return SWE_OK;
}
}  // namespace

extern "C" {

int swe_step_host(swe_ctx* c, const double* h, const double* hu, const double* hv, const double* b, double* h_out,
                  double* hu_out, double* hv_out, int8_t* flags_out) {
    if (!c) return set_error(SWE_E_INVALID, "null context");
    if (!c->has_mesh) return set_error(SWE_E_NOMESH, "upload a mesh first");
    if (n_inst(c) != 1) return set_error(SWE_E_INVALID, "swe_step_host takes a single-instance context");
    if (!h || !hu || !hv || !h_out || !hu_out || !hv_out) return set_error(SWE_E_INVALID, "null state array");
    if (!b && !c->has_state) return set_error(SWE_E_STATE, "b = NULL needs an uploaded state (its bathymetry)");
    const int64_t n = c->mesh[0].n_cells;
    const double* in[3] = {h, hu, hv};
    const double* out[3] = {h_out, hu_out, hv_out};
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            if (in[i] < out[j] + n && out[j] < in[i] + n)
                return set_error(SWE_E_INVALID, "input and output arrays overlap");
    cudaSetDevice(c->device);
    const char* names[8] = {"h", "hu", "hv", "h_out", "hu_out", "hv_out", "b", "flags_out"};
    const void* dv[8] = {nullptr};
    const void* src[8] = {h, hu, hv, h_out, hu_out, hv_out, b, flags_out};
    bool all_dev = true;
    for (int i = 0; i < 8; ++i) {
        if (!src[i]) continue;
        bool od = false;
        int rc = device_view(c, src[i], names[i], &dv[i], &od);
        if (rc) return rc;
        all_dev = all_dev && od;
    }
    double* io[6];
    for (int i = 0; i < 6; ++i) io[i] = const_cast<double*>(static_cast<const double*>(dv[i]));
    // the 1-D bulk copies stage device memory from 16-byte aligned bases (every
    // segment starts at an even cell); host memory is read with plain loads
    bool aligned = true;
    for (int i = 0; i < 3; ++i) aligned = aligned && ((uintptr_t)dv[i] & 15u) == 0;
    aligned = aligned && (!dv[6] || ((uintptr_t)dv[6] & 15u) == 0) && (dv[6] || c->b);
    return launch_steps(c, 1, nullptr, io, static_cast<const double*>(dv[6]),
                        static_cast<int8_t*>(const_cast<void*>(dv[7])), (all_dev && aligned) ? 1 : 0);
}

int swe_traverse_graph(swe_ctx* c, int64_t n_steps) {
    int rc = ready(c);
    if (rc) return rc;
    if (n_steps < 1 || n_steps > 100000) return set_error(SWE_E_INVALID, "n_steps %lld out of 1..100000",
                                                          (long long)n_steps);
    cudaSetDevice(c->device);
    auto it = c->graphs.find(n_steps);
    if (it == c->graphs.end()) {
        cudaGraph_t g = nullptr;
        CUDA_TRY(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
        c->capturing = true;
        rc = launch_steps(c, n_steps);
        c->capturing = false;
        cudaError_t e = cudaStreamEndCapture(c->stream, &g);
        if (rc) {
            if (g) cudaGraphDestroy(g);
            return rc;
        }
        if (e != cudaSuccess) return set_error(SWE_E_CUDA, "graph capture: %s", cudaGetErrorString(e));
        cudaGraphExec_t x = nullptr;
        e = cudaGraphInstantiate(&x, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return set_error(SWE_E_CUDA, "graph instantiate: %s", cudaGetErrorString(e));
        it = c->graphs.emplace(n_steps, x).first;
    }
    CUDA_TRY(cudaGraphLaunch(it->second, c->stream));
    c->step_mirror += n_steps;
    return SWE_OK;
}

int swe_set_dt_sequence(swe_ctx* c, int64_t n_steps, const double* dts) {
    if (!c) return set_error(SWE_E_INVALID, "null context");
    if (!c->has_mesh) return set_error(SWE_E_NOMESH, "upload a mesh first");
    if (n_steps < 0 || (n_steps > 0 && !dts)) return set_error(SWE_E_INVALID, "bad dt sequence");
    cudaSetDevice(c->device);
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    cudaFree(c->dt_seq);
    c->dt_seq = nullptr;
    c->dt_seq_len = 0;
    drop_graphs(c);
    if (n_steps == 0) return SWE_OK;
    const size_t bytes = sizeof(double) * (size_t)n_steps * (size_t)n_inst(c);
    int rc = device_alloc((void**)&c->dt_seq, bytes);
    if (rc) return rc;
    CUDA_TRY(cudaMemcpyAsync(c->dt_seq, dts, bytes, cudaMemcpyHostToDevice, c->stream));
    c->dt_seq_host.assign(dts, dts + (size_t)n_steps * (size_t)n_inst(c));
    mark_seq_base_kernel<<<1, 1, 0, c->stream>>>(c->gs);
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    c->seq_base_mirror = c->step_mirror;
    c->dt_seq_len = n_steps;
    return SWE_OK;
}

int swe_snapshot_store(swe_ctx* c, double* h, double* hu, double* hv, int64_t* step) {
    int rc = ready(c);
    if (rc) return rc;
    if (n_inst(c) != 1) return set_error(SWE_E_INVALID, "snapshots are for single-instance contexts");
    if (!h || !hu || !hv) return set_error(SWE_E_INVALID, "null snapshot buffer");
    cudaSetDevice(c->device);
    const long long s = c->step_mirror;
    const int k = (int)(s & 1);
    const size_t bytes = (size_t)c->mesh[0].n_cells * 8;
    CUDA_TRY(cudaMemcpyAsync(h, c->h[k], bytes, cudaMemcpyDeviceToDevice, c->stream));
    CUDA_TRY(cudaMemcpyAsync(hu, c->hu[k], bytes, cudaMemcpyDeviceToDevice, c->stream));
    CUDA_TRY(cudaMemcpyAsync(hv, c->hv[k], bytes, cudaMemcpyDeviceToDevice, c->stream));
    if (step) *step = s;
    return SWE_OK;
}

int swe_snapshot_restore(swe_ctx* c, const double* h, const double* hu, const double* hv, int64_t step) {
    if (!c) return set_error(SWE_E_INVALID, "null context");
    if (!c->has_mesh) return set_error(SWE_E_NOMESH, "upload a mesh first");
    if (n_inst(c) != 1) return set_error(SWE_E_INVALID, "snapshots are for single-instance contexts");
    if (!h || !hu || !hv || step < 0) return set_error(SWE_E_INVALID, "bad snapshot");
    cudaSetDevice(c->device);
    const int k = (int)(step & 1);
    const size_t bytes = (size_t)c->mesh[0].n_cells * 8;
    CUDA_TRY(cudaMemcpyAsync(c->h[k], h, bytes, cudaMemcpyDeviceToDevice, c->stream));
    CUDA_TRY(cudaMemcpyAsync(c->hu[k], hu, bytes, cudaMemcpyDeviceToDevice, c->stream));
    CUDA_TRY(cudaMemcpyAsync(c->hv[k], hv, bytes, cudaMemcpyDeviceToDevice, c->stream));
    set_step_kernel<<<1, 1, 0, c->stream>>>(c->gs, (long long)step);
    CUDA_TRY(cudaGetLastError());
    c->step_mirror = step;
    c->has_state = true;
    return SWE_OK;
}

int swe_sample_gauges(swe_ctx* c, int64_t n_gauges, const int64_t* cells, double* out) {
    int rc = ready(c);
    if (rc) return rc;
    if (n_inst(c) != 1) return set_error(SWE_E_INVALID, "gauges are for single-instance contexts");
    if (n_gauges < 0 || (n_gauges > 0 && (!cells || !out))) return set_error(SWE_E_INVALID, "bad gauge arrays");
    if (n_gauges == 0) return SWE_OK;
    cudaSetDevice(c->device);
    const int blocks = (int)std::min<int64_t>((n_gauges + 127) / 128, 1024);
    gauge_kernel<<<blocks, 128, 0, c->stream>>>(c->gs, c->h[0], c->h[1], n_gauges, cells, c->mesh[0].n_cells, out);
    CUDA_TRY(cudaGetLastError());
    return SWE_OK;
}

int swe_traverse_gauges(swe_ctx* c, int64_t n_steps, int64_t n_gauges, const int64_t* cells, double* out) {
    int rc = ready(c);
    if (rc) return rc;
    if (n_inst(c) != 1) return set_error(SWE_E_INVALID, "gauges are for single-instance contexts");
    if (n_steps < 0 || n_gauges < 1 || !cells || !out) return set_error(SWE_E_INVALID, "bad gauge arrays");
    cudaSetDevice(c->device);
    const int blocks = (int)std::min<int64_t>((n_gauges + 127) / 128, 1024);
    for (int64_t s = 0; s < n_steps; ++s) {
        if ((rc = launch_steps(c, 1))) return rc;
        gauge_kernel<<<blocks, 128, 0, c->stream>>>(c->gs, c->h[0], c->h[1], n_gauges, cells, c->mesh[0].n_cells,
                                                    out + (size_t)s * (size_t)n_gauges);
        CUDA_TRY(cudaGetLastError());
    }
    return SWE_OK;
}

int swe_traverse_frozen(swe_ctx* c, int64_t n_steps, int32_t mode, uint8_t* branch, int64_t branch_stride,
                        uint16_t* edges, int64_t edge_stride, int64_t n_gauges, const int64_t* cells, double* out) {
    int rc = ready(c);
    if (rc) return rc;
    if (n_inst(c) != 1) return set_error(SWE_E_INVALID, "branch-frozen runs are for single-instance contexts");
    if (c->params[0].solver != SWE_SOLVER_FWAVE)
        return set_error(SWE_E_INVALID, "branch-frozen runs support the f-wave solver");
    if (mode != 1 && mode != 2) return set_error(SWE_E_INVALID, "mode %d (1 record, 2 replay)", mode);
    if (n_steps < 0 || (n_steps > 0 && (!branch || !edges)) || branch_stride < c->cells_total ||
        edge_stride < c->n_tasks + c->n_xtasks)
        return set_error(SWE_E_INVALID, "bad record buffers (strides must be >= %lld cells, %lld edges)",
                         (long long)c->cells_total, (long long)(c->n_tasks + c->n_xtasks));
    if (n_gauges < 0 || (n_gauges > 0 && (!cells || !out))) return set_error(SWE_E_INVALID, "bad gauge arrays");
    cudaSetDevice(c->device);
    const int blocks = (int)std::min<int64_t>((n_gauges + 127) / 128, 1024);
    for (int64_t s = 0; s < n_steps; ++s) {
        if ((rc = launch_steps(c, 1, branch + s * branch_stride, nullptr, nullptr, nullptr, 1, mode,
                               edges + s * edge_stride)))
            return rc;
        if (n_gauges > 0) {
            gauge_kernel<<<blocks, 128, 0, c->stream>>>(c->gs, c->h[0], c->h[1], n_gauges, cells, c->mesh[0].n_cells,
                                                        out + (size_t)s * (size_t)n_gauges);
            CUDA_TRY(cudaGetLastError());
        }
    }
    return SWE_OK;
}

int swe_traverse_branches(swe_ctx* c, int64_t n_steps, uint8_t* branch, int64_t stride) {
    int rc = ready(c);
    if (rc) return rc;
    if (n_steps < 0 || (n_steps > 0 && !branch) || stride < c->cells_total)
        return set_error(SWE_E_INVALID, "bad branch buffer (stride must be >= %lld)", (long long)c->cells_total);
    cudaSetDevice(c->device);
    for (int64_t s = 0; s < n_steps; ++s)
        if ((rc = launch_steps(c, 1, branch + s * stride))) return rc;
    return SWE_OK;
}

int swe_step_back(swe_ctx* c) {
    if (!c) return set_error(SWE_E_INVALID, "null context");
    if (!c->has_mesh) return set_error(SWE_E_NOMESH, "upload a mesh first");
    cudaSetDevice(c->device);
    const long long s = c->step_mirror;
    if (s < 1) return set_error(SWE_E_STATE, "no step to go back from");
    set_step_kernel<<<1, 1, 0, c->stream>>>(c->gs, s - 1);
    CUDA_TRY(cudaGetLastError());
    c->step_mirror = s - 1;
    return SWE_OK;
}

}  // extern "C"

namespace {
typedef void (*AdjKernel)(AdjointArgs);
// The reverse step for the solvers the adjoint differentiates (else null).
AdjKernel adjoint_kernel_for(int solver) {
    switch (solver) {
        case FWAVE: return adjoint_kernel<FWAVE>;
        case AUG_RIEMANN: return adjoint_kernel<AUG_RIEMANN>;
        case LF: return adjoint_kernel<LF>;
        case LF_BATH: return adjoint_kernel<LF_BATH>;
        case LLF: return adjoint_kernel<LLF>;
        case LLF_BATH: return adjoint_kernel<LLF_BATH>;
        default: return nullptr;
    }
}

// The reverse of step t (the context's state is x_t, parity t & 1).
int launch_adjoint(swe_ctx* c, long long t, const uint8_t* branch, const double* lam_h, const double* lam_hu,
                   const double* lam_hv, double* out_h, double* out_hu, double* out_hv, double* bbar) {
    const long long k = t - c->seq_base_mirror;
    AdjointArgs A;
    const int in = (int)(t & 1);
    A.h = c->h[in];
    A.hu = c->hu[in];
    A.hv = c->hv[in];
    A.b = c->b;
    A.depth = c->depth;
    A.branch = branch;
    A.lam_h = lam_h;
    A.lam_hu = lam_hu;
    A.lam_hv = lam_hv;
    A.out_h = out_h;
    A.out_hu = out_hu;
    A.out_hv = out_hv;
    A.bbar = bbar;
    A.tasks = reinterpret_cast<const int4*>(c->tasks);
    A.seg_ptr = c->seg_ptr;
    A.seg_info = reinterpret_cast<const int4*>(c->seg_info);
    A.P = c->ip_host[0];
    A.dt = c->dt_seq_host[(size_t)k];
    A.n_seg = (int32_t)c->n_seg;
    A.seg_cells = c->seg_cells;
    A.n_cells_total = (int32_t)c->cells_total;
    A.parity = (int32_t)(t & 1);
    A.error = &c->gs->error;
    A.memo = c->memo;
    {
        const double s2 = A.P.scaling * A.P.scaling;
        for (int d = 0; d <= kMaxDepth; ++d) A.ndv_tab[d] = -A.dt / (s2 * c->vol[d]);
        for (int d = 0; d <= kMaxDepth + 1; ++d) A.len_tab[d] = A.P.scaling * c->leg[d];
    }
    // the reverse kernel holds more registers per thread than the step: it runs
    // 256 threads per CTA so an SM still has two CTAs' worth of warps
    const int threads = 256;
    const size_t smem = (size_t)21 * c->seg_cells * sizeof(double);
    const int solver = c->params[0].solver;
    const AdjKernel kern = adjoint_kernel_for(solver);
    if (!kern) return set_error(SWE_E_INVALID, "the adjoint differentiates the f-wave, augmented and Lax-Friedrichs fluxes");
    if (c->adj_seg_cells != c->seg_cells || c->adj_solver != solver) {
        if (int rc = raise_smem_limit((const void*)kern, smem)) return rc;
        int per_sm = 0;
        CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem));
        if (per_sm < 1) return set_error(SWE_E_INVALID, "adjoint tiling does not fit an SM");
        c->adj_grid = (int)std::max<int64_t>(1, std::min<int64_t>((int64_t)per_sm * c->num_sms, c->n_seg));
        c->adj_seg_cells = c->seg_cells;
        c->adj_solver = solver;
    }
    kern<<<c->adj_grid, threads, smem, c->stream>>>(A);
    CUDA_TRY(cudaGetLastError());
    return SWE_OK;
}
}  // namespace

extern "C" {

int swe_adjoint_step(swe_ctx* c, const uint8_t* branch, const double* lam_h, const double* lam_hu,
                     const double* lam_hv, double* out_h, double* out_hu, double* out_hv, double* bbar) {
    int rc = ready(c);
    if (rc) return rc;
    if (n_inst(c) != 1) return set_error(SWE_E_INVALID, "the adjoint runs on single-instance contexts");
    if (!adjoint_kernel_for(c->params[0].solver))
        return set_error(SWE_E_INVALID, "the adjoint step differentiates the f-wave, augmented and Lax-Friedrichs fluxes");
    if (!lam_h || !lam_hu || !lam_hv || !out_h || !out_hu || !out_hv || !bbar)
        return set_error(SWE_E_INVALID, "null cotangent buffer");
    cudaSetDevice(c->device);
    const long long t = c->step_mirror, k = t - c->seq_base_mirror;
    if (!c->dt_seq || k < 0 || k >= c->dt_seq_len)
        return set_error(SWE_E_STATE, "the adjoint needs a frozen dt sequence covering step %lld", t);
    if (!branch) {
        // forward step t -> t+1 recording the branches; x_t stays in buffer t & 1
        if (!c->branch && (rc = device_alloc((void**)&c->branch, (size_t)c->cells_total))) return rc;
        if ((rc = launch_steps(c, 1, c->branch))) return rc;  // the context moves to step t + 1
        branch = c->branch;
    }
    return launch_adjoint(c, t, branch, lam_h, lam_hu, lam_hv, out_h, out_hu, out_hv, bbar);
}

int swe_ensemble_get_refinements(swe_ctx* c, int8_t* flags, int64_t* n_refinements) {
    if (!c) return set_error(SWE_E_INVALID, "null context");
    if (!c->has_mesh) return set_error(SWE_E_NOMESH, "upload a mesh first");
    cudaSetDevice(c->device);
    if (flags) {
        int64_t p = 0;
        for (int i = 0; i < n_inst(c); ++i) {
            CUDA_TRY(cudaMemcpyAsync(flags + p, c->flags + c->offset[(size_t)i], (size_t)c->mesh[(size_t)i].n_cells,
                                     cudaMemcpyDeviceToHost, c->stream));
            p += c->mesh[(size_t)i].n_cells;
        }
    }
    std::vector<InstScalars> s((size_t)n_inst(c));
    CUDA_TRY(cudaMemcpyAsync(s.data(), c->is, sizeof(InstScalars) * s.size(), cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    if (n_refinements)
        for (size_t i = 0; i < s.size(); ++i) n_refinements[i] = (int64_t)s[i].n_refine;
    return SWE_OK;
}

int swe_get_refinements(swe_ctx* c, int8_t* flags, int64_t* n_refinements) {
    if (!c) return set_error(SWE_E_INVALID, "null context");
    if (!c->has_mesh) return set_error(SWE_E_NOMESH, "upload a mesh first");
    std::vector<int64_t> nr((size_t)n_inst(c));
    int rc = swe_ensemble_get_refinements(c, flags, nr.data());
    if (rc) return rc;
    if (n_refinements) *n_refinements = nr[0];
    return SWE_OK;
}

int swe_get_step_count(swe_ctx* c, int64_t* steps) {
    if (!c || !steps) return set_error(SWE_E_INVALID, "null argument");
    cudaSetDevice(c->device);
    long long s = 0;
    CUDA_TRY(cudaMemcpyAsync(&s, &c->gs->step, sizeof(s), cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    *steps = s;
    return SWE_OK;
}

int swe_set_fault_injection(swe_ctx* c, int32_t kind) {
    if (!c) return set_error(SWE_E_INVALID, "null context");
    if (kind != SWE_INJECT_NONE && kind != SWE_INJECT_STAGING_TX)
        return set_error(SWE_E_INVALID, "unknown fault injection %d", kind);
    c->inject = kind;
    return SWE_OK;
}

int swe_synchronize(swe_ctx* c) {
    if (!c) return set_error(SWE_E_INVALID, "null context");
    cudaSetDevice(c->device);
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    return check_device_error(c);
}

int swe_mesh_validate(int64_t n_cells, const int8_t* depth, const int8_t* plotter, int64_t n_edges,
                      const int64_t* edge_cells, const int8_t* edge_local, int64_t n_bnd, const int64_t* bnd_cell,
                      const int8_t* bnd_local) {
    HostMesh m;
    return ingest_mesh(m, n_cells, depth, plotter, n_edges, edge_cells, edge_local, n_bnd, bnd_cell, bnd_local);
}

int swe_riemann_batch(int32_t solver, int64_t n, const double* normals, const double* q_left, const double* q_right,
                      double dry_tolerance, double* out_left, double* out_right) {
    if (n < 0 || (n > 0 && (!normals || !q_left || !q_right || !out_left || !out_right)))
        return set_error(SWE_E_INVALID, "bad arguments");
    if (n == 0) return SWE_OK;
    decltype(&riemann_batch_kernel<FWAVE>) k = nullptr;
    switch (solver) {
        case FWAVE: k = riemann_batch_kernel<FWAVE>; break;
        case AUG_RIEMANN: k = riemann_batch_kernel<AUG_RIEMANN>; break;
        case LF: k = riemann_batch_kernel<LF>; break;
        case LF_BATH: k = riemann_batch_kernel<LF_BATH>; break;
        case LLF: k = riemann_batch_kernel<LLF>; break;
        case LLF_BATH: k = riemann_batch_kernel<LLF_BATH>; break;
        default: return set_error(SWE_E_INVALID, "unknown solver %d", solver);
    }
    int rc = upload_tables();
    if (rc) return rc;
    double* d = nullptr;
    if ((rc = device_alloc((void**)&d, (size_t)n * 18 * sizeof(double)))) return rc;
    double *dn = d, *dl = d + 2 * n, *dr = d + 6 * n, *ol = d + 10 * n, *orr = d + 14 * n;
    cudaError_t e = cudaMemcpy(dn, normals, 16 * (size_t)n, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dl, q_left, 32 * (size_t)n, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dr, q_right, 32 * (size_t)n, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        int blocks = (int)std::min<int64_t>((n + 127) / 128, 4096);
        k<<<blocks, 128>>>(n, dn, dl, dr, dry_tolerance, ol, orr);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(out_left, ol, 32 * (size_t)n, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(out_right, orr, 32 * (size_t)n, cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) return set_error(SWE_E_CUDA, "riemann batch: %s", cudaGetErrorString(e));
    return SWE_OK;
}

int swe_division_check(int64_t n, uint64_t seed, int32_t exponent_span, int64_t* mismatches) {
    if (n < 0 || !mismatches || exponent_span < 0 || exponent_span > 1022)
        return set_error(SWE_E_INVALID, "bad arguments");
    *mismatches = 0;
    if (n == 0) return SWE_OK;
    unsigned long long* d = nullptr;
    int rc = device_alloc((void**)&d, sizeof(unsigned long long));
    if (rc) return rc;
    cudaError_t e = cudaMemset(d, 0, sizeof(unsigned long long));
    if (e == cudaSuccess) {
        division_check_kernel<<<1216, 256>>>(n, (unsigned long long)seed, exponent_span, d);
        e = cudaGetLastError();
    }
    unsigned long long got = 0;
    if (e == cudaSuccess) e = cudaMemcpy(&got, d, sizeof(got), cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) return set_error(SWE_E_CUDA, "division check: %s", cudaGetErrorString(e));
    *mismatches = (int64_t)got;
    return SWE_OK;
}

int swe_mesh_uniform_vertices(int32_t depth, double* vertices) {
    if (!vertices) return set_error(SWE_E_INVALID, "null vertex array");
    int64_t n = 0, ne = 0, nb = 0;
    int rc = mesh_uniform(depth, &n, &ne, &nb, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr);
    if (rc) return rc;
    std::vector<int8_t> d((size_t)n), p((size_t)n), el((size_t)(2 * ne)), bl((size_t)nb);
    std::vector<int64_t> ec((size_t)(2 * ne)), bc((size_t)nb);
    return mesh_uniform(depth, &n, &ne, &nb, d.data(), p.data(), ec.data(), el.data(), bc.data(), bl.data(), nullptr,
                        vertices);
}

int swe_mesh_uniform(int32_t depth, int64_t* n_cells, int64_t* n_edges, int64_t* n_bnd, int8_t* depth_out,
                     int8_t* plotter_out, int64_t* edge_cells, int8_t* edge_local, int64_t* bnd_cell,
                     int8_t* bnd_local, double* centroids) {
    return mesh_uniform(depth, n_cells, n_edges, n_bnd, depth_out, plotter_out, edge_cells, edge_local, bnd_cell,
                        bnd_local, centroids);
}

}  // extern "C"

namespace {

// min(C(n, k), cap + 1), exactly (every partial product C(n - k + i, i) is an integer)
int64_t binom_capped(int64_t n, int64_t k, int64_t cap) {
    if (k < 0 || k > n) return 0;
    k = std::min(k, n - k);
    unsigned __int128 v = 1;
    for (int64_t i = 1; i <= k; ++i) {
        v = v * (unsigned __int128)(n - k + i) / (unsigned __int128)i;
        if (v > (unsigned __int128)cap) return cap + 1;
    }
    return (int64_t)v;
}

// First checkpoint offset for reversing `length` steps with the start state held
// and `free` more slots (revolve's offline rule, the same as adjoint.py's
// binomial_split): with c = free + 1 checkpoints and r repetitions C(c + r, c)
// steps can be reversed; the tail gets what c - 1 checkpoints reverse with r.
int64_t binomial_split(int64_t length, int64_t free_slots) {
    if (length <= 1 || free_slots <= 0) return 1;
    const int64_t c = free_slots + 1;
    int64_t r = 0;
    while (binom_capped(c + r, c, length) < length) ++r;
    const int64_t tail = binom_capped(c - 1 + r, c - 1, length);
    return std::max<int64_t>(1, length - std::min<int64_t>(tail, length - 1));
}

struct Sweep {
    swe_ctx* c = nullptr;
    long long s0 = 0;          // the context's step at the start (sweep step t is device step s0 + t)
    int64_t T = 0, N = 0, stride = 0, G = 0;
    double* slots = nullptr;   // [slot][3][N]
    std::vector<int> free_slots;
    uint8_t* branches = nullptr;  // [T][stride]
    const int64_t* gauges = nullptr;
    const double* obs = nullptr;  // [T][G]
    double* gv = nullptr;         // [T][G]
    std::vector<char> done;
    double* lam[2][3] = {{nullptr, nullptr, nullptr}, {nullptr, nullptr, nullptr}};
    int li = 0;
    double* bbar = nullptr;
    int64_t cur = 0;
    int64_t forward_steps = 0, adjoint_steps = 0;
    int rc = SWE_OK;

    double* slot(int k, int q) { return slots + ((size_t)k * 3 + (size_t)q) * (size_t)N; }

    int store(int64_t t, int* out) {
        if (free_slots.empty()) return set_error(SWE_E_STATE, "revolve ran out of snapshot slots");
        const int k = free_slots.back();
        free_slots.pop_back();
        const int b = (int)((s0 + t) & 1);
        const size_t bytes = (size_t)N * 8;
        CUDA_TRY(cudaMemcpyAsync(slot(k, 0), c->h[b], bytes, cudaMemcpyDeviceToDevice, c->stream));
        CUDA_TRY(cudaMemcpyAsync(slot(k, 1), c->hu[b], bytes, cudaMemcpyDeviceToDevice, c->stream));
        CUDA_TRY(cudaMemcpyAsync(slot(k, 2), c->hv[b], bytes, cudaMemcpyDeviceToDevice, c->stream));
        *out = k;
        return SWE_OK;
    }
    int restore(int k, int64_t t) {
        const int b = (int)((s0 + t) & 1);
        const size_t bytes = (size_t)N * 8;
        CUDA_TRY(cudaMemcpyAsync(c->h[b], slot(k, 0), bytes, cudaMemcpyDeviceToDevice, c->stream));
        CUDA_TRY(cudaMemcpyAsync(c->hu[b], slot(k, 1), bytes, cudaMemcpyDeviceToDevice, c->stream));
        CUDA_TRY(cudaMemcpyAsync(c->hv[b], slot(k, 2), bytes, cudaMemcpyDeviceToDevice, c->stream));
        set_step_kernel<<<1, 1, 0, c->stream>>>(c->gs, s0 + t);
        CUDA_TRY(cudaGetLastError());
        c->step_mirror = s0 + t;
        cur = t;
        return SWE_OK;
    }
    int advance(int64_t k) {
        for (int64_t i = 0; i < k; ++i) {
            const int64_t t = cur;
            int r = launch_steps(c, 1, branches + (size_t)t * (size_t)stride);
            if (r) return r;
            if (!done[(size_t)t]) {  // the first visit of step t records the gauges of x_{t+1}
                gauge_kernel<<<(int)std::min<int64_t>((G + 127) / 128, 1024), 128, 0, c->stream>>>(
                    c->gs, c->h[0], c->h[1], G, gauges, N, gv + (size_t)t * (size_t)G);
                CUDA_TRY(cudaGetLastError());
                done[(size_t)t] = 1;
            }
            cur = t + 1;
            ++forward_steps;
        }
        return SWE_OK;
    }
    int adjoint(int64_t t) {
        if (cur != t) return set_error(SWE_E_STATE, "revolve: state at %lld, reverse step %lld", (long long)cur,
                                       (long long)t);
        if (!done[(size_t)t]) {  // run step t once (branches, gauges), then x_t is still in its buffer
            int r = advance(1);
            if (r) return r;
            set_step_kernel<<<1, 1, 0, c->stream>>>(c->gs, s0 + t);
            CUDA_TRY(cudaGetLastError());
            c->step_mirror = s0 + t;
            cur = t;
        }
        double** in = lam[li];
        double** out = lam[li ^ 1];
        gauge_residual_kernel<<<1, (unsigned)std::min<int64_t>(std::max<int64_t>(G, 32), 256), 0, c->stream>>>(
            in[0], gauges, G, gv + (size_t)t * (size_t)G, obs + (size_t)t * (size_t)G);
        CUDA_TRY(cudaGetLastError());
        int r = launch_adjoint(c, s0 + t, branches + (size_t)t * (size_t)stride, in[0], in[1], in[2], out[0],
                               out[1], out[2], bbar);
        if (r) return r;
        li ^= 1;
        ++adjoint_steps;
        return SWE_OK;
    }
    int rev(int64_t a, int64_t b, int64_t sl, int slot_a) {
        const int64_t length = b - a;
        int r;
        if (length == 1) {
            if ((r = restore(slot_a, a))) return r;
            return adjoint(a);
        }
        if (sl == 0) {
            for (int64_t t = b - 1; t >= a; --t) {
                if ((r = restore(slot_a, a)) || (r = advance(t - a)) || (r = adjoint(t))) return r;
            }
            return SWE_OK;
        }
        const int64_t m = a + binomial_split(length, sl);
        int slot_m = -1;
        if ((r = restore(slot_a, a)) || (r = advance(m - a)) || (r = store(m, &slot_m))) return r;
        if ((r = rev(m, b, sl - 1, slot_m))) return r;
        free_slots.push_back(slot_m);
        return rev(a, m, sl, slot_a);
    }
};

}  // namespace

extern "C" {

int swe_gauge_gradient(swe_ctx* c, int64_t n_steps, const double* dts, int32_t snapshots, int64_t n_gauges,
                       const int64_t* gauges, const double* obs, double* gauge_values, double* grad_h,
                       double* grad_hu, double* grad_hv, double* grad_b, double* J, int64_t* forward_steps) {
    int rc = ready(c);
    if (rc) return rc;
    if (n_inst(c) != 1) return set_error(SWE_E_INVALID, "the adjoint runs on single-instance contexts");
    if (!adjoint_kernel_for(c->params[0].solver))
        return set_error(SWE_E_INVALID, "the adjoint differentiates the f-wave, augmented and Lax-Friedrichs fluxes");
    if (n_steps < 1 || !dts || snapshots < 1 || n_gauges < 1 || !gauges || !obs || !grad_h || !grad_b || !J)
        return set_error(SWE_E_INVALID, "bad arguments");
    cudaSetDevice(c->device);
    Sweep S;
    S.c = c;
    S.T = n_steps;
    S.N = c->mesh[0].n_cells;
    S.stride = c->cells_total;
    S.G = n_gauges;
    S.gauges = gauges;
    S.obs = obs;
    {  // gauge cells must be cells of the mesh
        std::vector<int64_t> g((size_t)n_gauges);
        CUDA_TRY(cudaMemcpy(g.data(), gauges, sizeof(int64_t) * g.size(), cudaMemcpyDeviceToHost));
        for (int64_t v : g)
            if (v < 0 || v >= S.N) return set_error(SWE_E_INVALID, "gauge cell %lld out of range", (long long)v);
    }
    if ((rc = swe_set_dt_sequence(c, n_steps, dts))) return rc;
    S.s0 = c->step_mirror;
    const size_t nb = (size_t)S.N * 8;
    double* work = nullptr;  // lam[2][3], out gauge values if not given
    const size_t n_work = 6 * (size_t)S.N + (gauge_values ? 0 : (size_t)n_steps * (size_t)n_gauges) + 1;
    if ((rc = device_alloc((void**)&work, n_work * 8))) return rc;
    if ((rc = device_alloc((void**)&S.slots, (size_t)snapshots * 3 * nb))) {
        cudaFree(work);
        return rc;
    }
    if ((rc = device_alloc((void**)&S.branches, (size_t)n_steps * (size_t)S.stride))) {
        cudaFree(work);
        cudaFree(S.slots);
        return rc;
    }
    for (int i = 0; i < 2; ++i)
        for (int q = 0; q < 3; ++q) S.lam[i][q] = work + (size_t)(3 * i + q) * (size_t)S.N;
    double* dJ = work + 6 * (size_t)S.N;
    S.gv = gauge_values ? gauge_values : dJ + 1;
    S.bbar = grad_b;
    S.done.assign((size_t)n_steps, 0);
    for (int k = snapshots - 1; k >= 0; --k) S.free_slots.push_back(k);
    cudaError_t e = cudaMemsetAsync(S.lam[0][0], 0, 3 * nb, c->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(grad_b, 0, nb, c->stream);
    if (e != cudaSuccess) rc = set_error(SWE_E_CUDA, "gauge gradient: %s", cudaGetErrorString(e));
    int slot0 = -1;
    S.cur = 0;
    if (!rc) rc = S.store(0, &slot0);
    if (!rc) rc = S.rev(0, n_steps, snapshots - 1, slot0);
    if (!rc) rc = S.restore(slot0, 0);  // leave the context at x_0, step s0
    if (!rc) {
        misfit_kernel<<<1, 256, 0, c->stream>>>(S.gv, obs, n_steps * n_gauges, dJ);
        e = cudaGetLastError();
        double* out[3] = {grad_h, grad_hu, grad_hv};
        for (int q = 0; q < 3 && e == cudaSuccess; ++q)
            if (out[q]) e = cudaMemcpyAsync(out[q], S.lam[S.li][q], nb, cudaMemcpyDeviceToDevice, c->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(J, dJ, 8, cudaMemcpyDeviceToHost, c->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
        if (e != cudaSuccess) rc = set_error(SWE_E_CUDA, "gauge gradient: %s", cudaGetErrorString(e));
    }
    cudaStreamSynchronize(c->stream);
    cudaFree(work);
    cudaFree(S.slots);
    cudaFree(S.branches);
    if (forward_steps) *forward_steps = S.forward_steps;
    if (!rc) rc = check_device_error(c);
    return rc;
}

}  // extern "C"
