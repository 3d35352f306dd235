// swe_step_noalloc: one SWE time step on caller-owned device memory that
// allocates nothing.
//
// Some callers cannot allocate device memory when they want to step: a host
// code that hands all its device memory out of its own pool, or that runs the
// step where a cudaMalloc would synchronise the device or be refused. This
// entry point takes every input and output as a device pointer the caller
// owns, and keeps the only scratch it needs (the per-(cell, local edge) edge
// updates and the reduction accumulators) in one file-scope __device__ array
// of fixed size, so it never calls cudaMalloc, cudaFree or an allocating
// library routine. The price is a size limit (kNoAllocMaxCells) and that the
// scratch array is held by every GPU that loads the library until exit.
//
// The step itself is the same arithmetic as the fused kernel, in two passes:
// one thread per edge writes the left/right updates into the scratch slots and
// counts its claim on each slot, then one thread per cell checks that each of
// its three slots was claimed exactly once, sums them in local edge order,
// updates the cell and reduces the CFL time step; the last block writes dt_new
// and the refinement count and clears the accumulators for the next call. A
// slot claimed by no edge or by two edges makes the call report -1 refinements
// instead of reading what an earlier call left in that slot.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cfloat>
#include <algorithm>
#include <cstdio>
#include <mutex>

#include "swe_internal.h"
#include "swe_riemann.cuh"

namespace swe_noalloc {

using namespace swe;

constexpr int64_t kNoAllocMaxCells = (int64_t)1 << 16;  // 65,536 cells
constexpr size_t kAccBytes = 256;                        // accumulators
constexpr size_t kClaimBytes = (size_t)3 * sizeof(unsigned int) * kNoAllocMaxCells;
constexpr size_t kScratchBytes = kAccBytes + kClaimBytes + (size_t)12 * sizeof(double) * kNoAllocMaxCells;

// The scratch: [0, 256) accumulators {dt bits, refinements, finished blocks,
// error}, then the claim counts [3 local edges][max cells] (zero between
// calls), then the edge-update slots [4 quantities][3 local edges][max cells].
static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

__constant__ double k_leg[kMaxDepth + 2];
__constant__ double k_vol[kMaxDepth + 1];
__constant__ double k_normal[17][3][2];

// All accumulators are zero between calls: the CFL minimum is kept as the
// complement of the (non-negative) double's bits, so that a running max of
// complements starting at 0 is the minimum.
struct Acc {
    unsigned long long dt_cbits;
    unsigned long long refine;
    unsigned int done;
    unsigned int error;
};

struct Args {
    int64_t n_cells, n_edges, n_bnd;
    const int8_t* depth;
    const int8_t* plotter;
    const int64_t* edge_cells;
    const int8_t* edge_local;
    const int64_t* bnd_cell;
    const int8_t* bnd_local;
    const double *h, *hu, *hv, *b;
    double *h_out, *hu_out, *hv_out;
    int8_t* flags;
    double* dt_new_out;
    int64_t* n_refine_out;
    double dt, drytol, scaling, thr_refine, thr_coarsen;
    int32_t min_depth, max_depth, bc, parity;
};

__device__ __forceinline__ State load(const Args& A, int64_t c) { return State{A.h[c], A.hu[c], A.hv[c], A.b[c]}; }

template <int SOLVER>
__global__ void edges_kernel(Args A, unsigned char* scratch) {
    Acc* acc = reinterpret_cast<Acc*>(scratch);
    unsigned int* claims = reinterpret_cast<unsigned int*>(scratch + kAccBytes);
    double* slots = reinterpret_cast<double*>(scratch + kAccBytes + kClaimBytes);
    const int64_t M = kNoAllocMaxCells;
    const int64_t total = A.n_edges + A.n_bnd;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        int64_t L, R = -1;
        int iL, iR = 0;
        if (t < A.n_edges) {
            // the lower-numbered cell is touched first on even steps, the higher on odd steps
            int64_t a = A.edge_cells[2 * t], c = A.edge_cells[2 * t + 1];
            int la = A.edge_local[2 * t] - 1, lc = A.edge_local[2 * t + 1] - 1;
            if (a > c) {
                int64_t tc = a; a = c; c = tc;
                int ti = la; la = lc; lc = ti;
            }
            if (A.parity & 1) {
                L = c; iL = lc; R = a; iR = la;
            } else {
                L = a; iL = la; R = c; iR = lc;
            }
        } else {
            L = A.bnd_cell[t - A.n_edges];
            iL = A.bnd_local[t - A.n_edges] - 1;
        }
        if (L < 0 || L >= A.n_cells || (R >= A.n_cells) || (t < A.n_edges && R < 0) || iL < 0 || iL > 2 || iR < 0 ||
            iR > 2) {
            atomicOr(&acc->error, 1u);
            continue;
        }
        const int pL = A.plotter[L] + 8;
        if (pL < 0 || pL > 16 || pL == 8) {
            atomicOr(&acc->error, 1u);
            continue;
        }
        atomicAdd(&claims[iL * M + L], 1u);
        if (R >= 0) atomicAdd(&claims[iR * M + R], 1u);
        const double n1 = k_normal[pL][iL][0], n2 = k_normal[pL][iL][1];
        const State QL = load(A, L);
        State QR;
        if (R < 0) {
            if (A.bc == BC_SLIP) QR = boundary_ghost<BC_SLIP>(n1, n2, QL);
            else if (A.bc == BC_NOSLIP) QR = boundary_ghost<BC_NOSLIP>(n1, n2, QL);
            else QR = QL;
        } else {
            QR = load(A, R);
        }
        double dL, dR, sqL, sqR, yL, yR;
        depth_terms(QL, A.drytol, dL, sqL, yL);
        depth_terms(QR, A.drytol, dR, sqR, yR);
        Update fL, fR;
        edge_flux<SOLVER>(n1, n2, QL, QR, dL, dR, sqL, sqR, yL, yR, A.drytol, fL, fR);
        slots[(0 * 3 + iL) * M + L] = fL.h;
        slots[(1 * 3 + iL) * M + L] = fL.p1;
        slots[(2 * 3 + iL) * M + L] = fL.p2;
        slots[(3 * 3 + iL) * M + L] = fL.s;
        if (R >= 0) {
            slots[(0 * 3 + iR) * M + R] = fR.h;
            slots[(1 * 3 + iR) * M + R] = fR.p1;
            slots[(2 * 3 + iR) * M + R] = fR.p2;
            slots[(3 * 3 + iR) * M + R] = fR.s;
        }
    }
}

__global__ void cells_kernel(Args A, unsigned char* scratch) {
    Acc* acc = reinterpret_cast<Acc*>(scratch);
    unsigned int* claims = reinterpret_cast<unsigned int*>(scratch + kAccBytes);
    const double* slots = reinterpret_cast<const double*>(scratch + kAccBytes + kClaimBytes);
    const int64_t M = kNoAllocMaxCells;
    __shared__ double red_min[32];
    __shared__ long long red_sum[32];
    __shared__ int s_last;
    const int k0 = (A.parity & 1) ? 2 : 0, k2 = (A.parity & 1) ? 0 : 2;
    double dtmin = DBL_MAX;
    long long nref = 0;
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < A.n_cells; c += (int64_t)gridDim.x * blockDim.x) {
        // each slot must hold exactly one edge's update of this call; the
        // counts go back to zero for the next call whatever they were
        bool bad = false;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            bad |= claims[k * M + c] != 1u;
            claims[k * M + c] = 0u;
        }
        const int d = A.depth[c];
        if (bad || d < 0 || d > kMaxDepth) {
            atomicOr(&acc->error, 1u);
            continue;
        }
        const double vol = (A.scaling * A.scaling) * k_vol[d];
        const double leg = A.scaling * k_leg[d + 1], hyp = A.scaling * k_leg[d];
        const double ndv = -A.dt / vol;
        double q[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            double v = z0(leg * slots[(k * 3 + k0) * M + c]) + hyp * slots[(k * 3 + 1) * M + c];
            q[k] = v + leg * slots[(k * 3 + k2) * M + c];
        }
        double dh = q[0], dp1 = q[1], dp2 = q[2];
        int8_t f = 0;
        const double nrm = fabs(dh);
        if (d < A.max_depth && nrm > A.thr_refine) {
            f = 1;
            ++nref;
        } else if (d > A.min_depth && nrm < A.thr_coarsen) {
            f = -1;
        }
        dtmin = dmn(dtmin, vol / q[3]);
        dh = ndv * dh;
        dp1 = ndv * dp1;
        dp2 = ndv * dp2;
        double h = A.h[c], p1 = A.hu[c], p2 = A.hv[c];
        const double b = A.b[c];
        if (h < b + A.drytol && dh > 0.0) {
            h = b + A.drytol;
            p1 = 0.0;
            p2 = 0.0;
        }
        h = h + dh;
        p1 = p1 + dp1;
        p2 = p2 + dp2;
        if (h < b + A.drytol) {
            h = dmn(b, 0.0);
            p1 = 0.0;
            p2 = 0.0;
        }
        A.h_out[c] = h;
        A.hu_out[c] = p1;
        A.hv_out[c] = p2;
        if (A.flags) A.flags[c] = f;
    }
    // block reduction, one atomic per block, last block publishes and clears
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        dtmin = dmn(dtmin, __shfl_xor_sync(0xffffffffu, dtmin, o));
        nref += __shfl_xor_sync(0xffffffffu, nref, o);
    }
    if (lane == 0) {
        red_min[warp] = dtmin;
        red_sum[warp] = nref;
    }
    __syncthreads();
    if (tid == 0) {
        const int nw = (blockDim.x + 31) >> 5;
        double m = DBL_MAX;
        long long s = 0;
        for (int w = 0; w < nw; ++w) {
            m = dmn(m, red_min[w]);
            s += red_sum[w];
        }
        atomicMax(&acc->dt_cbits, ~(unsigned long long)__double_as_longlong(m));
        atomicAdd(&acc->refine, (unsigned long long)s);
        __threadfence();
        s_last = atomicAdd(&acc->done, 1u) == gridDim.x - 1;
        if (s_last) {
            __threadfence();
            const unsigned long long bits = ~atomicAdd(&acc->dt_cbits, 0ull);
            const unsigned long long r = atomicAdd(&acc->refine, 0ull);
            const unsigned int err = atomicAdd(&acc->error, 0u);
            if (A.dt_new_out) *A.dt_new_out = __longlong_as_double((long long)bits);
            if (A.n_refine_out) *A.n_refine_out = err ? -1 : (int64_t)r;
            acc->dt_cbits = 0;
            acc->refine = 0;
            acc->done = 0;
            acc->error = 0;
        }
    }
}

// Once per device and CUDA context, with that device current: the scratch
// array's device address, the geometry tables of this file's kernels, and the
// accumulators and claim counts cleared. The context is recognised by its
// unique id (cuCtxGetId, reached through the runtime's driver entry point, so
// the library needs no link to the driver library): a device reset followed by
// a new primary context gets a new id and so a fresh set-up, instead of running
// on zeroed tables.
typedef CUresult (*CtxGetCurrentFn)(CUcontext*);
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long*);

struct DeviceSetup {
    bool ready = false;
    unsigned long long ctx_id = 0;
    unsigned char* scratch = nullptr;
};
static std::mutex g_setup_mutex;
static DeviceSetup g_setup[64];
static CtxGetCurrentFn g_ctx_current = nullptr;
static CtxGetIdFn g_ctx_id = nullptr;

static int driver_entry_points() {
    if (g_ctx_current && g_ctx_id) return SWE_OK;
    void* f1 = nullptr;
    void* f2 = nullptr;
    cudaDriverEntryPointQueryResult q1, q2;
    cudaError_t e = cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1);
    if (e == cudaSuccess) e = cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2);
    if (e != cudaSuccess || q1 != cudaDriverEntryPointSuccess || q2 != cudaDriverEntryPointSuccess || !f1 || !f2)
        return set_error(SWE_E_CUDA, "swe_step_noalloc: driver entry points cuCtxGetCurrent/cuCtxGetId unavailable");
    g_ctx_current = reinterpret_cast<CtxGetCurrentFn>(f1);
    g_ctx_id = reinterpret_cast<CtxGetIdFn>(f2);
    return SWE_OK;
}

// The current context's id, 0 when the calling thread has none yet.
static unsigned long long current_ctx_id() {
    CUcontext c = nullptr;
    unsigned long long id = 0;
    if (g_ctx_current(&c) != CUDA_SUCCESS || !c) return 0;
    if (g_ctx_id(c, &id) != CUDA_SUCCESS) return 0;
    return id;
}

static int setup_device(int dev, unsigned char** scratch) {
    if (dev < 0 || dev >= 64) return set_error(SWE_E_INVALID, "device %d out of range", dev);
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    int rc = driver_entry_points();
    if (rc) return rc;
    DeviceSetup& s = g_setup[dev];
    unsigned long long id = current_ctx_id();
    if (s.ready && id != 0 && id == s.ctx_id) {
        *scratch = s.scratch;
        return SWE_OK;
    }
    // binds the device's primary context to this thread if it is not yet
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
    if (e != cudaSuccess)
        return set_error(SWE_E_CUDA, "cudaGetSymbolAddress(scratch) failed: %s", cudaGetErrorString(e));
    id = current_ctx_id();
    if (id == 0) return set_error(SWE_E_CUDA, "swe_step_noalloc: no current CUDA context on device %d", dev);
    if (s.ready && id == s.ctx_id) {  // same context, first call from this thread
        *scratch = s.scratch;
        return SWE_OK;
    }
    s.ready = false;
    double leg[kMaxDepth + 2], vol[kMaxDepth + 1], nrm[17][3][2];
    geometry_tables(leg, vol, nrm);
    e = cudaMemcpyToSymbol(k_leg, leg, sizeof(leg));
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(k_vol, vol, sizeof(vol));
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(k_normal, nrm, sizeof(nrm));
    if (e != cudaSuccess) return set_error(SWE_E_CUDA, "geometry tables: %s", cudaGetErrorString(e));
    // accumulators and claim counts start at zero (each call clears them again)
    e = cudaMemset(p, 0, kAccBytes + kClaimBytes);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e != cudaSuccess) return set_error(SWE_E_CUDA, "scratch init: %s", cudaGetErrorString(e));
    s.scratch = static_cast<unsigned char*>(p);
    s.ctx_id = id;
    s.ready = true;
    *scratch = s.scratch;
    return SWE_OK;
}

// After a launch failed part-way, the accumulators and claim counts may hold
// this call's partial work: clear them on the stream so the next call starts
// from zero (a memset, no allocation).
static void clear_after_failure(unsigned char* scratch, cudaStream_t s) {
    (void)cudaMemsetAsync(scratch, 0, kAccBytes + kClaimBytes, s);
}

}  // namespace swe_noalloc

using namespace swe_noalloc;

extern "C" int swe_step_noalloc(const swe_params* p, int64_t n_cells, const int8_t* depth, const int8_t* plotter,
                                int64_t n_edges, const int64_t* edge_cells, const int8_t* edge_local, int64_t n_bnd,
                                const int64_t* bnd_cell, const int8_t* bnd_local, const double* h, const double* hu,
                                const double* hv, const double* b, double* h_out, double* hu_out, double* hv_out,
                                int8_t* flags, double dt, int32_t parity, double* dt_new, int64_t* n_refinements,
                                void* stream) {
    if (!p) return set_error(SWE_E_INVALID, "null params");
    if (n_cells < 1 || n_cells > kNoAllocMaxCells)
        return set_error(SWE_E_INVALID, "swe_step_noalloc: n_cells %lld outside 1..%lld (the fixed scratch limit)",
                         (long long)n_cells, (long long)kNoAllocMaxCells);
    // both counts are bounded before they enter the sum, which then cannot overflow
    if (n_edges < 0 || n_bnd < 0 || n_edges > 3 * kNoAllocMaxCells || n_bnd > 3 * kNoAllocMaxCells ||
        2 * n_edges + n_bnd != 3 * n_cells)
        return set_error(SWE_E_INVALID, "swe_step_noalloc: edge counts inconsistent");
    if (!depth || !plotter || (n_edges && (!edge_cells || !edge_local)) || (n_bnd && (!bnd_cell || !bnd_local)) ||
        !h || !hu || !hv || !b || !h_out || !hu_out || !hv_out)
        return set_error(SWE_E_INVALID, "swe_step_noalloc: null device pointer");
    if (p->bc < SWE_BC_OUTFLOW || p->bc > SWE_BC_NOSLIP || !(p->scaling > 0.0) || p->min_depth < 0 ||
        p->max_depth > kMaxDepth || p->min_depth > p->max_depth)
        return set_error(SWE_E_INVALID, "swe_step_noalloc: invalid parameters");
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return set_error(SWE_E_CUDA, "cudaGetDevice: %s", cudaGetErrorString(e));
    unsigned char* scratch = nullptr;
    int rc = setup_device(dev, &scratch);
    if (rc) return rc;
    double leg[kMaxDepth + 2], vol[kMaxDepth + 1], nrm[17][3][2];
    geometry_tables(leg, vol, nrm);
    Args A;
    A.n_cells = n_cells; A.n_edges = n_edges; A.n_bnd = n_bnd;
    A.depth = depth; A.plotter = plotter; A.edge_cells = edge_cells; A.edge_local = edge_local;
    A.bnd_cell = bnd_cell; A.bnd_local = bnd_local;
    A.h = h; A.hu = hu; A.hv = hv; A.b = b;
    A.h_out = h_out; A.hu_out = hu_out; A.hv_out = hv_out; A.flags = flags;
    A.dt_new_out = dt_new; A.n_refine_out = n_refinements;
    A.dt = dt;
    A.drytol = p->dry_tolerance;
    A.scaling = p->scaling;
    A.thr_refine = (5.0 * p->scaling) * leg[p->max_depth + 1];
    A.thr_coarsen = A.thr_refine / 8.0;
    A.min_depth = p->min_depth; A.max_depth = p->max_depth; A.bc = p->bc; A.parity = parity;
    cudaStream_t s = (cudaStream_t)stream;
    const int threads = 256;
    const int eblocks = (int)std::max<int64_t>(1, std::min<int64_t>((n_edges + n_bnd + threads - 1) / threads, 1024));
    const int cblocks = (int)std::max<int64_t>(1, std::min<int64_t>((n_cells + threads - 1) / threads, 1024));
    switch (p->solver) {
        case FWAVE: edges_kernel<FWAVE><<<eblocks, threads, 0, s>>>(A, scratch); break;
        case AUG_RIEMANN: edges_kernel<AUG_RIEMANN><<<eblocks, threads, 0, s>>>(A, scratch); break;
        case LF: edges_kernel<LF><<<eblocks, threads, 0, s>>>(A, scratch); break;
        case LF_BATH: edges_kernel<LF_BATH><<<eblocks, threads, 0, s>>>(A, scratch); break;
        case LLF: edges_kernel<LLF><<<eblocks, threads, 0, s>>>(A, scratch); break;
        case LLF_BATH: edges_kernel<LLF_BATH><<<eblocks, threads, 0, s>>>(A, scratch); break;
        default: return set_error(SWE_E_INVALID, "swe_step_noalloc: unknown solver %d", p->solver);
    }
    e = cudaGetLastError();
    if (e != cudaSuccess) {
        clear_after_failure(scratch, s);
        return set_error(SWE_E_CUDA, "edges kernel: %s", cudaGetErrorString(e));
    }
    cells_kernel<<<cblocks, threads, 0, s>>>(A, scratch);
    e = cudaGetLastError();
    if (e != cudaSuccess) {
        clear_after_failure(scratch, s);
        return set_error(SWE_E_CUDA, "cells kernel: %s", cudaGetErrorString(e));
    }
    return SWE_OK;
}
