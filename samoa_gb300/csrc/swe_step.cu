// The SWE explicit Euler time step on the GPU (sm_103a) and its C ABI.
//
// One kernel launch is one time step of t_swe_euler_timestep_traversal
// (src/SWE/SWE_euler_timestep.f90). Cells are split into contiguous
// segments of the space-filling-curve order; a CTA takes one segment at a
// time (persistent grid):
//   1. stage the segment's h, hu, hv, b into shared memory with 1-D TMA bulk
//      copies (cp.async.bulk, completion on an mbarrier);
//   2. evaluate every edge task of the segment once: the Riemann solver runs
//      with the first-touched cell as the left side and writes the left and
//      right updates into per-(cell, local edge) slots in shared memory, so no
//      atomics are needed; an edge between two segments is evaluated by both
//      CTAs, each keeping its own side;
//   3. update each cell from its three slots in local edge index order (the
//      order the reference sums them in), clamp wet/dry, write the state to the
//      other buffer, set the refinement flag, and fold volume/sum(len*speed)
//      into a CTA minimum with warp shuffles;
//   4. the last CTA to finish turns the minimum into the next dt, advances the
//      time and the step counter, and resets the accumulators.
// The traversal direction of the reference alternates every step
// (src/SFC_generic_traversal_ringbuffer.f90:420); the kernel reads the step
// parity from device memory: on odd steps the higher-numbered cell of an edge
// is touched first and the two leg updates are summed in the other order.
#include <cuda_runtime.h>

#include <cfloat>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "swe_internal.h"
#include "swe_riemann.cuh"

namespace swe {

// ---------------------------------------------------------------------------
// errors
// ---------------------------------------------------------------------------

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

// ---------------------------------------------------------------------------
// device tables (context independent: unscaled lengths and normals)
// ---------------------------------------------------------------------------

__constant__ double c_leg[kMaxDepth + 2];  // sqrt(0.5)**i at [i + 1], i = -1..60
__constant__ double c_vol[kMaxDepth + 1];  // 0.5**(i + 1)
__constant__ double c_normal[17][3][2];    // [plotter + 8][local edge][x, y]

struct StepArgs {
    double* h[2];
    double* hu[2];
    double* hv[2];
    const double* b;
    const int8_t* depth;
    int8_t* flags;
    const int4* tasks;
    const long long* seg_ptr;
    DevScalars* scal;
    double drytol, courant, scaling, thr_refine, thr_coarsen, max_time, tout;
    int32_t n_cells, seg_cells, n_seg;
    int32_t min_depth, max_depth;  // refinement limits (cfg)
    int32_t dmin, ndepth;          // depth range present in the mesh
    int32_t bc;
    int32_t use_tma;
};

constexpr int kWaitLimit = 1 << 24;  // polls of an mbarrier before a kernel gives up

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// 1-D bulk copy global -> this CTA's shared memory; both addresses 16-byte
// aligned, size a multiple of 16.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ void fence_proxy_async() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ double warp_min(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = dmn(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

__device__ __forceinline__ long long warp_sum(long long v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

template <int SOLVER>
__global__ void __launch_bounds__(256) step_kernel(const StepArgs A) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int T = A.seg_cells;
    double* sh_h = reinterpret_cast<double*>(smem_raw);
    double* sh_hu = sh_h + T;
    double* sh_hv = sh_hu + T;
    double* sh_b = sh_hv + T;
    double* upd = sh_b + T;                 // [4 quantities][3 local edges][T cells]
    double* tab_leg = upd + 12 * T;         // per depth present in the mesh
    double* tab_hyp = tab_leg + A.ndepth;
    double* tab_vol = tab_hyp + A.ndepth;
    double* tab_ndv = tab_vol + A.ndepth;   // -dt / volume
    __shared__ uint64_t bar;
    __shared__ double red_min[32];
    __shared__ long long red_sum[32];
    __shared__ unsigned int s_error;

    const int tid = threadIdx.x;
    const long long step = A.scal->step;
    const int odd = (int)(step & 1);
    const double* hin = A.h[odd];
    const double* huin = A.hu[odd];
    const double* hvin = A.hv[odd];
    double* hout = A.h[odd ^ 1];
    double* huout = A.hu[odd ^ 1];
    double* hvout = A.hv[odd ^ 1];

    // pre_traversal_grid_op (src/SWE/SWE_euler_timestep.f90:89-109): clamp dt
    double dt = A.scal->dt;
    if (A.max_time > 0.0) dt = dmn(A.max_time, dt);
    if (A.tout > 0.0) dt = dmn(A.tout, dt);

    if (tid == 0) {
        s_error = 0;
        mbar_init(&bar, 1);
        fence_mbar_init();
    }
    for (int i = tid; i < A.ndepth; i += blockDim.x) {
        const int d = A.dmin + i;
        const double vol = (A.scaling * A.scaling) * c_vol[d];
        tab_leg[i] = A.scaling * c_leg[d + 1];
        tab_hyp[i] = A.scaling * c_leg[d];
        tab_vol[i] = vol;
        tab_ndv[i] = -dt / vol;
    }
    __syncthreads();

    double dtmin = DBL_MAX;  // r_dt_new = huge(1.0) (pre_traversal_op)
    long long nref = 0;
    uint32_t phase = 0;

    for (int seg = blockIdx.x; seg < A.n_seg; seg += gridDim.x) {
        const int c0 = seg * T;
        const int cn = min(T, A.n_cells - c0);
        // ---- 1. stage the segment's state
        const int cbulk = A.use_tma ? (cn & ~1) : 0;  // 16-byte multiple
        if (cbulk > 0) {
            if (tid == 0) {
                fence_proxy_async();
                const uint32_t bytes = (uint32_t)cbulk * 8u;
                mbar_arrive_expect_tx(&bar, 4u * bytes);
                bulk_g2s(sh_h, hin + c0, bytes, &bar);
                bulk_g2s(sh_hu, huin + c0, bytes, &bar);
                bulk_g2s(sh_hv, hvin + c0, bytes, &bar);
                bulk_g2s(sh_b, A.b + c0, bytes, &bar);
            }
        }
        for (int i = cbulk + tid; i < cn; i += blockDim.x) {
            sh_h[i] = hin[c0 + i];
            sh_hu[i] = huin[c0 + i];
            sh_hv[i] = hvin[c0 + i];
            sh_b[i] = A.b[c0 + i];
        }
        if (cbulk > 0) {
            int polls = 0;
            while (!mbar_try_wait(&bar, phase)) {
                if (++polls > kWaitLimit) {
                    s_error = 2u;
                    break;
                }
            }
            phase ^= 1u;
        }
        __syncthreads();
        if (s_error) break;

        // ---- 2. edge tasks
        const long long t0 = A.seg_ptr[seg], t1 = A.seg_ptr[seg + 1];
        for (long long t = t0 + tid; t < t1; t += blockDim.x) {
            const int4 tk = __ldg(&A.tasks[t]);
            const uint32_t meta = (uint32_t)tk.z;
            const bool bnd = (meta >> 14) & 1u;
            int L, R, iL, iR, pL;
            if (bnd || !odd) {
                L = tk.x; iL = meta & 3u; pL = (meta >> 4) & 31u;
                R = tk.y; iR = (meta >> 2) & 3u;
            } else {
                L = tk.y; iL = (meta >> 2) & 3u; pL = (meta >> 9) & 31u;
                R = tk.x; iR = meta & 3u;
            }
            if ((unsigned)L >= (unsigned)A.n_cells || (!bnd && (unsigned)R >= (unsigned)A.n_cells) || iL > 2 ||
                iR > 2 || pL > 16) {
                atomicOr(&s_error, 1u);
                continue;
            }
            const double n1 = c_normal[pL][iL][0], n2 = c_normal[pL][iL][1];
            const int sl = L - c0, sr = R - c0;
            const bool lin = (unsigned)sl < (unsigned)cn;
            const bool rin = !bnd && (unsigned)sr < (unsigned)cn;
            State QL, QR;
            if (lin) QL = State{sh_h[sl], sh_hu[sl], sh_hv[sl], sh_b[sl]};
            else QL = State{hin[L], huin[L], hvin[L], A.b[L]};
            if (bnd) {
                if (A.bc == BC_SLIP) QR = boundary_ghost<BC_SLIP>(n1, n2, QL);
                else if (A.bc == BC_NOSLIP) QR = boundary_ghost<BC_NOSLIP>(n1, n2, QL);
                else QR = QL;
            } else if (rin) {
                QR = State{sh_h[sr], sh_hu[sr], sh_hv[sr], sh_b[sr]};
            } else {
                QR = State{hin[R], huin[R], hvin[R], A.b[R]};
            }
            Update fL, fR;
            edge_flux<SOLVER>(n1, n2, QL, QR, A.drytol, fL, fR);
            if (lin) {
                upd[(0 * 3 + iL) * T + sl] = fL.h;
                upd[(1 * 3 + iL) * T + sl] = fL.p1;
                upd[(2 * 3 + iL) * T + sl] = fL.p2;
                upd[(3 * 3 + iL) * T + sl] = fL.s;
            }
            if (rin) {
                upd[(0 * 3 + iR) * T + sr] = fR.h;
                upd[(1 * 3 + iR) * T + sr] = fR.p1;
                upd[(2 * 3 + iR) * T + sr] = fR.p2;
                upd[(3 * 3 + iR) * T + sr] = fR.s;
            }
        }
        __syncthreads();

        // ---- 3. cell updates: cell_update_op + volume_op (src/SWE/SWE_euler_timestep.f90:257-355)
        const int k0 = odd ? 2 : 0, k2 = odd ? 0 : 2;
        for (int i = tid; i < cn; i += blockDim.x) {
            const int c = c0 + i;
            const int d = A.depth[c];
            const int di = d - A.dmin;
            const double leg = tab_leg[di], hyp = tab_hyp[di], vol = tab_vol[di], ndv = tab_ndv[di];
            double dh = z0(leg * upd[(0 * 3 + k0) * T + i]) + hyp * upd[(0 * 3 + 1) * T + i];
            dh = dh + leg * upd[(0 * 3 + k2) * T + i];
            double dp1 = z0(leg * upd[(1 * 3 + k0) * T + i]) + hyp * upd[(1 * 3 + 1) * T + i];
            dp1 = dp1 + leg * upd[(1 * 3 + k2) * T + i];
            double dp2 = z0(leg * upd[(2 * 3 + k0) * T + i]) + hyp * upd[(2 * 3 + 1) * T + i];
            dp2 = dp2 + leg * upd[(2 * 3 + k2) * T + i];
            double ds = z0(leg * upd[(3 * 3 + k0) * T + i]) + hyp * upd[(3 * 3 + 1) * T + i];
            ds = ds + leg * upd[(3 * 3 + k2) * T + i];
            // refinement flag
            int8_t f = 0;
            const double nrm = fabs(dh);
            if (d < A.max_depth && nrm > A.thr_refine) {
                f = 1;
                ++nref;
            } else if (d > A.min_depth && nrm < A.thr_coarsen) {
                f = -1;
            }
            dtmin = dmn(dtmin, vol / ds);
            dh = ndv * dh;
            dp1 = ndv * dp1;
            dp2 = ndv * dp2;
            double h = sh_h[i], p1 = sh_hu[i], p2 = sh_hv[i];
            const double b = sh_b[i];
            // wetting: flooded land starts at the dry tolerance, at rest
            if (h < b + A.drytol && dh > 0.0) {
                h = b + A.drytol;
                p1 = 0.0;
                p2 = 0.0;
            }
            h = h + dh;
            p1 = p1 + dp1;
            p2 = p2 + dp2;
            // drying: surface to min(b, 0), at rest
            if (h < b + A.drytol) {
                h = dmn(b, 0.0);
                p1 = 0.0;
                p2 = 0.0;
            }
            hout[c] = h;
            huout[c] = p1;
            hvout[c] = p2;
            A.flags[c] = f;
        }
        __syncthreads();
    }

    // ---- 4. reductions and the last-CTA finalisation
    dtmin = warp_min(dtmin);
    nref = warp_sum(nref);
    const int warp = tid >> 5, lane = tid & 31;
    if (lane == 0) {
        red_min[warp] = dtmin;
        red_sum[warp] = nref;
    }
    __syncthreads();
    if (warp == 0) {
        const int nw = (blockDim.x + 31) >> 5;
        double m = lane < nw ? red_min[lane] : DBL_MAX;
        long long s = lane < nw ? red_sum[lane] : 0;
        m = warp_min(m);
        s = warp_sum(s);
        if (lane == 0) {
            DevScalars* S = A.scal;
            if (s_error) atomicOr(&S->error, s_error);
            atomicMin(&S->dt_acc, (unsigned long long)__double_as_longlong(m));
            atomicAdd(&S->refine_acc, (unsigned long long)s);
            __threadfence();
            const unsigned int ticket = atomicAdd(&S->done, 1u);
            if (ticket == gridDim.x - 1) {
                __threadfence();
                const double dtn = __longlong_as_double((long long)atomicAdd(&S->dt_acc, 0ull));
                const unsigned long long r = atomicExch(&S->refine_acc, 0ull);
                // post_traversal_grid_op (src/SWE/SWE_euler_timestep.f90:111-131)
                S->time = S->time + dt;
                S->dt_new = dtn;
                S->dt = A.courant * dtn;
                S->n_refine = r;
                S->dt_acc = (unsigned long long)__double_as_longlong(DBL_MAX);
                S->done = 0;
                S->step = step + 1;
                __threadfence();
            }
        }
    }
}

__global__ void set_scalars_kernel(DevScalars* S, double time, double dt, int reset_step) {
    S->time = time;
    S->dt = dt;
    S->dt_acc = (unsigned long long)__double_as_longlong(DBL_MAX);
    S->refine_acc = 0;
    S->done = 0;
    if (reset_step) {
        S->step = 0;
        S->dt_new = DBL_MAX;
        S->n_refine = 0;
        S->error = 0;
    }
}

template <int SOLVER>
__global__ void riemann_batch_kernel(int64_t n, const double* nrm, const double* ql, const double* qr, double drytol,
                                     double* ol, double* orr) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        State L{ql[4 * i], ql[4 * i + 1], ql[4 * i + 2], ql[4 * i + 3]};
        State R{qr[4 * i], qr[4 * i + 1], qr[4 * i + 2], qr[4 * i + 3]};
        Update fL, fR;
        edge_flux<SOLVER>(nrm[2 * i], nrm[2 * i + 1], L, R, drytol, fL, fR);
        ol[4 * i] = fL.h; ol[4 * i + 1] = fL.p1; ol[4 * i + 2] = fL.p2; ol[4 * i + 3] = fL.s;
        orr[4 * i] = fR.h; orr[4 * i + 1] = fR.p1; orr[4 * i + 2] = fR.p2; orr[4 * i + 3] = fR.s;
    }
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

static int upload_tables_once() {
    // __constant__ symbols are per device; each context uploads for its device
    double leg[kMaxDepth + 2], vol[kMaxDepth + 1], nrm[17][3][2];
    geometry_tables(leg, vol, nrm);
    CUDA_TRY(cudaMemcpyToSymbol(c_leg, leg, sizeof(leg)));
    CUDA_TRY(cudaMemcpyToSymbol(c_vol, vol, sizeof(vol)));
    CUDA_TRY(cudaMemcpyToSymbol(c_normal, nrm, sizeof(nrm)));
    return SWE_OK;
}

}  // namespace swe

using namespace swe;

struct swe_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t own_stream = nullptr;
    swe_params params{};
    bool has_params = false, has_mesh = false, has_state = false;
    HostMesh mesh;
    int32_t seg_cells = 512, block_threads = 256;
    int64_t n_seg = 0, n_tasks = 0;
    int grid = 0;
    size_t smem = 0;
    double* h[2] = {nullptr, nullptr};
    double* hu[2] = {nullptr, nullptr};
    double* hv[2] = {nullptr, nullptr};
    double* b = nullptr;
    int8_t* depth = nullptr;
    int8_t* flags = nullptr;
    Task* tasks = nullptr;
    long long* seg_ptr = nullptr;
    DevScalars* scal = nullptr;
    int num_sms = 0;
    double leg[kMaxDepth + 2], vol[kMaxDepth + 1], nrm[17][3][2];
};

namespace {

void free_mesh_buffers(swe_ctx* c) {
    for (int k = 0; k < 2; ++k) {
        cudaFree(c->h[k]); cudaFree(c->hu[k]); cudaFree(c->hv[k]);
        c->h[k] = c->hu[k] = c->hv[k] = nullptr;
    }
    cudaFree(c->b); cudaFree(c->depth); cudaFree(c->flags); cudaFree(c->tasks); cudaFree(c->seg_ptr);
    c->b = nullptr; c->depth = nullptr; c->flags = nullptr; c->tasks = nullptr; c->seg_ptr = nullptr;
    c->has_mesh = c->has_state = false;
}

int device_alloc(void** p, size_t bytes) {
    cudaError_t e = cudaMalloc(p, bytes ? bytes : 16);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return set_error(SWE_E_NOMEM, "cudaMalloc(%zu) failed: %s", bytes, cudaGetErrorString(e));
    }
    return SWE_OK;
}

size_t smem_bytes(const swe_ctx* c) {
    const int nd = c->has_mesh ? c->mesh.max_depth - c->mesh.min_depth + 1 : kMaxDepth + 1;
    return (size_t)16 * c->seg_cells * sizeof(double) + (size_t)4 * nd * sizeof(double);
}

int configure_launch(swe_ctx* c) {
    c->smem = smem_bytes(c);
    StepKernel k = kernel_for(c->params.solver ? c->params.solver : FWAVE);
    if (!k) return set_error(SWE_E_INVALID, "unknown solver %d", c->params.solver);
    for (int s : {FWAVE, AUG_RIEMANN, LF, LF_BATH, LLF, LLF_BATH})
        CUDA_TRY(cudaFuncSetAttribute(kernel_for(s), cudaFuncAttributeMaxDynamicSharedMemorySize, (int)c->smem));
    int per_sm = 0;
    CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, c->block_threads, c->smem));
    if (per_sm < 1) return set_error(SWE_E_INVALID, "tiling %d cells x %d threads does not fit an SM", c->seg_cells,
                                     c->block_threads);
    int64_t g = (int64_t)per_sm * c->num_sms;
    c->grid = (int)(g < c->n_seg ? g : c->n_seg);
    if (c->grid < 1) c->grid = 1;
    return SWE_OK;
}

int rebuild_tasks(swe_ctx* c) {
    std::vector<int64_t> seg_ptr;
    std::vector<Task> tasks;
    int rc = build_tasks(c->mesh, c->seg_cells, seg_ptr, tasks);
    if (rc) return rc;
    cudaFree(c->tasks);
    cudaFree(c->seg_ptr);
    c->tasks = nullptr;
    c->seg_ptr = nullptr;
    c->n_seg = (int64_t)seg_ptr.size() - 1;
    c->n_tasks = (int64_t)tasks.size();
    if ((rc = device_alloc((void**)&c->tasks, sizeof(Task) * tasks.size()))) return rc;
    if ((rc = device_alloc((void**)&c->seg_ptr, sizeof(long long) * seg_ptr.size()))) return rc;
    CUDA_TRY(cudaMemcpyAsync(c->tasks, tasks.data(), sizeof(Task) * tasks.size(), cudaMemcpyHostToDevice, c->stream));
    CUDA_TRY(cudaMemcpyAsync(c->seg_ptr, seg_ptr.data(), sizeof(long long) * seg_ptr.size(), cudaMemcpyHostToDevice,
                             c->stream));
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    return configure_launch(c);
}

int check_device_error(swe_ctx* c) {
    unsigned int err = 0;
    CUDA_TRY(cudaMemcpyAsync(&err, &c->scal->error, sizeof(err), cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    if (err) {
        return set_error(SWE_E_DEVICE, "step kernel reported error 0x%x (%s)", err,
                         (err & 2u) ? "TMA wait ran out" : "edge task index out of range");
    }
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
    swe_ctx* c = new swe_ctx();
    c->device = device;
    int rc = upload_tables_once();
    if (rc) { delete c; return rc; }
    cudaError_t e = cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) { delete c; return set_error(SWE_E_CUDA, "stream: %s", cudaGetErrorString(e)); }
    c->stream = c->own_stream;
    cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device);
    if ((rc = device_alloc((void**)&c->scal, sizeof(DevScalars)))) { cudaStreamDestroy(c->own_stream); delete c; return rc; }
    set_scalars_kernel<<<1, 1, 0, c->stream>>>(c->scal, 0.0, 0.0, 1);
    geometry_tables(c->leg, c->vol, c->nrm);
    c->params.solver = SWE_SOLVER_FWAVE;
    c->params.bc = SWE_BC_OUTFLOW;
    c->params.dry_tolerance = 0.01;
    c->params.courant = 0.45;
    c->params.scaling = 1.0;
    c->params.min_depth = 0;
    c->params.max_depth = 14;
    c->params.max_time = -1.0;
    c->params.output_time_step = -1.0;
    c->has_params = true;
    e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) { swe_destroy(c); return set_error(SWE_E_CUDA, "init: %s", cudaGetErrorString(e)); }
    *out = c;
    return SWE_OK;
}

int swe_destroy(swe_ctx* c) {
    if (!c) return SWE_OK;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    free_mesh_buffers(c);
    cudaFree(c->scal);
    if (c->own_stream) cudaStreamDestroy(c->own_stream);
    delete c;
    return SWE_OK;
}

int swe_set_stream(swe_ctx* c, void* stream) {
    if (!c) return set_error(SWE_E_INVALID, "null context");
    c->stream = stream ? (cudaStream_t)stream : c->own_stream;
    return SWE_OK;
}

int swe_set_params(swe_ctx* c, const swe_params* p) {
    if (!c || !p) return set_error(SWE_E_INVALID, "null argument");
    if (!kernel_for(p->solver)) return set_error(SWE_E_INVALID, "unknown solver %d", p->solver);
    if (p->bc < SWE_BC_OUTFLOW || p->bc > SWE_BC_NOSLIP) return set_error(SWE_E_INVALID, "unknown bc %d", p->bc);
    if (!(p->scaling > 0.0)) return set_error(SWE_E_INVALID, "scaling must be > 0");
    if (!(p->dry_tolerance >= 0.0)) return set_error(SWE_E_INVALID, "dry tolerance must be >= 0");
    if (p->min_depth < 0 || p->max_depth > kMaxDepth || p->min_depth > p->max_depth)
        return set_error(SWE_E_INVALID, "depth limits %d..%d invalid", p->min_depth, p->max_depth);
    c->params = *p;
    c->has_params = true;
    if (c->has_mesh) {
        cudaSetDevice(c->device);
        return configure_launch(c);
    }
    return SWE_OK;
}

int swe_set_tiling(swe_ctx* c, int32_t seg_cells, int32_t block_threads) {
    if (!c) return set_error(SWE_E_INVALID, "null context");
    if (seg_cells && (seg_cells < 64 || seg_cells > 1536 || (seg_cells & 1)))
        return set_error(SWE_E_INVALID, "segment_cells %d: need an even value in 64..1536", seg_cells);
    if (block_threads && (block_threads < 64 || block_threads > 256 || (block_threads & 31)))
        return set_error(SWE_E_INVALID, "block_threads %d: need a multiple of 32 in 64..256", block_threads);
    if (seg_cells) c->seg_cells = seg_cells;
    if (block_threads) c->block_threads = block_threads;
    if (c->has_mesh) {
        cudaSetDevice(c->device);
        return rebuild_tasks(c);
    }
    return SWE_OK;
}

int swe_get_tiling(swe_ctx* c, int32_t* seg_cells, int32_t* block_threads) {
    if (!c) return set_error(SWE_E_INVALID, "null context");
    if (seg_cells) *seg_cells = c->seg_cells;
    if (block_threads) *block_threads = c->block_threads;
    return SWE_OK;
}

int swe_mesh_upload(swe_ctx* c, int64_t n_cells, const int8_t* depth, const int8_t* plotter, int64_t n_edges,
                    const int64_t* edge_cells, const int8_t* edge_local, int64_t n_bnd, const int64_t* bnd_cell,
                    const int8_t* bnd_local) {
    if (!c) return set_error(SWE_E_INVALID, "null context");
    cudaSetDevice(c->device);
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    free_mesh_buffers(c);
    int rc = ingest_mesh(c->mesh, n_cells, depth, plotter, n_edges, edge_cells, edge_local, n_bnd, bnd_cell,
                         bnd_local);
    if (rc) return rc;
    const size_t n = (size_t)n_cells;
    for (int k = 0; k < 2; ++k) {
        if ((rc = device_alloc((void**)&c->h[k], n * 8)) || (rc = device_alloc((void**)&c->hu[k], n * 8)) ||
            (rc = device_alloc((void**)&c->hv[k], n * 8))) {
            free_mesh_buffers(c);
            return rc;
        }
    }
    if ((rc = device_alloc((void**)&c->b, n * 8)) || (rc = device_alloc((void**)&c->depth, n)) ||
        (rc = device_alloc((void**)&c->flags, n))) {
        free_mesh_buffers(c);
        return rc;
    }
    CUDA_TRY(cudaMemcpyAsync(c->depth, c->mesh.depth.data(), n, cudaMemcpyHostToDevice, c->stream));
    CUDA_TRY(cudaMemsetAsync(c->flags, 0, n, c->stream));
    c->has_mesh = true;
    if ((rc = rebuild_tasks(c))) {
        free_mesh_buffers(c);
        return rc;
    }
    set_scalars_kernel<<<1, 1, 0, c->stream>>>(c->scal, 0.0, 0.0, 1);
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    return SWE_OK;
}

static int current_index(swe_ctx* c, int* idx) {
    long long step = 0;
    CUDA_TRY(cudaMemcpyAsync(&step, &c->scal->step, sizeof(step), cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    *idx = (int)(step & 1);
    return SWE_OK;
}

int swe_state_upload(swe_ctx* c, const double* h, const double* hu, const double* hv, const double* b) {
    if (!c || !h || !hu || !hv || !b) return set_error(SWE_E_INVALID, "null argument");
    if (!c->has_mesh) return set_error(SWE_E_NOMESH, "upload a mesh first");
    cudaSetDevice(c->device);
    int k, rc;
    if ((rc = current_index(c, &k))) return rc;
    const size_t bytes = (size_t)c->mesh.n_cells * 8;
    CUDA_TRY(cudaMemcpyAsync(c->h[k], h, bytes, cudaMemcpyHostToDevice, c->stream));
    CUDA_TRY(cudaMemcpyAsync(c->hu[k], hu, bytes, cudaMemcpyHostToDevice, c->stream));
    CUDA_TRY(cudaMemcpyAsync(c->hv[k], hv, bytes, cudaMemcpyHostToDevice, c->stream));
    CUDA_TRY(cudaMemcpyAsync(c->b, b, bytes, cudaMemcpyHostToDevice, c->stream));
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    c->has_state = true;
    return SWE_OK;
}

int swe_state_download(swe_ctx* c, double* h, double* hu, double* hv, double* b) {
    if (!c) return set_error(SWE_E_INVALID, "null context");
    if (!c->has_state) return set_error(SWE_E_STATE, "no state uploaded");
    cudaSetDevice(c->device);
    int k, rc;
    if ((rc = current_index(c, &k))) return rc;
    const size_t bytes = (size_t)c->mesh.n_cells * 8;
    if (h) CUDA_TRY(cudaMemcpyAsync(h, c->h[k], bytes, cudaMemcpyDeviceToHost, c->stream));
    if (hu) CUDA_TRY(cudaMemcpyAsync(hu, c->hu[k], bytes, cudaMemcpyDeviceToHost, c->stream));
    if (hv) CUDA_TRY(cudaMemcpyAsync(hv, c->hv[k], bytes, cudaMemcpyDeviceToHost, c->stream));
    if (b) CUDA_TRY(cudaMemcpyAsync(b, c->b, bytes, cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    return SWE_OK;
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

int swe_set_time(swe_ctx* c, double time, double dt) {
    if (!c) return set_error(SWE_E_INVALID, "null context");
    cudaSetDevice(c->device);
    set_scalars_kernel<<<1, 1, 0, c->stream>>>(c->scal, time, dt, 0);
    CUDA_TRY(cudaGetLastError());
    return SWE_OK;
}

int swe_get_time(swe_ctx* c, double* time, double* dt, double* dt_new) {
    if (!c) return set_error(SWE_E_INVALID, "null context");
    cudaSetDevice(c->device);
    DevScalars s;
    CUDA_TRY(cudaMemcpyAsync(&s, c->scal, sizeof(s), cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    if (time) *time = s.time;
    if (dt) *dt = s.dt;
    if (dt_new) *dt_new = s.dt_new;
    return SWE_OK;
}

int swe_traverse(swe_ctx* c, int64_t n_steps) {
    if (!c) return set_error(SWE_E_INVALID, "null context");
    if (!c->has_mesh) return set_error(SWE_E_NOMESH, "upload a mesh first");
    if (!c->has_state) return set_error(SWE_E_STATE, "upload a state first");
    if (n_steps < 0) return set_error(SWE_E_INVALID, "n_steps < 0");
    cudaSetDevice(c->device);
    const swe_params& p = c->params;
    StepArgs A;
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
    A.scal = c->scal;
    A.drytol = p.dry_tolerance;
    A.courant = p.courant;
    A.scaling = p.scaling;
    // refinement thresholds: refinement_threshold * scaling * get_edge_size(dmax) (:339,:342)
    A.thr_refine = (5.0 * p.scaling) * c->leg[p.max_depth + 1];
    A.thr_coarsen = A.thr_refine / 8.0;
    A.max_time = p.max_time;
    A.tout = p.output_time_step;
    A.n_cells = (int32_t)c->mesh.n_cells;
    A.seg_cells = c->seg_cells;
    A.n_seg = (int32_t)c->n_seg;
    A.min_depth = p.min_depth;
    A.max_depth = p.max_depth;
    A.dmin = c->mesh.min_depth;
    A.ndepth = c->mesh.max_depth - c->mesh.min_depth + 1;
    A.bc = p.bc;
    A.use_tma = 1;
    StepKernel k = kernel_for(p.solver);
    for (int64_t s = 0; s < n_steps; ++s) {
        k<<<c->grid, c->block_threads, c->smem, c->stream>>>(A);
        CUDA_TRY(cudaGetLastError());
    }
    return SWE_OK;
}

int swe_get_refinements(swe_ctx* c, int8_t* flags, int64_t* n_refinements) {
    if (!c) return set_error(SWE_E_INVALID, "null context");
    if (!c->has_mesh) return set_error(SWE_E_NOMESH, "upload a mesh first");
    cudaSetDevice(c->device);
    if (flags) CUDA_TRY(cudaMemcpyAsync(flags, c->flags, (size_t)c->mesh.n_cells, cudaMemcpyDeviceToHost, c->stream));
    DevScalars s;
    CUDA_TRY(cudaMemcpyAsync(&s, c->scal, sizeof(s), cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    if (n_refinements) *n_refinements = (int64_t)s.n_refine;
    return SWE_OK;
}

int swe_get_step_count(swe_ctx* c, int64_t* steps) {
    if (!c || !steps) return set_error(SWE_E_INVALID, "null argument");
    cudaSetDevice(c->device);
    long long s = 0;
    CUDA_TRY(cudaMemcpyAsync(&s, &c->scal->step, sizeof(s), cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    *steps = s;
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
    int dev = 0;
    CUDA_TRY(cudaGetDevice(&dev));
    int rc = upload_tables_once();
    if (rc) return rc;
    double* d = nullptr;
    const size_t tot = (size_t)n * 18;
    if ((rc = device_alloc((void**)&d, tot * sizeof(double)))) return rc;
    double *dn = d, *dl = d + 2 * n, *dr = d + 6 * n, *ol = d + 10 * n, *orr = d + 14 * n;
    cudaError_t e = cudaMemcpy(dn, normals, 16 * (size_t)n, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dl, q_left, 32 * (size_t)n, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dr, q_right, 32 * (size_t)n, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        int blocks = (int)((n + 127) / 128);
        if (blocks > 4096) blocks = 4096;
        k<<<blocks, 128>>>(n, dn, dl, dr, dry_tolerance, ol, orr);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(out_left, ol, 32 * (size_t)n, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(out_right, orr, 32 * (size_t)n, cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) return set_error(SWE_E_CUDA, "riemann batch: %s", cudaGetErrorString(e));
    return SWE_OK;
}

int swe_mesh_uniform(int32_t depth, int64_t* n_cells, int64_t* n_edges, int64_t* n_bnd, int8_t* depth_out,
                     int8_t* plotter_out, int64_t* edge_cells, int8_t* edge_local, int64_t* bnd_cell,
                     int8_t* bnd_local, double* centroids) {
    return mesh_uniform(depth, n_cells, n_edges, n_bnd, depth_out, plotter_out, edge_cells, edge_local, bnd_cell,
                        bnd_local, centroids);
}

}  // extern "C"
