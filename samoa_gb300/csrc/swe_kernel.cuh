// The fused SWE time-step kernel (sm_103a).
//
// One launch = one explicit Euler time step of every instance of the context
// (one instance for the plain step, many for an ensemble) of
// t_swe_euler_timestep_traversal (src/SWE/SWE_euler_timestep.f90). Cells are
// cut into segments of consecutive cells of the space-filling curve; a
// segment never spans two instances. A persistent grid of CTAs walks the
// segments; per segment:
//   1. stage h, hu, hv, b into shared memory with 1-D TMA bulk copies
//      (cp.async.bulk, completion on an mbarrier with a bounded wait), then
//      the depth h - b and sqrt(g * depth) once per cell;
//   2. evaluate each edge task once: the Riemann solver with the first-touched
//      cell as the left side writes left/right updates into per-(cell, local
//      edge) slots in shared memory, each slot written by one task, no atomics;
//      an edge between two segments is evaluated by both CTAs, each keeping
//      its own side, so no CTA waits for another;
//   3. update each cell from its three slots in local edge index order, clamp
//      wet/dry, write the other state buffer, set the refinement flag, fold
//      volume / sum(len * speed) into a running minimum;
// at an instance change and at the end the CTA reduces the minimum with warp
// shuffles and folds it into the instance with one atomic; the last CTA to
// finish advances every instance's time and dt and the step counter.
// The reference's traversal direction alternates every step
// (src/SFC_generic_traversal_ringbuffer.f90:420): on odd steps the
// higher-numbered cell of an edge is touched first and the two leg updates are
// summed in the other order.
#pragma once

// The kernels are compiled twice: in namespace swe with strict IEEE rounding
// (no contraction) and in namespace swe_fma with FMA contraction (SWE_KNS).
#ifndef SWE_KNS
#define SWE_KNS swe
#endif

#include <cfloat>
#include <cstdint>

#include "swe_internal.h"
#include "swe_riemann.cuh"

namespace SWE_KNS {
using namespace ::swe;

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
    const int4* seg_info;      // {first cell, cells, instance, halo tasks at the end of its list}
    const int32_t* seg_order;  // the order segments are handed out in (a permutation), or null: curve order
    const int4* xtasks;        // cross-segment edges (Task layout, pad = instance)
    double* xflux;             // [n_xtasks][cell a, cell b][h, hu, hv, max wave speed] of the current step
    long long n_xtasks;
    uint16_t* erec;            // branch-frozen runs: this step's edge decisions, per task ...
    uint16_t* xrec;            // ... and per cross-segment edge
    const InstParams* ip;
    InstScalars* is;
    GlobalScalars* gs;
    uint8_t* branch;           // optional per-cell output: bit 0 wetting fix, bit 1 drying clamp (adjoint)
    const double* dt_seq;      // frozen dt sequence [k * n_inst + inst] or null
    long long dt_seq_len;      // steps in the sequence
    int32_t n_seg, n_inst, seg_cells, max_ndepth, n_cells_total;
    int32_t use_tma;
    int32_t fixed_io;          // 1: read h[0], hu[0], hv[0] and write h[1].. on every step (caller's buffers)
    int32_t stage_depth;       // 1: stage a segment, then work on it; 2: stage the next one meanwhile
    int32_t halo_solve;        // 1: solve the halo tasks here (no cross-edge pass); 0: copy the pass's updates
    double2* memo;             // per cell (d, sqrt(g d)) of an earlier step, or null: see the staging loop
    uint32_t extra_tx;         // fault injection only: bytes the staging barrier expects beyond the copies (0)
    unsigned long long wait_ns;  // limit of one mbarrier wait, in ns of the global timer
};

// Launch bounds of the step kernel: at most 256 threads; with SWE_MIN_BLOCKS
// defined, also that many resident CTAs of 256 threads (registers capped at
// 65536 / (256 * SWE_MIN_BLOCKS)). Undefined: the compiler's own register choice.
#ifdef SWE_MIN_BLOCKS
#define SWE_STEP_BOUNDS __launch_bounds__(256, SWE_MIN_BLOCKS)
#else
#define SWE_STEP_BOUNDS __launch_bounds__(256)
#endif

// An mbarrier wait gives up after wait_ns of the global timer (1 s by default;
// the copies it waits for take microseconds), or after kPollLimit polls
// whatever the timer says, so that every wait ends.
constexpr unsigned long long kWaitNs = 1000000000ull;
constexpr unsigned int kPollLimit = 1u << 30;

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

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

// 1-D bulk copy global -> this CTA's shared memory; addresses 16-byte aligned,
// size a multiple of 16.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

// Prefetch into L2 the 16-byte-aligned part of [p, p + bytes), for any p (the
// bulk prefetch wants a 16-byte aligned address and size): it touches no byte
// outside the range, writes nothing, and has no completion to wait for.
__device__ __forceinline__ void prefetch_l2(const void* p, size_t bytes) {
    const uintptr_t a = ((uintptr_t)p + 15u) & ~(uintptr_t)15u, e = ((uintptr_t)p + bytes) & ~(uintptr_t)15u;
    if (e > a)
        asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(a), "r"((uint32_t)(e - a)));
}

__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

__device__ __forceinline__ double warp_min(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = dmn(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

__device__ __forceinline__ unsigned long long warp_max_u64(unsigned long long v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long w = __shfl_xor_sync(0xffffffffu, v, o);
        v = w > v ? w : v;
    }
    return v;
}

__device__ __forceinline__ long long warp_sum(long long v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// dt of step `step` for instance `inst`: the frozen sequence if one is set,
// else grid%r_dt clamped as in pre_traversal_grid_op (src/SWE/SWE_euler_timestep.f90:89-109)
__device__ __forceinline__ double step_dt(const StepArgs& A, const InstParams& P, int inst, long long k) {
    if (A.dt_seq && k >= 0 && k < A.dt_seq_len) return A.dt_seq[k * A.n_inst + inst];
    double dt = A.is[inst].dt;
    if (P.max_time > 0.0) dt = dmn(P.max_time, dt);
    if (P.tout > 0.0) dt = dmn(P.tout, dt);
    return dt;
}

// Block-wide reduction of (dtmin, dskey, nref) into instance `inst`; all threads call it.
__device__ __forceinline__ void flush_instance(const StepArgs& A, int inst, double& dtmin, unsigned long long& dskey,
                                               long long& nref, double* red_min, unsigned long long* red_max,
                                               long long* red_sum) {
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    double m = warp_min(dtmin);
    unsigned long long x = warp_max_u64(dskey);
    long long s = warp_sum(nref);
    if (lane == 0) {
        red_min[warp] = m;
        red_max[warp] = x;
        red_sum[warp] = s;
    }
    __syncthreads();
    if (warp == 0) {
        const int nw = (blockDim.x + 31) >> 5;
        m = lane < nw ? red_min[lane] : DBL_MAX;
        x = lane < nw ? red_max[lane] : 0ull;
        s = lane < nw ? red_sum[lane] : 0;
        m = warp_min(m);
        x = warp_max_u64(x);
        s = warp_sum(s);
        if (lane == 0) {
            // non-negative doubles order like their bit patterns
            if (m != DBL_MAX) atomicMin(&A.is[inst].dt_acc, (unsigned long long)__double_as_longlong(m));
            if (x) atomicMax(&A.is[inst].ds_acc, x);
            if (s) atomicAdd(&A.is[inst].refine_acc, (unsigned long long)s);
        }
    }
    __syncthreads();
    dtmin = DBL_MAX;
    dskey = 0;
    nref = 0;
}

// The edges between two segments, one thread each, before the step kernel:
// the same flux as the step kernel's edge tasks (orientation by the step's
// parity, pre-update states), both sides' updates stored by cell (a, then b).
// depth_terms for the cross-edge pass: sqrt(g d) from the memo when the depth has
// the same bits (the pass only reads it; the step kernel's owner CTAs write it),
// and, for the f-wave, no RN(1 / d) for a cell with both momenta +-0 (its
// quotients are zeros with the numerator's sign for any positive reciprocal).
template <int SOLVER>
__device__ __forceinline__ void cross_depth_terms(const StepArgs& A, int c, const State& Q, double drytol, double& d,
                                                  double& sq, double& y) {
    d = Q.h - Q.b;
    const bool wet = lt(drytol, d);
    sq = 0.0;
    y = 0.0;
    if (!wet) return;
    bool hit = false;
    if (A.memo) {
        const double2 m = A.memo[c];
        if (dbits(m.x) == dbits(d)) {
            sq = m.y;
            hit = true;
        }
    }
    if (!hit) sq = sqrt(kG * d);
    const bool still = ((dbits(Q.p1) | dbits(Q.p2)) << 1) == 0;
    y = (SOLVER == FWAVE && still) ? 1.0 : recip_rn(d).y;
}

template <int SOLVER, int FZ = 0>
__global__ void __launch_bounds__(256) cross_edges_kernel(const StepArgs A) {
    const long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= A.n_xtasks) return;
    const long long step = A.gs->step;
    const int odd = (int)(step & 1);
    const int ib = A.fixed_io ? 0 : odd;
    const double* hin = A.h[ib];
    const double* huin = A.hu[ib];
    const double* hvin = A.hv[ib];
    const int4 tk = __ldg(&A.xtasks[j]);
    const uint32_t meta = (uint32_t)tk.z;
    int L, R, iL, pL;
    if (!odd) {
        L = tk.x; iL = meta & 3u; pL = (meta >> 4) & 31u;
        R = tk.y;
    } else {
        L = tk.y; iL = (meta >> 2) & 3u; pL = (meta >> 9) & 31u;
        R = tk.x;
    }
    if ((unsigned)L >= (unsigned)A.n_cells_total || (unsigned)R >= (unsigned)A.n_cells_total || iL > 2 ||
        pL > 16 || (unsigned)tk.w >= (unsigned)A.n_inst || ((meta >> 14) & 1u)) {
        atomicOr(&A.gs->error, 1u);
        return;
    }
    const double drytol = A.ip[tk.w].drytol;
    const double n1 = c_normal[pL][iL][0], n2 = c_normal[pL][iL][1];
    const State QL{hin[L], huin[L], hvin[L], A.b[L]};
    const State QR{hin[R], huin[R], hvin[R], A.b[R]};
    double dL, dR, sqL, sqR, yL, yR;
    cross_depth_terms<SOLVER>(A, L, QL, drytol, dL, sqL, yL);
    cross_depth_terms<SOLVER>(A, R, QR, drytol, dR, sqR, yR);
    Update fL, fR;
    edge_flux<SOLVER, FZ>(n1, n2, QL, QR, dL, dR, sqL, sqR, yL, yR, drytol, fL, fR, (int)((meta >> 15) & 3u),
                          FZ ? &A.xrec[j] : nullptr);
    const Update& ua = odd ? fR : fL;
    const Update& ub = odd ? fL : fR;
    double2* out = reinterpret_cast<double2*>(A.xflux + 8 * j);
    out[0] = make_double2(ua.h, ua.p1);
    out[1] = make_double2(ua.p2, ua.s);
    out[2] = make_double2(ub.h, ub.p1);
    out[3] = make_double2(ub.p2, ub.s);
}

// Round-up float of |x| for x = +-0 or 2^-100 <= |x| < 2^101, from the bit
// pattern (integer operations): the significand truncated to 23 bits plus one
// unit in the last place (a carry into the exponent is still an upper bound).
// False for other x (tiny, huge, inf, NaN).
__device__ __forceinline__ bool float_up(double x, float& f) {
    const unsigned long long a = (unsigned long long)abs_bits(x);
    f = 0.0f;
    if (a == 0ull) return true;
    const int e = (int)(a >> 52) - 1023;
    if (e < -100 || e > 100) return false;
    f = __uint_as_float(((unsigned)(e + 127) << 23 | (unsigned)((a >> 29) & 0x7fffffull)) + 1u);
    return true;
}

// True when the CFL key RN(ds 2^k) of a cell is certainly below the key m (bits
// of a nonnegative double), so that the cell cannot raise a maximum >= m; ds =
// RN(RN(RN(leg s0) + RN(hyp s1)) + RN(leg s2)) is the cell update's speed sum,
// up = (leg, hyp) rounded up to float. U = leg s0 + hyp s1 + leg s2 evaluated in
// float with every operand and every operation rounded up bounds the exact sum
// of the magnitudes S; the three roundings of ds give |ds| <= S (1 + 2^-53)^3
// (and an absolute error below 2^-1072 where a result is subnormal), both below
// the margin U 2^-20 of a normal float U; 2^k scales exactly, and a bound that
// is not a finite double gives false. The float work runs beside the FP64 pipe.
__device__ __forceinline__ bool key_below(float2 up, double s0, double s1, double s2, int k, unsigned long long m) {
    float f0, f1, f2;
    if (!float_up(s0, f0) || !float_up(s1, f1) || !float_up(s2, f2)) return false;
    float U = __fmaf_ru(up.x, f0, __fmaf_ru(up.y, f1, __fmul_ru(up.x, f2)));
    U = __fmul_ru(U, 1.00000095367431640625f);  // 1 + 2^-20
    const unsigned int ub = __float_as_uint(U);
    const int ef = (int)(ub >> 23);  // U >= 0
    if (ef == 0 || ef == 255) return false;
    const int eb = ef - 127 + 1023 + k;
    if (eb >= 2047) return false;
    const unsigned long long bound = ((unsigned long long)eb << 52) | ((unsigned long long)(ub & 0x7fffffu) << 29);
    return bound < m;
}

template <int SOLVER, int FZ = 0>
__global__ void SWE_STEP_BOUNDS step_kernel(const StepArgs A) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int T = A.seg_cells;
    // staging buffers [stage_depth][h, hu, hv, b][T]: with depth 2 the next
    // segment's bulk copies land in one buffer while the CTA works on the other
    const bool depth2 = A.stage_depth > 1;
    double* stage = reinterpret_cast<double*>(smem_raw);
    double* sh_rh = stage + (depth2 ? 8 : 4) * T;  // RN(1 / depth) where the cell is wet
    double* sh_sq = sh_rh + T;      // sqrt(g * depth) where the cell is wet
    double* upd = sh_sq + T;        // [4 quantities][3 local edges][T cells]
    double* tab_leg = upd + 12 * T; // per depth of the current instance
    double* tab_hyp = tab_leg + A.max_ndepth;
    double* tab_vol = tab_hyp + A.max_ndepth;
    double* tab_ndv = tab_vol + A.max_ndepth;  // -dt / volume
    double* tab_pow = tab_ndv + A.max_ndepth;  // 2^(d+1)
    float2* tab_up = reinterpret_cast<float2*>(tab_pow + A.max_ndepth);  // (leg, hyp) rounded up to float
    __shared__ uint64_t bar[2];
    __shared__ double red_min[32];
    __shared__ unsigned long long red_max[32];
    __shared__ long long red_sum[32];
    __shared__ unsigned int s_error;
    __shared__ int s_last;
    __shared__ int s_seg;

    const int tid = threadIdx.x;
    const long long step = A.gs->step;
    const long long kseq = step - A.gs->dt_seq_base;
    const int odd = (int)(step & 1);
    const int ib = A.fixed_io ? 0 : odd;
    const double* hin = A.h[ib];
    const double* huin = A.hu[ib];
    const double* hvin = A.hv[ib];
    double* hout = A.h[ib ^ 1];
    double* huout = A.hu[ib ^ 1];
    double* hvout = A.hv[ib ^ 1];

    if (tid == 0) {
        s_error = 0;
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        fence_mbar_init();
    }
    __syncthreads();

    double dtmin = DBL_MAX;  // r_dt_new = huge(1.0) (pre_traversal_op, :133-140)
    unsigned long long dskey = 0;  // bits of max ds * 2^(d+1) (dt_by_max)
    long long nref = 0;
    uint32_t phase = 0;    // bit k: parity of barrier k
    uint32_t pending = 0;  // bit k: bulk copies in flight into buffer k
    int cur = -1;
    InstParams P;

    // Stage segment `sg` into buffer k: bulk copies of the 16-byte multiple (the
    // segment starts at an even cell) completing on barrier k, plain loads for an
    // odd tail cell or for host memory. All threads call it.
    auto issue = [&](int sg, int k) {
        const int4 si = __ldg(&A.seg_info[sg]);
        const int c0 = si.x, cn = si.y;
        double* bh = stage + (size_t)k * 4 * T;
        const int cbulk = A.use_tma ? (cn & ~1) : 0;
        if (cbulk > 0) {
            if (tid == 0) {
                fence_proxy_async();
                const uint32_t bytes = (uint32_t)cbulk * 8u;
                mbar_arrive_expect_tx(&bar[k], 4u * bytes + A.extra_tx);
                bulk_g2s(bh, hin + c0, bytes, &bar[k]);
                bulk_g2s(bh + T, huin + c0, bytes, &bar[k]);
                bulk_g2s(bh + 2 * T, hvin + c0, bytes, &bar[k]);
                bulk_g2s(bh + 3 * T, A.b + c0, bytes, &bar[k]);
            }
            pending |= 1u << k;
        }
        if (tid == 0) {
            // the segment's edge tasks, memo entries and depths, read later in
            // task or thread order, are on their way to L2 while its state lands
            const long long a = __ldg(&A.seg_ptr[sg]), e = __ldg(&A.seg_ptr[sg + 1]);
            prefetch_l2(A.tasks + a, (size_t)(e - a) * 16u);
            if (A.memo) prefetch_l2(A.memo + c0, (size_t)cn * 16u);
            prefetch_l2(A.depth + c0, (size_t)cn);
        }
        for (int i = cbulk + tid; i < cn; i += blockDim.x) {
            bh[i] = hin[c0 + i];
            bh[T + i] = huin[c0 + i];
            bh[2 * T + i] = hvin[c0 + i];
            bh[3 * T + i] = A.b[c0 + i];
        }
    };
    // Wait (one thread, bounded) for buffer k's bulk copies.
    auto wait = [&](int k) {
        if (pending & (1u << k)) {
            if (tid == 0) {
                unsigned int polls = 0;
                unsigned long long t0 = 0;
                while (!mbar_try_wait(&bar[k], (phase >> k) & 1u)) {
                    ++polls;
                    if ((polls & 63u) == 1u) {
                        const unsigned long long now = global_ns();
                        if (polls == 1u) t0 = now;
                        else if (now - t0 > A.wait_ns) polls = kPollLimit;
                    }
                    if (polls >= kPollLimit) {
                        s_error = 2u;
                        break;
                    }
                }
            }
            phase ^= 1u << k;
            pending &= ~(1u << k);
        }
    };

    // segments are handed out dynamically (CTAs that draw cheap segments, e.g.
    // dry land, take more), in the order seg_order gives: spread over the
    // domain, so that the CTAs an SM holds at one time mix wet and dry work
    auto draw = [&]() {
        const int k = (int)atomicAdd(&A.gs->next_seg, 1u);
        s_seg = k < A.n_seg ? (A.seg_order ? __ldg(&A.seg_order[k]) : k) : A.n_seg;
    };
    if (tid == 0) draw();
    __syncthreads();
    int seg = s_seg;
    int kbuf = 0;
    if (seg < A.n_seg) issue(seg, 0);
    while (seg < A.n_seg) {
        int seg_next = A.n_seg;
        if (depth2) {  // draw and stage the next segment before working on this one
            __syncthreads();
            if (tid == 0) draw();
            __syncthreads();
            seg_next = s_seg;
            if (seg_next < A.n_seg) issue(seg_next, kbuf ^ 1);
        }
        const int4 si = __ldg(&A.seg_info[seg]);
        const int c0 = si.x, cn = si.y, inst = si.z;
        if (inst != cur) {  // uniform across the CTA
            if (cur >= 0) flush_instance(A, cur, dtmin, dskey, nref, red_min, red_max, red_sum);
            P = A.ip[inst];
            const double dt = step_dt(A, P, inst, kseq);
            for (int i = tid; i < P.ndepth; i += blockDim.x) {
                const int d = P.dmin + i;
                const double vol = (P.scaling * P.scaling) * c_vol[d];
                const double leg = P.scaling * c_leg[d + 1], hyp = P.scaling * c_leg[d];
                tab_leg[i] = leg;
                tab_hyp[i] = hyp;
                tab_up[i] = make_float2(__double2float_ru(leg), __double2float_ru(hyp));
                tab_vol[i] = vol;
                tab_ndv[i] = -dt / vol;
                tab_pow[i] = ldexp(2.0, d);
            }
            cur = inst;
        }
        // ---- 1. the segment's state, staged in buffer kbuf
        wait(kbuf);
        __syncthreads();
        if (s_error) break;
        double* sh_h = stage + (size_t)kbuf * 4 * T;
        double* sh_hu = sh_h + T;
        double* sh_hv = sh_hu + T;
        double* sh_b = sh_hv + T;
        for (int i = tid; i < cn; i += blockDim.x) {
            // depth_terms, with the square root and reciprocal skipped by warps of dry cells.
            // The f-wave path divides only the cell's own (rotated) momenta by its depth:
            // with both momenta +-0 every such quotient is a zero with the numerator's
            // sign for any positive reciprocal, so those cells skip RN(1 / d) (1.0 stands in)
            // sqrt(g d) comes from the memo when the cell's depth has the same bits as
            // the depth it was last taken for (water at rest keeps its depth from step
            // to step); the memo holds only pairs (d, sqrt(g d)), written by the CTA
            // that owns the cell, so a hit is the value the square root would give
            const double d = sh_h[i] - sh_b[i];
            const bool wet = lt(P.drytol, d);
            const bool need_y = wet && (SOLVER != FWAVE || ((dbits(sh_hu[i]) | dbits(sh_hv[i])) << 1) != 0);
            double sq = 0.0, y = wet ? 1.0 : 0.0;
            bool miss = wet;
            if (wet && A.memo) {
                const double2 m = A.memo[c0 + i];
                if (dbits(m.x) == dbits(d)) {
                    sq = m.y;
                    miss = false;
                }
            }
            if (__any_sync(__activemask(), miss)) {
                if (miss) {
                    sq = sqrt(kG * d);
                    if (A.memo) A.memo[c0 + i] = make_double2(d, sq);
                }
            }
            if (__any_sync(__activemask(), need_y)) y = need_y ? recip_rn(d).y : y;
            sh_rh[i] = y;
            sh_sq[i] = sq;
        }
        // halo tasks: the cross-edge pass computed these edges' updates; copy
        // this segment's side into its slot
        const long long t0 = A.seg_ptr[seg], t1 = A.seg_ptr[seg + 1];
        const long long tm = A.halo_solve ? t1 : t1 - min((long long)max(si.w, 0), t1 - t0);
        for (long long t = tm + tid; t < t1; t += blockDim.x) {
            const int4 tk = __ldg(&A.tasks[t]);
            const uint32_t meta = (uint32_t)tk.z;
            const int sa = tk.x - c0;
            const bool ain = (unsigned)sa < (unsigned)cn;
            const int cl = ain ? sa : tk.y - c0;
            const int le = ain ? (int)(meta & 3u) : (int)((meta >> 2) & 3u);
            if ((unsigned)cl >= (unsigned)cn || le > 2 || !(meta & (1u << 17)) ||
                (unsigned long long)(unsigned)tk.w >= (unsigned long long)A.n_xtasks) {
                atomicOr(&s_error, 1u);
                continue;
            }
            const double2* u = reinterpret_cast<const double2*>(A.xflux + 8 * (long long)(unsigned)tk.w + (ain ? 0 : 4));
            const double2 u0 = u[0], u1 = u[1];
            upd[(0 * 3 + le) * T + cl] = u0.x;
            upd[(1 * 3 + le) * T + cl] = u0.y;
            upd[(2 * 3 + le) * T + cl] = u1.x;
            upd[(3 * 3 + le) * T + cl] = u1.y;
        }
        __syncthreads();

        // ---- 2. edge tasks (skeleton_scalar_op / bnd_skeleton_scalar_op, :196-255)
        // each thread loads its next task while it works on the current one
        int4 tk_next = make_int4(0, 0, 0, 0);
        if (t0 + tid < tm) tk_next = __ldg(&A.tasks[t0 + tid]);
        for (long long t = t0 + tid; t < tm; t += blockDim.x) {
            const int4 tk = tk_next;
            if (t + blockDim.x < tm) tk_next = __ldg(&A.tasks[t + blockDim.x]);
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
            if ((unsigned)L >= (unsigned)A.n_cells_total || (!bnd && (unsigned)R >= (unsigned)A.n_cells_total) ||
                iL > 2 || iR > 2 || pL > 16) {
                atomicOr(&s_error, 1u);
                continue;
            }
            const double n1 = c_normal[pL][iL][0], n2 = c_normal[pL][iL][1];
            const int sl = L - c0, sr = R - c0;
            const bool lin = (unsigned)sl < (unsigned)cn;
            const bool rin = !bnd && (unsigned)sr < (unsigned)cn;
            State QL, QR;
            double dL, dR, sqL, sqR, yL, yR;
            if (lin) {
                QL = State{sh_h[sl], sh_hu[sl], sh_hv[sl], sh_b[sl]};
                dL = QL.h - QL.b;
                sqL = sh_sq[sl];
                yL = sh_rh[sl];
            } else {
                QL = State{hin[L], huin[L], hvin[L], A.b[L]};
                depth_terms(QL, P.drytol, dL, sqL, yL);
            }
            if (bnd) {  // the ghost has the cell's h and b
                if (P.bc == BC_SLIP) QR = boundary_ghost<BC_SLIP>(n1, n2, QL);
                else if (P.bc == BC_NOSLIP) QR = boundary_ghost<BC_NOSLIP>(n1, n2, QL);
                else QR = QL;
                dR = dL;
                sqR = sqL;
                yR = yL;
            } else if (rin) {
                QR = State{sh_h[sr], sh_hu[sr], sh_hv[sr], sh_b[sr]};
                dR = QR.h - QR.b;
                sqR = sh_sq[sr];
                yR = sh_rh[sr];
            } else {
                QR = State{hin[R], huin[R], hvin[R], A.b[R]};
                depth_terms(QR, P.drytol, dR, sqR, yR);
            }
            Update fL, fR;
            edge_flux<SOLVER, FZ>(n1, n2, QL, QR, dL, dR, sqL, sqR, yL, yR, P.drytol, fL, fR,
                                  (int)((meta >> 15) & 3u), FZ ? &A.erec[t] : nullptr);
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
        // With one staging buffer, thread 0 takes the next segment's ticket now and
        // reads it after its cells, so the atomic's round trip overlaps the updates.
        unsigned int ticket = 0u;
        if (!depth2 && tid == 0) ticket = atomicAdd(&A.gs->next_seg, 1u);
        const int k0 = odd ? 2 : 0, k2 = odd ? 0 : 2;
        // the largest CFL key the lanes of this warp have taken so far (dt_by_max);
        // a cell whose key is certainly below it cannot raise the maximum
        const unsigned long long wkey = P.dt_by_max ? warp_max_u64(dskey) : 0ull;
        for (int i = tid; i < cn; i += blockDim.x) {
            const int c = c0 + i;
            const int d = A.depth[c];
            const int di = d - P.dmin;
            const double leg = tab_leg[di], hyp = tab_hyp[di], ndv = tab_ndv[di];
            double u[4][3];
            long long nz = 0, sz = 0;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                u[q][0] = upd[(q * 3 + k0) * T + i];
                u[q][1] = upd[(q * 3 + 1) * T + i];
                u[q][2] = upd[(q * 3 + k2) * T + i];
                (q < 3 ? nz : sz) |= (dbits(u[q][0]) | dbits(u[q][1]) | dbits(u[q][2])) << 1;
            }
            // quiet: every update of h, hu, hv is +-0 (dry land, water at rest). Then
            // each sum below is +0 (positive edge lengths), RN(ndv * +0) is a zero with
            // ndv's sign, and adding it leaves the state as add_zero says: the same
            // bits, without the FP64 arithmetic. Water at rest still has wave speeds,
            // so the speed sum ds has its own test below.
            const bool quiet = nz == 0 && is_finite(ndv);
            double dh = 0.0, dp1 = 0.0, dp2 = 0.0, ds = 0.0;
            if (__any_sync(__activemask(), !quiet)) {
                if (!quiet) {
                    dh = z0(prod_cell(leg, u[0][0])) + prod_cell(hyp, u[0][1]);
                    dh = dh + prod_cell(leg, u[0][2]);
                    dp1 = z0(prod_cell(leg, u[1][0])) + prod_cell(hyp, u[1][1]);
                    dp1 = dp1 + prod_cell(leg, u[1][2]);
                    dp2 = z0(prod_cell(leg, u[2][0])) + prod_cell(hyp, u[2][1]);
                    dp2 = dp2 + prod_cell(leg, u[2][2]);
                }
            }
            // ds is +0 when every speed is +-0 (dry land) or when the cell's key stays
            // below wkey (key_below), else it is summed
            bool need_ds = sz != 0;
            if (need_ds && wkey != 0ull) need_ds = !key_below(tab_up[di], u[3][0], u[3][1], u[3][2], d + 1, wkey);
            if (__any_sync(__activemask(), need_ds)) {
                if (need_ds) {
                    ds = z0(prod_cell(leg, u[3][0])) + prod_cell(hyp, u[3][1]);
                    ds = ds + prod_cell(leg, u[3][2]);
                }
            }
            int8_t f = 0;
            // |dh| > thr and |dh| < thr / 8 on the bit patterns (thresholds are positive;
            // a NaN |dh| passes neither test, as in IEEE)
            const long long nrm = abs_bits(dh);
            if (d < P.max_depth && not_nan(nrm) && nrm > __double_as_longlong(P.thr_refine)) {
                f = 1;
                ++nref;
            } else if (d > P.min_depth && nrm < __double_as_longlong(P.thr_coarsen)) {
                f = -1;
            }
            if (P.dt_by_max) {  // ds >= 0, so its bits order like its value; RN(ds * 2^(d+1))
                const unsigned long long x = (unsigned long long)dbits(scale_pow2(ds, d + 1, tab_pow[di]));
                dskey = x > dskey ? x : dskey;
            } else {
                dtmin = dmn(dtmin, tab_vol[di] / ds);
            }
            if (quiet) {
                dh = dp1 = dp2 = bitsd(dbits(ndv) & (long long)0x8000000000000000ULL);  // RN(ndv * +0)
            } else {
                dh = prod_cell(ndv, dh);
                dp1 = prod_cell(ndv, dp1);
                dp2 = prod_cell(ndv, dp2);
            }
            double h = sh_h[i], p1 = sh_hu[i], p2 = sh_hv[i];
            const double b = sh_b[i];
            uint8_t br = 0;
            const double bdry = b + P.drytol;
            const uint8_t rb = FZ == 2 ? A.branch[c] : 0;  // a branch-frozen run takes the recorded fixes
            // flooded land starts at the dry tolerance, at rest
            if (FZ == 2 ? (rb & 1u) != 0 : (lt(h, bdry) && gt0(dh))) {
                h = bdry;
                p1 = 0.0;
                p2 = 0.0;
                br = 1;
            }
            if (quiet) {
                h = add_zero(h, dh);
                p1 = add_zero(p1, dp1);
                p2 = add_zero(p2, dp2);
            } else {
                h = h + dh;
                p1 = p1 + dp1;
                p2 = p2 + dp2;
            }
            if (FZ == 2 ? (rb & 2u) != 0 : lt(h, bdry)) {  // dried out: surface to min(b, 0), at rest
                h = lt0(b) ? b : 0.0;
                p1 = 0.0;
                p2 = 0.0;
                br |= 2;
            }
            if (FZ != 2 && A.branch) A.branch[c] = br;
            hout[c] = h;
            huout[c] = p1;
            hvout[c] = p2;
            A.flags[c] = f;
        }
        if (!depth2 && tid == 0) {
            const int k = (int)ticket;
            s_seg = k < A.n_seg ? (A.seg_order ? __ldg(&A.seg_order[k]) : k) : A.n_seg;
        }
        __syncthreads();
        if (!depth2) {  // stage the next segment now
            seg_next = s_seg;
            if (seg_next < A.n_seg) issue(seg_next, 0);
        } else {
            kbuf ^= 1;
        }
        seg = seg_next;
    }
    if (pending) {  // left early on an error: let the copies in flight land first (bounded)
        wait(0);
        wait(1);
    }

    // ---- 4. reductions and the last-CTA finalisation (post_traversal_grid_op, :111-131)
    if (cur >= 0) flush_instance(A, cur, dtmin, dskey, nref, red_min, red_max, red_sum);
    if (tid == 0) {
        if (s_error) atomicOr(&A.gs->error, s_error);
        __threadfence();
        s_last = atomicAdd(&A.gs->done, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (s_last) {
        __threadfence();
        for (int i = tid; i < A.n_inst; i += blockDim.x) {
            const InstParams Q = A.ip[i];
            const double dt = step_dt(A, Q, i, kseq);
            InstScalars* S = &A.is[i];
            double dtn = __longlong_as_double((long long)atomicAdd(&S->dt_acc, 0ull));
            const unsigned long long x = atomicAdd(&S->ds_acc, 0ull);
            if (x) dtn = dmn(dtn, (Q.scaling * Q.scaling) / __longlong_as_double((long long)x));
            S->time = S->time + dt;
            S->dt_new = dtn;
            S->dt = Q.courant * dtn;
            S->n_refine = atomicExch(&S->refine_acc, 0ull);
            S->dt_acc = (unsigned long long)__double_as_longlong(DBL_MAX);
            S->ds_acc = 0;
        }
        __syncthreads();
        if (tid == 0) {
            A.gs->done = 0;
            A.gs->next_seg = 0;
            A.gs->step = step + 1;
            __threadfence();
        }
    }
}

}  // namespace SWE_KNS
