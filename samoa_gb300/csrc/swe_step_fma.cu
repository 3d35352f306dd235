// The step kernels compiled with FMA contraction (--fmad=true) in namespace
// swe_fma: the same source as the strict kernels, so the same algorithm and
// branches, with a*b+c fused where the compiler chooses. Results are not bit
// identical to the strict IEEE step; they stay within a few ulps per step.
#include <cuda_runtime.h>

#define SWE_KNS swe_fma
#include "swe_kernel.cuh"

namespace swe {

void* fma_step_kernel(int solver) {
    switch (solver) {
        case swe_fma::FWAVE: return (void*)swe_fma::step_kernel<swe_fma::FWAVE>;
        case swe_fma::AUG_RIEMANN: return (void*)swe_fma::step_kernel<swe_fma::AUG_RIEMANN>;
        case swe_fma::LF: return (void*)swe_fma::step_kernel<swe_fma::LF>;
        case swe_fma::LF_BATH: return (void*)swe_fma::step_kernel<swe_fma::LF_BATH>;
        case swe_fma::LLF: return (void*)swe_fma::step_kernel<swe_fma::LLF>;
        case swe_fma::LLF_BATH: return (void*)swe_fma::step_kernel<swe_fma::LLF_BATH>;
        default: return nullptr;
    }
}

void* fma_cross_kernel(int solver) {
    switch (solver) {
        case swe_fma::FWAVE: return (void*)swe_fma::cross_edges_kernel<swe_fma::FWAVE>;
        case swe_fma::AUG_RIEMANN: return (void*)swe_fma::cross_edges_kernel<swe_fma::AUG_RIEMANN>;
        case swe_fma::LF: return (void*)swe_fma::cross_edges_kernel<swe_fma::LF>;
        case swe_fma::LF_BATH: return (void*)swe_fma::cross_edges_kernel<swe_fma::LF_BATH>;
        case swe_fma::LLF: return (void*)swe_fma::cross_edges_kernel<swe_fma::LLF>;
        case swe_fma::LLF_BATH: return (void*)swe_fma::cross_edges_kernel<swe_fma::LLF_BATH>;
        default: return nullptr;
    }
}

cudaError_t fma_upload_tables() {
    double leg[kMaxDepth + 2], vol[kMaxDepth + 1], nrm[17][3][2];
    geometry_tables(leg, vol, nrm);
    cudaError_t e = cudaMemcpyToSymbol(swe_fma::c_leg, leg, sizeof(leg));
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(swe_fma::c_vol, vol, sizeof(vol));
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(swe_fma::c_normal, nrm, sizeof(nrm));
    return e;
}

}  // namespace swe
