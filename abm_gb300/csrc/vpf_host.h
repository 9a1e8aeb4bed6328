// vpf_host.h -- host-side helpers shared by the library's translation units.
#pragma once
#include <cuda_runtime.h>

#include <vector>

#include "vpf_common.cuh"

namespace abm {

int set_error(int code, const char *fmt, ...);
int check_cuda(cudaError_t e, const char *what);
// Raise a kernel's dynamic shared-memory limit to `bytes` on the current device, once per
// (device, kernel).
int allow_dynamic_smem(const void *func, int bytes, const char *what);

// Launch with programmatic stream serialisation (see allow_dependent_launch): the kernel must
// call wait_primary_grid before it touches global memory that earlier work uses.
template <typename Args>
cudaError_t launch_pdl(void (*kern)(Args), unsigned blocks, unsigned threads, size_t smem,
                       cudaStream_t s, const Args &a) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(blocks);
    cfg.blockDim = dim3(threads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kern, a);
}

// Host copies of one grid's tables (built in FP64 / long double).
struct GridHostTables {
    GridDev g;                       // device pointers unset
    std::vector<float> mid, cot2;
    std::vector<long long> q, cpt;
};

int build_grid_host(int rv, double fov0, double fov1, GridHostTables &t);

// Cached device tables for (current device, rv, fov); built synchronously on first use.
const GridDev *grid_for(int rv, double fov0, double fov1, int *status);
// Integration-only tables for an explicit Phi grid (abm_vswrm_integrals).
const GridDev *grid_for_phi(int rv, const double *phi, int *status);

int np_arange_phi(int rv, std::vector<double> *out);
// Per-device global copy of the double-float sincos table used by df_sincos, and its host
// construction (cos/sin(k 2 pi / kSinCosTab) as (cos hi, cos lo, sin hi, sin lo)).
const float4 *sincos_table_dev(int *status);
void sincos_table_host(std::vector<float> &tab);
void np_linspace_pi(int n, std::vector<double> &out);
int find_nearest(const std::vector<double> &a, double v);

}  // namespace abm
