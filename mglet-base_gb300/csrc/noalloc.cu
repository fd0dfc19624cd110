// noalloc.cu -- an allocation-free variant of the divergence maximum of
// itinfo (compdivmax, src/flow/timeintegration_mod.F90:376-414).
//
// mglet_gpu_itinfo works on a context the library allocated.  Some callers
// cannot let this library allocate device memory:
//  * a Fortran build whose fields already live on the device under another
//    runtime's ownership -- the reference's OpenMP-offload build maps every
//    field_t%arr with `omp target enter data` and hands device addresses to C
//    through use_device_ptr; a helper that called cudaMalloc behind that
//    runtime's back would split device memory between two allocators;
//  * per-step diagnostics inside the time loop (itinfo runs every itinfo
//    steps): cudaMalloc and cudaFree synchronise the whole device, which
//    stalls the stream the stage runs on.
// mglet_gpu_divmax_noalloc takes the fields and spacing as device pointers,
// writes its result to a device pointer, and keeps its only scratch -- one
// partial maximum per grid -- in a file-scope __device__ array of
// MGLET_NOALLOC_MAX_GRIDS doubles (512 KiB) that every GPU which loads the
// library holds until the process exits.
#include <mutex>

#include "../../include/mglet_gpu.h"
#include "internal.h"

namespace mg {
namespace {

// The scratch every call shares.  Its contents after a call are the per-grid
// maxima of that call; each call writes all the slots it reads, so nothing
// has to be cleared first.
static __device__ __align__(256) double g_noalloc_scratch[MGLET_NOALLOC_MAX_GRIDS];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
double* g_scratch_addr[kMaxDevices] = {nullptr};

// Device address of the scratch array on the current device.  Host code may
// not use g_noalloc_scratch directly: on the host that name is a stand-in
// object, not the device allocation.
int scratch_address(double** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_fail(e, "divmax_noalloc: cudaGetDevice");
    if (dev < 0 || dev >= kMaxDevices) {
        set_error("divmax_noalloc: device index beyond the supported range");
        return MGLET_ERR_ARG;
    }
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return cuda_fail(e, "divmax_noalloc: cudaGetSymbolAddress");
        g_scratch_addr[dev] = static_cast<double*>(p);
    }
    *out = g_scratch_addr[dev];
    return 0;
}

#define IX(k, j, i) ((long long)((i) - 1) * kk * jj + (long long)((j) - 1) * kk + ((k) - 1))

// max |div| over the interior of one grid (ib type noib: BP = 1, SDIV = 0).
__global__ void __launch_bounds__(256) k_divmax_grid(const double* __restrict__ U,
                                                     const double* __restrict__ V,
                                                     const double* __restrict__ W, int kk, int jj,
                                                     int ii, const double* __restrict__ RDDX,
                                                     const double* __restrict__ RDDY,
                                                     const double* __restrict__ RDDZ,
                                                     double* __restrict__ scratch) {
    __shared__ double sh[32];
    const int g = blockIdx.x;
    const long long o = (long long)g * kk * jj * ii;
    const double *u = U + o, *v = V + o, *w = W + o;
    const double *rddx = RDDX + (long long)g * ii - 1, *rddy = RDDY + (long long)g * jj - 1,
                 *rddz = RDDZ + (long long)g * kk - 1;
    const int ni = ii - 4, nj = jj - 4, nk = kk - 4;
    double dm = 0.0;
    for (int t = threadIdx.x; t < ni * nj * nk; t += blockDim.x) {
        const int k = t % nk + 3, j = (t / nk) % nj + 3, i = t / (nk * nj) + 3;
        const double div = (u[IX(k, j, i)] - u[IX(k, j, i - 1)]) * rddx[i] +
                           (v[IX(k, j, i)] - v[IX(k, j - 1, i)]) * rddy[j] +
                           (w[IX(k, j, i)] - w[IX(k - 1, j, i)]) * rddz[k];
        const double a = fabs(div);
        dm = (a > dm || a != a) ? a : dm;
    }
    for (int off = 16; off > 0; off >>= 1) {
        const double b = __shfl_xor_sync(0xffffffffu, dm, off);
        dm = (b > dm || b != b) ? b : dm;
    }
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = dm;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int q = 1; q < (int)(blockDim.x >> 5); ++q) dm = (sh[q] > dm || sh[q] != sh[q]) ? sh[q] : dm;
        scratch[g] = dm;
    }
}

__global__ void k_divmax_final(const double* __restrict__ scratch, int ngrid, double* out) {
    __shared__ double sh[32];
    double dm = 0.0;
    for (int g = threadIdx.x; g < ngrid; g += blockDim.x) {
        const double a = scratch[g];
        dm = (a > dm || a != a) ? a : dm;
    }
    for (int off = 16; off > 0; off >>= 1) {
        const double b = __shfl_xor_sync(0xffffffffu, dm, off);
        dm = (b > dm || b != b) ? b : dm;
    }
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = dm;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int q = 1; q < (int)(blockDim.x >> 5); ++q) dm = (sh[q] > dm || sh[q] != sh[q]) ? sh[q] : dm;
        out[0] = dm;
    }
}

}  // namespace
}  // namespace mg

extern "C" int mglet_gpu_divmax_noalloc(const double* u, const double* v, const double* w,
                                        int32_t ngrid, int32_t kk, int32_t jj, int32_t ii,
                                        const double* rddx, const double* rddy,
                                        const double* rddz, double* divmax, void* stream) {
    using namespace mg;
    if (!u || !v || !w || !rddx || !rddy || !rddz || !divmax) {
        set_error("divmax_noalloc: null pointer argument");
        return MGLET_ERR_ARG;
    }
    if (ngrid <= 0 || kk < 5 || jj < 5 || ii < 5) {
        set_error("divmax_noalloc: grid count and dimensions must be positive with interior cells");
        return MGLET_ERR_ARG;
    }
    if (ngrid > MGLET_NOALLOC_MAX_GRIDS) {
        set_error("divmax_noalloc: ngrid exceeds MGLET_NOALLOC_MAX_GRIDS (65536); "
                  "use mglet_gpu_itinfo on a context for larger hierarchies");
        return MGLET_ERR_SIZE;
    }
    double* scratch = nullptr;
    if (int rc = scratch_address(&scratch)) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    k_divmax_grid<<<ngrid, 256, 0, s>>>(u, v, w, kk, jj, ii, rddx, rddy, rddz, scratch);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "divmax_noalloc: launch");
    k_divmax_final<<<1, 1024, 0, s>>>(scratch, ngrid, divmax);
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "divmax_noalloc: launch");
    return 0;
}
