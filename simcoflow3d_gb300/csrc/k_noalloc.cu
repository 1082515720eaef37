// k_noalloc.cu -- operator apply that allocates nothing.
//
// scf_apply_operator_noalloc computes y = A x and the energy x.Ax for a
// caller-owned operator (diagonal and E/N/T couplings) and vector, all in
// caller-owned device memory.  It exists for callers that cannot allocate
// device memory in the middle of their time step: GPU-resident hosts that
// hand out every byte of device memory from their own preallocated arena,
// and programs that run near a fixed memory budget on a shared GPU, where a
// late cudaMalloc can fail or, because it synchronises the device, stall an
// otherwise asynchronous pipeline.  The only scratch it needs -- one partial
// sum per thread block of the dot product -- lives in a file-scope device
// array of SCF_NOALLOC_PARTIALS doubles that the module reserves once per
// device when the library is loaded on it.
#include <mutex>
#include "scf_kernels.h"
#include "../../include/scf_projection.h"

namespace {

// Block partials of x.Ax and the final sum.  Every call overwrites the slots
// it reads, so nothing has to be cleared between calls; calls that overlap on
// the GPU (for example on two streams) share this array and race.
static __device__ __align__(256) double g_noalloc_scratch[SCF_NOALLOC_PARTIALS + 1];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
double *g_scratch_ptr[kMaxDevices] = {nullptr};

__global__ void __launch_bounds__(256) k_apply_noalloc(LevelView<double> A, const double *__restrict__ x,
                                                       double *__restrict__ y, double *__restrict__ part)
{
    const long long n = (long long)A.n0 * A.n1 * A.n2;
    double v = 0.0;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
         t += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(t % A.n0) + 1;
        const int j = (int)((t / A.n0) % A.n1) + 1;
        const int k = (int)(t / ((long long)A.n0 * A.n1)) + 1;
        const int c = i + A.sy * j + A.sz * k;
        const double r = apply_row(A, x, c);
        y[c] = r;
        v += x[c] * r;
    }
    v = block_sum(v);
    if (threadIdx.x == 0) part[blockIdx.x] = v;
}

__global__ void __launch_bounds__(1024) k_apply_noalloc_sum(const double *__restrict__ part, int nblocks,
                                                            double *__restrict__ out_scratch,
                                                            double *__restrict__ out_user)
{
    double s = 0.0;
    for (int t = threadIdx.x; t < nblocks; t += blockDim.x) s += part[t];
    s = block_sum(s);
    if (threadIdx.x == 0) {
        *out_scratch = s;
        if (out_user) *out_user = s;
    }
}

// Device address of the scratch array for the current device, looked up once
// per device (the host-side symbol is not a device address).
int scratch_for_current_device(double **out)
{
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return SCF_ERR_CUDA;
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_ptr[dev]) {
        double *p = nullptr;
        if (cudaGetSymbolAddress((void **)&p, g_noalloc_scratch) != cudaSuccess || !p) return SCF_ERR_CUDA;
        g_scratch_ptr[dev] = p;
    }
    *out = g_scratch_ptr[dev];
    return SCF_OK;
}

}  // namespace

extern "C" int scf_apply_operator_noalloc(int32_t imax, int32_t jmax, int32_t kmax, const double *diag,
                                          const double *cpl_e, const double *cpl_n, const double *cpl_t,
                                          const double *x, double *y, double *x_dot_ax, void *stream)
{
    if (imax < 1 || jmax < 1 || kmax < 1) return SCF_ERR_BAD_ARG;
    // each factor is at most 2^31 + 1, so the first product fits in 64 bits;
    // the second is formed only once the first is known to be in range
    const long long g0 = (long long)imax + 2, g1 = (long long)jmax + 2, g2 = (long long)kmax + 2;
    if (g0 > SCF_NOALLOC_MAX_CELLS || g1 > SCF_NOALLOC_MAX_CELLS || g2 > SCF_NOALLOC_MAX_CELLS) return SCF_ERR_BAD_ARG;
    const long long g01 = g0 * g1;
    if (g01 > SCF_NOALLOC_MAX_CELLS || g01 * g2 > SCF_NOALLOC_MAX_CELLS) return SCF_ERR_BAD_ARG;
    if (!diag || !cpl_e || !cpl_n || !cpl_t || !x || !y) return SCF_ERR_BAD_ARG;
    double *scratch = nullptr;
    int rc = scratch_for_current_device(&scratch);
    if (rc) return rc;
    LevelView<double> A;
    A.n0 = imax; A.n1 = jmax; A.n2 = kmax;
    A.sy = imax + 2; A.sz = (imax + 2) * (jmax + 2);
    A.diag = diag; A.dinv = nullptr; A.cE = cpl_e; A.cN = cpl_n; A.cT = cpl_t;
    const long long n = (long long)imax * jmax * kmax;
    long long want = (n + 255) / 256;
    const int blocks = (int)(want < SCF_NOALLOC_PARTIALS ? want : SCF_NOALLOC_PARTIALS);
    cudaStream_t st = (cudaStream_t)stream;
    k_apply_noalloc<<<blocks, 256, 0, st>>>(A, x, y, scratch);
    k_apply_noalloc_sum<<<1, 1024, 0, st>>>(scratch, blocks, scratch + SCF_NOALLOC_PARTIALS, x_dot_ax);
    return cudaGetLastError() == cudaSuccess ? SCF_OK : SCF_ERR_CUDA;
}
