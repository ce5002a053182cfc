// pf_noalloc.cu -- element-by-element product u = K p that allocates nothing.
//
// For callers that cannot allocate device memory once they are running:
// codes whose device memory is reserved up front by a pool or a host
// framework (and that forbid cudaMalloc in the solve phase), callers that hold
// a lock under which cudaMalloc/cudaFree would synchronise the device, and
// embedded drivers that run with a fixed memory budget.  They pass their own
// device buffers (storkm, g_g, p, u); the only other memory the product needs
// -- the element results and the inverse of g_g used for the deterministic
// scatter -- lives in the file-scope array below.
//
// The array holds PF_NOALLOC_MAX_NELS elements and PF_NOALLOC_MAX_NEQ
// equations (about 14.3 MiB).  Every GPU that loads libpfgpu.so keeps it
// until the process exits; with CUDA's lazy module loading the device memory
// is taken when the first call on a device looks the array up, so a caller
// makes that first call (a set-up-only call with *nels = 0 does just that)
// before it reserves the rest of device memory.  All calls share the array:
// calls that overlap on the GPU (from two host threads, or on two streams)
// race on it and must not be made.  A call runs on the legacy default stream
// and waits for the whole device before it returns.
#include "pfgpu.h"

#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>

namespace pf {
void set_error(const char *fmt, ...);
int host_exception(const char *name);   // pf_abi.cu: an exception -> PF_FAILURE
}
using pf::set_error;

#define PF_NOALLOC_MAX_NELS 16384
#define PF_NOALLOC_MAX_NEQ 262144

namespace {

struct NoallocScratch {
    double utemp[PF_NOALLOC_MAX_NELS * 60];     // element results utemp(60, nels)
    int list[PF_NOALLOC_MAX_NELS * 60];         // (e*60+i) grouped by equation
    int cnt[PF_NOALLOC_MAX_NEQ + 1];            // contributions per equation
    int ptr[PF_NOALLOC_MAX_NEQ + 1];            // exclusive prefix of cnt
    int fill[PF_NOALLOC_MAX_NEQ + 1];           // fill cursor per equation
    int err;                                    // 1: a g_g entry outside 0..neq
};

static __device__ __align__(256) NoallocScratch g_noalloc_scratch;

constexpr unsigned FULL = 0xffffffffu;

// Clears everything a call relies on starting at zero.
__global__ void k_na_clear(int neq, NoallocScratch *S)
{
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q <= neq; q += gridDim.x * blockDim.x) {
        S->cnt[q] = 0;
        S->fill[q] = 0;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) S->err = 0;
}

// One warp per element: gather p through g_g (p(0) = 0, GATHER of
// gather_scatter.f90:547-692), the 60x60 product with the same FMA order as
// the library's k_elem, and a count of each equation's contributions.
__global__ void __launch_bounds__(256)
k_na_elem(int nels, int neq, const double *__restrict__ km, const int *__restrict__ g_g,
          const double *__restrict__ p, NoallocScratch *S)
{
    const int lane = threadIdx.x & 31;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    const int j1 = lane + 32;
    for (int e = warp; e < nels; e += nwarps) {
        int q0 = g_g[(size_t)e * 60 + lane];
        int q1 = j1 < 60 ? g_g[(size_t)e * 60 + j1] : 0;
        if (q0 < 0 || q0 > neq) { S->err = 1; q0 = 0; }
        if (q1 < 0 || q1 > neq) { S->err = 1; q1 = 0; }
        const double p0 = q0 > 0 ? p[q0 - 1] : 0.0;
        const double p1 = q1 > 0 ? p[q1 - 1] : 0.0;
        if (q0 > 0) atomicAdd(&S->cnt[q0 - 1], 1);
        if (q1 > 0) atomicAdd(&S->cnt[q1 - 1], 1);
        const double *ke = km + (size_t)e * 3600 + 2 * lane;
        double a0 = 0.0, a1 = 0.0;
#pragma unroll 12
        for (int j = 0; j < 60; ++j) {
            const double pj = __shfl_sync(FULL, j < 32 ? p0 : p1, j & 31);
            if (lane < 30) {
                const double2 k2 = __ldg(reinterpret_cast<const double2 *>(ke + 60 * j));
                a0 = fma(k2.x, pj, a0);
                a1 = fma(k2.y, pj, a1);
            }
        }
        if (lane < 30) {
            S->utemp[(size_t)e * 60 + 2 * lane] = a0;
            S->utemp[(size_t)e * 60 + 2 * lane + 1] = a1;
        }
    }
}

// Exclusive prefix sum of cnt[0..neq) into ptr[0..neq] (one block).
__global__ void __launch_bounds__(1024) k_na_scan(int neq, NoallocScratch *S)
{
    __shared__ int part[1024];
    const int t = threadIdx.x, nt = blockDim.x;
    const int chunk = (neq + nt - 1) / nt;
    const int b = t * chunk, e = min(neq, b + chunk);
    int s = 0;
    for (int q = b; q < e; ++q) s += S->cnt[q];
    part[t] = s;
    __syncthreads();
    for (int off = 1; off < nt; off <<= 1) {   // inclusive Hillis-Steele scan
        const int v = t >= off ? part[t - off] : 0;
        __syncthreads();
        part[t] += v;
        __syncthreads();
    }
    int run = t > 0 ? part[t - 1] : 0;
    for (int q = b; q < e; ++q) {
        S->ptr[q] = run;
        run += S->cnt[q];
    }
    if (t == nt - 1) S->ptr[neq] = part[nt - 1];
}

// Places every contribution in its equation's bucket (bucket order is fixed
// later by the sort in k_na_gather).
__global__ void k_na_fill(int nels, int neq, const int *__restrict__ g_g, NoallocScratch *S)
{
    const size_t n = (size_t)nels * 60;
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x) {
        const int q = g_g[k];
        if (q < 1 || q > neq) continue;
        const int pos = S->ptr[q - 1] + atomicAdd(&S->fill[q - 1], 1);
        S->list[pos] = (int)k;
    }
}

// Per equation: sort the bucket by (element, local dof) and sum in that
// order -- the order of the serial SCATTER (gather_scatter.f90:694-854).
// Writes nothing when k_na_elem found a g_g entry out of range, so the
// caller's u survives a failed call.
__global__ void k_na_gather(int neq, NoallocScratch *S, double *__restrict__ u)
{
    if (S->err) return;   // written by k_na_elem, earlier on the same stream
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < neq; q += gridDim.x * blockDim.x) {
        const int b = S->ptr[q], e = S->ptr[q + 1];
        int *L = S->list;
        for (int i = b + 1; i < e; ++i) {   // insertion sort: buckets are short
            const int v = L[i];
            int j = i - 1;
            while (j >= b && L[j] > v) {
                L[j + 1] = L[j];
                --j;
            }
            L[j + 1] = v;
        }
        double acc = 0.0;
        for (int i = b; i < e; ++i) acc += S->utemp[L[i]];
        u[q] = acc;
    }
}

// Device address of the scratch array, looked up once per device.
constexpr int kMaxDevices = 64;
std::mutex g_mu;
NoallocScratch *g_addr[kMaxDevices] = {nullptr};

int scratch_for_current_device(NoallocScratch **out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        set_error("pf_ebe_matvec_noalloc: no usable current device (%s)", cudaGetErrorString(e));
        return 1;
    }
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_addr[dev]) {
        void *ptr = nullptr;
        e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (e != cudaSuccess || !ptr) {
            set_error("pf_ebe_matvec_noalloc: cudaGetSymbolAddress failed on device %d: %s", dev,
                      cudaGetErrorString(e));
            return 1;
        }
        g_addr[dev] = (NoallocScratch *)ptr;
    }
    *out = g_addr[dev];
    return 0;
}

// Device memory of device dev (the scratch belongs to the current device),
// or managed memory.
bool is_device_pointer(const void *p, int dev)
{
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return (a.type == cudaMemoryTypeDevice && a.device == dev) || a.type == cudaMemoryTypeManaged;
}

}  // namespace

// u(neq) = K p over the elements of g_g, all buffers on the current device.
// The first call on each device looks up the scratch array's address (and so
// loads it); make that first call during set-up and before capturing any
// stream.  *nels = *neq = 0 does only that set-up.
extern "C" int pf_ebe_matvec_noalloc(const int *nels_p, const int *neq_p, const double *d_storkm,
                                     const int *d_g_g, const double *d_p, double *d_u)
try {
    if (nels_p && neq_p && *nels_p == 0 && *neq_p == 0) {   // set-up only
        NoallocScratch *S = nullptr;
        return scratch_for_current_device(&S) ? PF_FAILURE : PF_SUCCESS;
    }
    if (!nels_p || !neq_p || !d_storkm || !d_g_g || !d_p || !d_u) {
        set_error("pf_ebe_matvec_noalloc: null argument");
        return PF_FAILURE;
    }
    const int nels = *nels_p, neq = *neq_p;
    if (nels < 1 || nels > PF_NOALLOC_MAX_NELS || neq < 1 || neq > PF_NOALLOC_MAX_NEQ) {
        set_error("pf_ebe_matvec_noalloc: nels=%d neq=%d outside the fixed scratch limits "
                  "(1..%d elements, 1..%d equations); use pf_ebe_matvec",
                  nels, neq, PF_NOALLOC_MAX_NELS, PF_NOALLOC_MAX_NEQ);
        return PF_FAILURE;
    }
    int cur = 0;
    if (cudaGetDevice(&cur) != cudaSuccess) {
        set_error("pf_ebe_matvec_noalloc: no current device");
        return PF_FAILURE;
    }
    if (!is_device_pointer(d_storkm, cur) || !is_device_pointer(d_g_g, cur) || !is_device_pointer(d_p, cur) ||
        !is_device_pointer(d_u, cur)) {
        set_error("pf_ebe_matvec_noalloc: storkm, g_g, p and u must be memory of the current device %d", cur);
        return PF_FAILURE;
    }
    NoallocScratch *S = nullptr;
    if (scratch_for_current_device(&S)) return PF_FAILURE;
    int nsm = 0, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    if (nsm < 1) nsm = 1;
    const int gq = (neq + 256) / 256 < nsm * 8 ? (neq + 256) / 256 : nsm * 8;
    const int ge = (nels + 7) / 8 < nsm * 8 ? (nels + 7) / 8 : nsm * 8;
    k_na_clear<<<gq, 256>>>(neq, S);
    k_na_elem<<<ge, 256>>>(nels, neq, d_storkm, d_g_g, d_p, S);
    k_na_scan<<<1, 1024>>>(neq, S);
    k_na_fill<<<ge, 256>>>(nels, neq, d_g_g, S);
    k_na_gather<<<gq, 256>>>(neq, S, d_u);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e != cudaSuccess) {
        set_error("pf_ebe_matvec_noalloc: %s", cudaGetErrorString(e));
        return PF_FAILURE;
    }
    int err = 0;
    e = cudaMemcpy(&err, &S->err, sizeof(int), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) {
        set_error("pf_ebe_matvec_noalloc: %s", cudaGetErrorString(e));
        return PF_FAILURE;
    }
    if (err) {
        set_error("pf_ebe_matvec_noalloc: g_g holds an equation number outside 0..%d (u left unchanged)", neq);
        return PF_FAILURE;
    }
    return PF_SUCCESS;
} catch (...) {
    return pf::host_exception("pf_ebe_matvec_noalloc");
}
