// pf_device.cuh -- device helpers shared by the kernel translation units:
// deterministic reductions and the element routines of the 20-node brick.
#pragma once
#include "pf_internal.h"

#include <cmath>

namespace pf {

#define FULLMASK 0xffffffffu

// ---------------------------------------------------------------------------
// reductions
static __device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULLMASK, v, o);
    return v;
}
static __device__ __forceinline__ double warp_max(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(FULLMASK, v, o));
    return v;
}

// Reduces NV values over the block (kinds bit k set = max, else sum).  The
// result is valid in every thread on return.  blockDim.x <= 1024.
template <int NV>
static __device__ __forceinline__ void block_reduce(double (&v)[NV], unsigned kinds)
{
    __shared__ double sh[NV][32];
    __shared__ double res[NV];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
    for (int k = 0; k < NV; ++k) v[k] = ((kinds >> k) & 1) ? warp_max(v[k]) : warp_sum(v[k]);
    if (lane == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k) sh[k][wid] = v[k];
    }
    __syncthreads();
    if (wid == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            double t = (lane < nw) ? sh[k][lane] : 0.0;
            t = ((kinds >> k) & 1) ? warp_max(t) : warp_sum(t);
            if (lane == 0) res[k] = t;
        }
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < NV; ++k) v[k] = res[k];
    __syncthreads();
}

// Block-uniform read of the stop flag: thread 0 reads it once for the whole
// block, so a block never splits at a barrier when another block of the same
// kernel sets the flag meanwhile.
static __device__ __forceinline__ bool block_stopped(const PcgState *st)
{
    __shared__ int s_stop;
    if (threadIdx.x == 0) s_stop = st ? st->stop : 0;
    __syncthreads();
    const bool v = s_stop != 0;
    __syncthreads();
    return v;
}

// Grid-wide barrier of a cooperative launch (every block resident at once).
// The arrival counter only grows: a block adds one and waits until it
// reaches the next multiple of the block count, which holds while every
// launch that uses the counter has the same block count and completes its
// barriers (the host zeroes it before a run).  Thread 0 releases the
// block's writes before arriving and acquires the others' after the wait.
// The wait is bounded: a block that gives up writes code 3 to *err, sets
// the PCG stop flag (so later launches of the run return at once) and
// returns false; its caller returns, and the blocks still waiting give up
// in turn.  (A two-level form, 16 group counters on separate lines feeding
// a top counter, measured no faster on 600-block grids.)
constexpr long long kGridSpinLimit = 1LL << 22;

static __device__ __forceinline__ bool grid_barrier(unsigned long long *bar, int *err, PcgState *st)
{
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        const unsigned long long nb = gridDim.x;
        const unsigned long long target = (atomicAdd(bar, 1ULL) / nb + 1) * nb;
        int ok = 0;
        for (long long i = 0; i < kGridSpinLimit; ++i) {
            unsigned long long v;
            asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(bar) : "memory");
            if (v >= target) {
                ok = 1;
                break;
            }
            __nanosleep(32);
        }
        if (!ok) {
            atomicExch(err, 3);
            atomicExch(&st->stop, 1);
        }
        __threadfence();
        s_ok = ok;
    }
    __syncthreads();
    const bool ok = s_ok != 0;
    __syncthreads();
    return ok;
}

// Sums (or maxes) G block partials in a fixed order; same value in every block.
static __device__ __forceinline__ double reduce_partials(const double *part, int G, bool is_max)
{
    double acc = 0.0;
    for (int i = threadIdx.x; i < G; i += blockDim.x) acc = is_max ? fmax(acc, part[i]) : acc + part[i];
    double v[1] = {acc};
    block_reduce<1>(v, is_max ? 1u : 0u);
    return v[0];
}

// SHAPE_DER for one node l of the 20-node brick (new_library.f90:865-896).
static __constant__ int c_xii[20] = {-1, -1, -1, 0, 1, 1, 1, 0, -1, -1, 1, 1, -1, -1, -1, 0, 1, 1, 1, 0};
static __constant__ int c_etai[20] = {-1, -1, -1, -1, -1, -1, -1, -1, 0, 0, 0, 0, 1, 1, 1, 1, 1, 1, 1, 1};
static __constant__ int c_zetai[20] = {-1, 0, 1, 1, 1, 0, -1, -1, -1, 1, 1, -1, -1, 0, 1, 1, 1, 0, -1, -1};

static __device__ __forceinline__ void shape_der20(int l, double xi, double eta, double zeta, double *d)
{
    const double xii = c_xii[l], etai = c_etai[l], zetai = c_zetai[l];
    const double xi0 = xi * xii, eta0 = eta * etai, zeta0 = zeta * zetai;
    const int n = l + 1;
    if (n == 4 || n == 8 || n == 16 || n == 20) {
        d[0] = -.5 * xi * (1. + eta0) * (1. + zeta0);
        d[1] = (.25 * etai) * (1. - xi * xi) * (1. + zeta0);
        d[2] = (.25 * zetai) * (1. - xi * xi) * (1. + eta0);
    } else if (n >= 9 && n <= 12) {
        d[0] = (.25 * xii) * (1. - eta * eta) * (1. + zeta0);
        d[1] = -.5 * eta * (1. + xi0) * (1. + zeta0);
        d[2] = (.25 * zetai) * (1. + xi0) * (1. - eta * eta);
    } else if (n == 2 || n == 6 || n == 14 || n == 18) {
        d[0] = (.25 * xii) * (1. + eta0) * (1. - zeta * zeta);
        d[1] = (.25 * etai) * (1. + xi0) * (1. - zeta * zeta);
        d[2] = -.5 * zeta * (1. + xi0) * (1. + eta0);
    } else {
        d[0] = (.125 * xii) * (1. + eta0) * (1. + zeta0) * (2. * xi0 + eta0 + zeta0 - 1.);
        d[1] = (.125 * etai) * (1. + xi0) * (1. + zeta0) * (xi0 + 2. * eta0 + zeta0 - 1.);
        d[2] = (.125 * zetai) * (1. + xi0) * (1. + eta0) * (xi0 + eta0 + 2. * zeta0 - 1.);
    }
}

// SHAPE_DER for one node l of the 8-node brick (new_library.f90:769-793):
// node signs (xi, eta, zeta) in Smith-Griffiths order, l = 0..7.
static __device__ __forceinline__ void shape_der8(int l, double xi, double eta, double zeta, double *d)
{
    const double sx = (l == 2 || l == 3 || l == 6 || l == 7) ? 1.0 : -1.0;
    const double se = l >= 4 ? 1.0 : -1.0;
    const double sz = (l == 1 || l == 2 || l == 5 || l == 6) ? 1.0 : -1.0;
    const double a = 1.0 + xi * sx, b = 1.0 + eta * se, c = 1.0 + zeta * sz;
    d[0] = 0.125 * sx * b * c;
    d[1] = 0.125 * se * a * c;
    d[2] = 0.125 * sz * a * b;
}

// DEEMAT nst=6 (new_library.f90:1671-1689): the three distinct entries.
static __device__ __forceinline__ void deemat3(double e, double v, double &d11, double &d12, double &d44)
{
    const double v2 = v / (1.0 - v);
    const double vv = (1.0 - 2.0 * v) / (1.0 - v) * 0.5;
    const double den = 2.0 * (1.0 + v) * vv;
    d11 = 1.0 * e / den;
    d12 = v2 * e / den;
    d44 = vv * e / den;
}

// DETERMINANT + INVERT of a 3x3 held column-major (maths.f90:490-633).
static __device__ __forceinline__ double det_invert3(double *m)
{
#define M(a, b) m[((a) - 1) + 3 * ((b) - 1)]
    double det = M(1, 1) * (M(2, 2) * M(3, 3) - M(3, 2) * M(2, 3));
    det = det - M(1, 2) * (M(2, 1) * M(3, 3) - M(3, 1) * M(2, 3));
    det = det + M(1, 3) * (M(2, 1) * M(3, 2) - M(3, 1) * M(2, 2));
    const double j11 = M(2, 2) * M(3, 3) - M(3, 2) * M(2, 3);
    const double j21 = -M(2, 1) * M(3, 3) + M(3, 1) * M(2, 3);
    const double j31 = M(2, 1) * M(3, 2) - M(3, 1) * M(2, 2);
    const double j12 = -M(1, 2) * M(3, 3) + M(3, 2) * M(1, 3);
    const double j22 = M(1, 1) * M(3, 3) - M(3, 1) * M(1, 3);
    const double j32 = -M(1, 1) * M(3, 2) + M(3, 1) * M(1, 2);
    const double j13 = M(1, 2) * M(2, 3) - M(2, 2) * M(1, 3);
    const double j23 = -M(1, 1) * M(2, 3) + M(2, 1) * M(1, 3);
    const double j33 = M(1, 1) * M(2, 2) - M(2, 1) * M(1, 2);
    M(1, 1) = j11 / det; M(1, 2) = j12 / det; M(1, 3) = j13 / det;
    M(2, 1) = j21 / det; M(2, 2) = j22 / det; M(2, 3) = j23 / det;
    M(3, 1) = j31 / det; M(3, 2) = j32 / det; M(3, 3) = j33 / det;
#undef M
    return det;
}


}  // namespace pf
